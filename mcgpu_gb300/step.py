"""Host-side mirror of MCGPU's SimulationStep contract over the GB300 C ABI.

``GpuSimulationStep`` keeps the names, argument meaning and call order of the
reference's strategy object (src/Metropolis/SimulationStep.h:24-94,
src/Metropolis/BruteForceStep.h): ``choose_molecule``,
``calc_molecular_energy_contribution(curr, start)``,
``calc_molecule_energy``, ``change_molecule``, ``rollback`` and
``calc_system_energy``.  The random draws come from the C library's
``rand()`` in the reference's order (MathLibrary.cpp:27-33), so a run driven
by ``run_plain`` proposes exactly the moves ``metrosim -s`` proposes.

Every energy is computed by the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref
from dataclasses import dataclass

import numpy as np

from . import _abi
from .workloads import BoxData

RAND_MAX = 2147483647
KBOLTZ = 0.00198717  # SimBox.h:16


class Context:
    """One CUDA device context (mcgpu_ctx_create).  Boxes, batches and
    servers made from it register here; closing the context closes them
    first (the C ABI requires them destroyed before their context)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        self._children = weakref.WeakSet()
        L = _abi.lib()
        _abi.check(L.mcgpu_ctx_create(C.byref(self._h), int(device)))
        self.device = device

    def adopt(self, child) -> None:
        self._children.add(child)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def set_stream(self, stream_ptr: int | None) -> None:
        """Launch on the caller's CUDA stream (an integer cudaStream_t, e.g.
        torch.cuda.Stream().cuda_stream); None restores the context's own."""
        _abi.check(_abi.lib().mcgpu_ctx_set_stream(self._h, C.c_void_p(stream_ptr or 0)),
                   self._h)

    def close(self) -> None:
        if self._h:
            for child in list(self._children):
                child.close()
            _abi.lib().mcgpu_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LibcRand:
    """The reference's RNG: srand/rand of the C library (MathLibrary.cpp:27-33)."""

    def __init__(self, seed: int):
        self._libc = C.CDLL(None)
        self._libc.rand.restype = C.c_int
        self._libc.srand.argtypes = [C.c_uint]
        self._libc.srand(int(seed) & 0xFFFFFFFF)

    def rand(self) -> int:
        return int(self._libc.rand())

    def random_real(self, start: float, end: float) -> float:
        """randomReal (MathLibrary.cpp:31-33)."""
        return (end - start) * (float(self.rand()) / RAND_MAX) + start


class GpuBox:
    """A box resident on the GPU (mcgpu_box_upload), FP64 or mixed pairs."""

    def __init__(self, ctx: Context, box: BoxData, precision: int = _abi.PREC_FP64):
        self.ctx = ctx
        self.data = box.copy().normalise()
        self._desc = self.data.desc()
        self._h = C.c_void_p()
        _abi.check(_abi.lib().mcgpu_box_upload(ctx.handle, C.byref(self._desc), int(precision),
                                               C.byref(self._h)), ctx.handle)
        self.precision = precision
        self.topology = None
        self.intra = False
        ctx.adopt(self)

    def _check(self, st: int) -> None:
        _abi.check(st, self.ctx.handle)

    def close(self) -> None:
        if self._h:
            _abi.lib().mcgpu_box_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_mol(self) -> int:
        return self.data.n_mol

    def mol_energy(self, curr: int, start: int) -> float:
        out = C.c_double()
        self._check(_abi.lib().mcgpu_mol_energy(self._h, int(curr), int(start), C.byref(out)))
        return out.value

    def change_molecule(self, mol: int, vertex: int, dx: float, dy: float, dz: float,
                        rx: float, ry: float, rz: float) -> None:
        mv = _abi.Move(int(vertex), 0, dx, dy, dz, rx, ry, rz)
        self._check(_abi.lib().mcgpu_change_molecule(self._h, int(mol), C.byref(mv)))

    def move_energies(self, mol: int, vertex: int, dx: float, dy: float, dz: float,
                      rx: float, ry: float, rz: float) -> tuple[float, float]:
        mv = _abi.Move(int(vertex), 0, dx, dy, dz, rx, ry, rz)
        eo, en = C.c_double(), C.c_double()
        self._check(_abi.lib().mcgpu_move_energies(self._h, int(mol), C.byref(mv), C.byref(eo),
                                                   C.byref(en)))
        return eo.value, en.value

    def rollback(self, mol: int) -> None:
        self._check(_abi.lib().mcgpu_rollback(self._h, int(mol)))

    def system_energy(self) -> float:
        out = C.c_double()
        self._check(_abi.lib().mcgpu_system_energy(self._h, C.byref(out)))
        return out.value

    def download(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = self.data.n_atom
        x, y, z = np.empty(n), np.empty(n), np.empty(n)
        dp = C.POINTER(C.c_double)
        self._check(_abi.lib().mcgpu_box_download(self._h, x.ctypes.data_as(dp),
                                                  y.ctypes.data_as(dp), z.ctypes.data_as(dp),
                                                  None))
        return x, y, z

    def set_verlet(self, skin: float) -> None:
        """Verlet neighbour lists (skin in Angstrom, <= 0 off) for chain_run."""
        self._check(_abi.lib().mcgpu_box_set_verlet(self._h, float(skin)))

    def set_window(self, k: int) -> None:
        """Windows of k steps (1, 2, 4, 8) for chain_run: a cluster of k CTAs
        evaluates each window's moves at once and takes the decisions in step
        order (mcgpu_chain_set_window); results equal k = 1."""
        self._check(_abi.lib().mcgpu_chain_set_window(self._h, int(k)))

    def run_plain_native(self, seed: int, n_steps: int, fused: bool = False) -> "_abi.PlainStats":
        """Simulation::run's NVT loop in the library's C++ (mcgpu_run_plain):
        the same calls and the same rand() draws as run_plain over
        GpuSimulationStep(self, LibcRand(seed))."""
        st = _abi.PlainStats()
        self._check(_abi.lib().mcgpu_run_plain(self._h, int(seed) & 0xFFFFFFFF, int(n_steps),
                                               1 if fused else 0, C.byref(st)))
        return st

    def run_plain_device(self, seed: int, n_steps: int) -> "_abi.PlainStats":
        """The same loop as run_plain_native entirely on the device
        (mcgpu_run_plain_device): one CTA, the C library's generator
        restated on the device and seeded as srand(seed) seeds it."""
        st = _abi.PlainStats()
        self._check(_abi.lib().mcgpu_run_plain_device(self._h, int(seed) & 0xFFFFFFFF,
                                                      int(n_steps), C.byref(st)))
        return st

    # ---- flexible molecules (the reference's code behind ENABLE_INTRA) ----

    def set_topology(self, topo) -> None:
        """Bond / angle / exclusion rows (workloads.Topology) for this box
        (mcgpu_box_set_topology); intramolecular moves stay off."""
        t = topo.copy().normalise()
        self._topo = t
        d = t.desc()
        self._check(_abi.lib().mcgpu_box_set_topology(self._h, C.byref(d)))
        self.topology = t

    def set_intra(self, on: bool = True) -> None:
        """ENABLE_INTRA for this box (mcgpu_box_set_intra): molecule and
        system energies carry the intramolecular term, change_molecule makes
        the intramolecular move with its rand() draws, rollback restores the
        bond lengths and angle sizes."""
        self._check(_abi.lib().mcgpu_box_set_intra(self._h, 1 if on else 0))
        self.intra = bool(on)

    def intra_energy(self, mol: int) -> float:
        out = C.c_double()
        self._check(_abi.lib().mcgpu_intra_energy(self._h, int(mol), C.byref(out)))
        return out.value

    def stretch_bond(self, mol: int, bond: int, dist: float) -> None:
        self._check(_abi.lib().mcgpu_stretch_bond(self._h, int(mol), int(bond), float(dist)))

    def expand_angle(self, mol: int, angle: int, deg: float) -> None:
        self._check(_abi.lib().mcgpu_expand_angle(self._h, int(mol), int(angle), float(deg)))

    def save_intra(self, mol: int) -> None:
        self._check(_abi.lib().mcgpu_save_intra(self._h, int(mol)))

    def intramolecular_move(self, mol: int) -> None:
        self._check(_abi.lib().mcgpu_intramolecular_move(self._h, int(mol)))

    def set_step(self, step: int) -> None:
        self._check(_abi.lib().mcgpu_intra_set_step(self._h, int(step)))

    def intra_state(self) -> dict:
        t = self.topology
        bl, asz = np.empty(max(t.n_bond, 1)), np.empty(max(t.n_angle, 1))
        st = _abi.IntraState()
        dp = C.POINTER(C.c_double)
        self._check(_abi.lib().mcgpu_intra_get(self._h, bl.ctypes.data_as(dp),
                                               asz.ctypes.data_as(dp), C.byref(st)))
        return dict(bond_len=bl[:t.n_bond], angle_size=asz[:t.n_angle],
                    max_bond_delta=st.max_bond_delta, max_angle_delta=st.max_angle_delta,
                    step_num=st.step_num, bond_moves=st.bond_moves,
                    bond_accepted=st.bond_accepted, angle_moves=st.angle_moves,
                    angle_accepted=st.angle_accepted)

    def chain_run(self, seed: int, n_steps: int, chain_id: int = 0,
                  rotation: int = _abi.ROT_AXIS, trace: bool = False):
        st = _abi.ChainStats()
        tr = (_abi.Trace * max(n_steps, 1))() if trace else None
        self._check(_abi.lib().mcgpu_chain_run(self._h, int(seed) & (2 ** 64 - 1), int(chain_id),
                                               int(n_steps), int(rotation), C.byref(st),
                                               tr if trace else None))
        return st, (list(tr)[:n_steps] if trace else None)


class GpuSimulationStep:
    """The SimulationStep contract (SimulationStep.h:24-94) on the GPU."""

    def __init__(self, gbox: GpuBox, rng: LibcRand):
        self.box = gbox
        self.rng = rng
        self.max_translate = gbox.data.max_translate
        self.max_rotate = gbox.data.max_rotate
        self.kT = gbox.data.temperature * KBOLTZ  # SimBoxBuilder.cpp:29

    # SimulationStep::chooseMolecule (SimulationStep.cpp:25-27).  The cast
    # can give n_mol when rand() == RAND_MAX; that index is clamped to
    # n_mol - 1 (the reference would read past its rows).
    def choose_molecule(self) -> int:
        return min(int(self.rng.random_real(0, self.box.n_mol)), self.box.n_mol - 1)

    # BruteForceCalcs::calcMolecularEnergyContribution (BruteForceStep.cpp:15-46).
    def calc_molecular_energy_contribution(self, curr: int, start: int) -> float:
        return self.box.mol_energy(curr, start)

    # SimulationStep::calcMoleculeEnergy (SimulationStep.cpp:15-18): with
    # intramolecular moves on (GpuBox.set_intra) the library adds the
    # intramolecular energy to the molecule's.
    def calc_molecule_energy(self, curr: int, start: int) -> float:
        return self.calc_molecular_energy_contribution(curr, start)

    def draw_move(self, mol: int) -> tuple:
        """The seven draws of SimCalcs::intermolecularMove (SimulationStep.cpp:
        527-535), in order; the vertex is clamped like chooseMolecule."""
        n = int(self.box.data.mol_len[mol])
        vertex = min(int(self.rng.random_real(0, n)), n - 1)
        t, r = self.max_translate, self.max_rotate
        dx = self.rng.random_real(-t, t)
        dy = self.rng.random_real(-t, t)
        dz = self.rng.random_real(-t, t)
        rx = self.rng.random_real(-r, r)
        ry = self.rng.random_real(-r, r)
        rz = self.rng.random_real(-r, r)
        return vertex, dx, dy, dz, rx, ry, rz

    # SimulationStep::changeMolecule -> SimCalcs::intermolecularMove (and,
    # with intramolecular moves on, SimCalcs::intramolecularMove, whose draws
    # the library takes from the same C-library rand()).
    def change_molecule(self, mol: int) -> tuple:
        mv = self.draw_move(mol)
        self.box.change_molecule(mol, *mv)
        return mv

    # SimulationStep::rollback -> SimCalcs::rollback.
    def rollback(self, mol: int) -> None:
        self.box.rollback(mol)

    # SimulationStep::calcSystemEnergy with subLJ = subCharge = 0.
    def calc_system_energy(self) -> float:
        return self.box.system_energy()

    # SimCalcs::acceptMove (SimulationStep.cpp:794-803).
    def accept_move(self, delta_e: float) -> bool:
        if delta_e < 0:
            return True
        return math.exp(-delta_e / self.kT) >= self.rng.random_real(0.0, 1.0)


def run_plain_device_many(boxes: list, seeds, n_steps: int) -> list:
    """The device loop of several boxes (one context, one pair precision) in
    one launch, one CTA per box (mcgpu_boxes_run_plain_device); box i seeded
    with seeds[i].  Returns each box's PlainStats."""
    n = len(boxes)
    hs = (C.c_void_p * n)(*[b._h.value for b in boxes])
    sd = (C.c_uint * n)(*[int(s) & 0xFFFFFFFF for s in seeds])
    out = (_abi.PlainStats * n)()
    _abi.check(_abi.lib().mcgpu_boxes_run_plain_device(hs, n, sd, int(n_steps), out),
               boxes[0].ctx.handle)
    return list(out)


@dataclass
class PlainResult:
    energy: float
    accepted: int
    rejected: int
    initial_energy: float


def run_plain(step: GpuSimulationStep, n_steps: int, fused: bool = False) -> PlainResult:
    """Simulation::run's NVT loop (Simulation.cpp:219-264) driving the GPU
    step object: choose, old energy, change, new energy, accept or roll back.
    With fused=True the old energy, move and new energy go in one launch
    (mcgpu_move_energies); the draws and decisions are the same.  With
    intramolecular moves on the calls are made one by one (fused moves are
    rigid)."""
    e = step.calc_system_energy()
    e0 = e
    acc = rej = 0
    intra = getattr(step.box, "intra", False)
    step0 = step.box.intra_state()["step_num"] if intra else 0
    for s in range(n_steps):
        if intra:
            # the counter Simulation::run increments after every step
            # (Simulation.cpp:263), read by the intramolecular width tuning
            step.box.set_step(step0 + s)
        idx = step.choose_molecule()
        if fused and not intra:
            mv = step.draw_move(idx)
            old, new = step.box.move_energies(idx, *mv)
        else:
            old = step.calc_molecule_energy(idx, 0)
            step.change_molecule(idx)
            new = step.calc_molecule_energy(idx, 0)
        if step.accept_move(new - old):
            acc += 1
            e += new - old
        else:
            rej += 1
            step.rollback(idx)
    if intra:
        step.box.set_step(step0 + n_steps)
    return PlainResult(e, acc, rej, e0)
