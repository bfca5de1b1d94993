"""ctypes wrapper of the oracle (TEST INFRASTRUCTURE ONLY).

* ``OracleBox``   the C restatement (oracle/mcgpu_oracle.c, built into
                  oracle/_build/liboracle.so) over a BoxData's rows.
* ``RefHarness``  the reference's own compiled CPU path plus the white-box
                  harness (oracle/_ref/libmcgpu_ref.so); present only where
                  the reference sources were available to compile.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "liboracle.so"
REF_SO = HERE / "_ref" / "libmcgpu_ref.so"
REF_BIN = HERE / "_ref" / "metrosim"
REFERENCE_SRC = Path(os.environ.get("MCGPU_REFERENCE", "/root/reference"))

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class OrcBox(C.Structure):
    _fields_ = [
        ("n_mol", C.c_int), ("n_atom", C.c_int), ("n_pidx", C.c_int), ("largest_mol", C.c_int),
        ("x", _dp), ("y", _dp), ("z", _dp),
        ("sigma", _dp), ("epsilon", _dp), ("charge", _dp),
        ("mol_start", _ip), ("mol_len", _ip), ("mol_pidx_start", _ip), ("mol_pidx_count", _ip),
        ("pidx", _ip),
        ("rb_x", _dp), ("rb_y", _dp), ("rb_z", _dp),
        ("size", C.c_double * 3),
        ("cutoff", C.c_double), ("kT", C.c_double), ("max_translate", C.c_double),
        ("max_rotate", C.c_double),
    ]


class OrcMove(C.Structure):
    _fields_ = [("mol", C.c_int), ("vertex", C.c_int), ("mode", C.c_int), ("pad", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("r0", C.c_double), ("r1", C.c_double), ("r2", C.c_double), ("r3", C.c_double),
                ("u", C.c_double)]


class OrcChainS(C.Structure):
    _fields_ = [("b", C.POINTER(OrcBox)), ("A", C.POINTER(C.c_uint32)),
                ("q", C.POINTER(C.c_float)), ("tpl", C.POINTER(C.c_float)),
                ("off", C.POINTER(C.c_float)), ("rot_mode", C.c_int)]


class OrcMoveF(C.Structure):
    _fields_ = [("mol", C.c_int), ("vertex", C.c_int), ("dx", C.c_float), ("dy", C.c_float),
                ("dz", C.c_float), ("qw", C.c_float), ("qx", C.c_float), ("qy", C.c_float),
                ("qz", C.c_float), ("u", C.c_float)]


class OrcTrace(C.Structure):
    _fields_ = [("mol", C.c_int), ("accepted", C.c_int), ("e_old", C.c_double),
                ("e_new", C.c_double), ("de", C.c_double), ("u", C.c_double)]


class OrcTopo(C.Structure):
    _fields_ = [
        ("n_bond", C.c_int), ("n_angle", C.c_int), ("n_type", C.c_int),
        ("max_intra_moves", C.c_int),
        ("bond_a1", _ip), ("bond_a2", _ip), ("bond_var", _ip),
        ("bond_k", _dp), ("bond_eq", _dp), ("bond_len", _dp), ("bond_len_rb", _dp),
        ("angle_a1", _ip), ("angle_a2", _ip), ("angle_mid", _ip), ("angle_var", _ip),
        ("angle_k", _dp), ("angle_eq", _dp), ("angle_size", _dp), ("angle_size_rb", _dp),
        ("mol_bond_start", _ip), ("mol_bond_count", _ip), ("mol_angle_start", _ip),
        ("mol_angle_count", _ip), ("mol_type", _ip),
        ("type_natom", _ip), ("type_off", _ip), ("pair_code", C.POINTER(C.c_uint8)),
        ("uf", _ip),
        ("max_bond_delta", C.c_double), ("max_angle_delta", C.c_double),
        ("step_num", C.c_longlong),
        ("bond_moves", C.c_longlong), ("bond_accepted", C.c_longlong),
        ("angle_moves", C.c_longlong), ("angle_accepted", C.c_longlong),
        ("flex_bonds", C.c_int), ("flex_angles", C.c_int),
    ]


def build(reference: bool = True) -> None:
    """Compiles the restatement and, where the reference sources exist, the
    reference harness."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if reference and REFERENCE_SRC.is_dir():
        subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "ref", f"REF={REFERENCE_SRC}"],
                       check=True)


_orc = None


def orc_lib() -> C.CDLL:
    global _orc
    if _orc is None:
        if not ORACLE_SO.exists():
            build(reference=False)
        L = C.CDLL(str(ORACLE_SO))
        P = C.POINTER(OrcBox)
        protos = {
            "orc_mol_energy": (C.c_double, [P, C.c_int, C.c_int]),
            "orc_system_energy": (C.c_double, [P]),
            "orc_mol_energy_abs": (C.c_double, [P, C.c_int, C.c_int]),
            "orc_mol_energy_absk": (C.c_double, [P, C.c_int, C.c_int]),
            "orc_mol_pair_energy": (C.c_double, [P, C.c_int, C.c_int]),
            "orc_count_pairs": (C.c_int, [P, C.c_int, C.POINTER(C.c_longlong),
                                          C.POINTER(C.c_longlong)]),
            "orc_apply_move": (None, [P, C.POINTER(OrcMove)]),
            "orc_rollback": (None, [P, C.c_int]),
            "orc_keep_in_box": (None, [P, C.c_int]),
            "orc_wrap_all": (None, [P]),
            "orc_accept": (C.c_int, [C.c_double, C.c_double, C.c_double]),
            "orc_random_real": (C.c_double, [C.c_double, C.c_double, C.c_int]),
            "orc_make_periodic": (C.c_double, [C.c_double, C.c_double]),
            "orc_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                         C.POINTER(C.c_uint32)]),
            "orc_philox_move": (None, [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, _ip,
                                       C.c_double, C.c_double, C.c_int, C.POINTER(OrcMove)]),
            "orc_chain_run": (C.c_double, [P, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_int,
                                           C.c_double, C.POINTER(OrcTrace),
                                           C.POINTER(C.c_longlong)]),
            "orc_chains_run_mt": (C.c_double, [P, C.c_int, C.POINTER(C.c_uint64), C.c_uint64,
                                               C.c_int, C.c_int, C.c_int,
                                               C.POINTER(C.c_longlong)]),
            "orc_resize_box_centres": (None, [P, C.c_double]),
            "orc_fchain_init": (None, [C.POINTER(OrcChainS)]),
            "orc_fchain_draw": (None, [C.POINTER(OrcChainS), C.c_uint64, C.c_uint32, C.c_uint64,
                                       C.POINTER(OrcMoveF)]),
            "orc_fchain_run": (C.c_double, [C.POINTER(OrcChainS), C.c_uint64, C.c_uint32,
                                            C.c_uint64, C.c_int, C.c_double, C.POINTER(OrcTrace),
                                            C.POINTER(C.c_longlong)]),
            "orc_fchain_run_window": (C.c_double, [C.POINTER(OrcChainS), C.c_uint64, C.c_uint32,
                                                   C.c_uint64, C.c_int, C.c_int, C.c_double,
                                                   C.POINTER(OrcTrace), C.POINTER(C.c_longlong),
                                                   C.POINTER(C.c_longlong), C.c_int]),
            "orc_sincos_f32": (None, [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "orc_fchain_volume": (C.c_int, [C.POINTER(OrcChainS), C.c_uint64, C.c_uint32,
                                            C.c_uint64, C.c_double, C.c_double, C.c_float,
                                            C.c_double,
                                            C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]),
            "orc_accept_volume": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double,
                                            C.c_int, C.c_double, C.c_double]),
            "orc_build_centres": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_uint64,
                                            _dp]),
            "orc_bond_energy": (C.c_double, [C.POINTER(OrcTopo), C.c_int]),
            "orc_angle_energy": (C.c_double, [C.POINTER(OrcTopo), C.c_int]),
            "orc_intra_energy": (C.c_double, [P, C.POINTER(OrcTopo), C.c_int]),
            "orc_stretch_bond": (None, [P, C.POINTER(OrcTopo), C.c_int, C.c_int, C.c_double]),
            "orc_expand_angle": (None, [P, C.POINTER(OrcTopo), C.c_int, C.c_int, C.c_double]),
            "orc_save_intra": (None, [C.POINTER(OrcTopo), C.c_int]),
            "orc_rollback_intra": (None, [C.POINTER(OrcTopo), C.c_int]),
            "orc_intramolecular_move": (None, [P, C.POINTER(OrcTopo), C.c_int]),
            "orc_system_energy_intra": (C.c_double, [P, C.POINTER(OrcTopo)]),
            "orc_run_plain_intra": (C.c_double, [P, C.POINTER(OrcTopo), C.c_int, C.c_double,
                                                 C.POINTER(C.c_int)]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _orc = L
    return _orc


KBOLTZ = 0.00198717


class OracleBox:
    """An FP64 box the restatement mutates in place (numpy rows)."""

    def __init__(self, box):
        b = box.copy().normalise()
        self.data = b
        self.largest = int(b.mol_len.max())
        self.rb = [np.zeros(self.largest) for _ in range(3)]
        s = OrcBox()
        s.n_mol, s.n_atom, s.n_pidx, s.largest_mol = b.n_mol, b.n_atom, b.n_pidx, self.largest
        for k in ("x", "y", "z", "sigma", "epsilon", "charge"):
            setattr(s, k, getattr(b, k).ctypes.data_as(_dp))
        for k in ("mol_start", "mol_len", "mol_pidx_start", "mol_pidx_count", "pidx"):
            setattr(s, k, getattr(b, k).ctypes.data_as(_ip))
        s.rb_x, s.rb_y, s.rb_z = (r.ctypes.data_as(_dp) for r in self.rb)
        for i in range(3):
            s.size[i] = float(b.size[i])
        s.cutoff = b.cutoff
        s.kT = b.temperature * KBOLTZ
        s.max_translate = b.max_translate
        s.max_rotate = b.max_rotate
        self.s = s

    @property
    def ref(self):
        return C.byref(self.s)

    def mol_energy(self, curr: int, start: int = 0) -> float:
        return orc_lib().orc_mol_energy(self.ref, curr, start)

    def system_energy(self) -> float:
        return orc_lib().orc_system_energy(self.ref)

    def mol_energy_abs(self, curr: int, start: int = 0) -> float:
        """Scale of an FP32-pair result's rounding: the sum over the pair
        terms of |term| times its condition number with respect to distance
        (12 for 4 eps s^12, 6 for 4 eps s^6, 1 for Coulomb)."""
        return orc_lib().orc_mol_energy_absk(self.ref, curr, start)

    def count_pairs(self, curr: int) -> tuple[int, int]:
        a, b = C.c_longlong(), C.c_longlong()
        orc_lib().orc_count_pairs(self.ref, curr, C.byref(a), C.byref(b))
        return a.value, b.value

    def apply_move(self, mol, vertex, dx, dy, dz, r0, r1, r2, r3=0.0, mode=0) -> None:
        mv = OrcMove(int(mol), int(vertex), int(mode), 0, dx, dy, dz, r0, r1, r2, r3, 0.0)
        orc_lib().orc_apply_move(self.ref, C.byref(mv))

    def rollback(self, mol: int) -> None:
        orc_lib().orc_rollback(self.ref, int(mol))

    def coords(self) -> np.ndarray:
        return np.stack([self.data.x, self.data.y, self.data.z], axis=1).copy()

    def philox_move(self, seed: int, chain: int, step: int, mode: int) -> OrcMove:
        mv = OrcMove()
        b = self.data
        orc_lib().orc_philox_move(int(seed) & (2 ** 64 - 1), int(chain), int(step), b.n_mol,
                                  b.mol_len.ctypes.data_as(_ip), b.max_translate, b.max_rotate,
                                  int(mode), C.byref(mv))
        return mv

    def chain_run(self, seed: int, chain: int, n_steps: int, mode: int, e0: float = 0.0,
                  step0: int = 0):
        tr = (OrcTrace * max(1, n_steps))()
        acc = C.c_longlong()
        e = orc_lib().orc_chain_run(self.ref, int(seed) & (2 ** 64 - 1), int(chain), int(step0),
                                    int(n_steps), int(mode), float(e0), tr, C.byref(acc))
        return e, acc.value, list(tr)[:n_steps]


class OracleFlex:
    """A box of flexible molecules on the restatement: an OracleBox plus the
    bond / angle rows of a Topology (mcgpu_gb300.workloads), mutated in
    place, with the intramolecular functions as the reference runs them with
    ENABLE_INTRA true.  Random draws come from the C library's rand()
    (seed it with srand, e.g. through LibcRand)."""

    def __init__(self, box, topo):
        self.ob = OracleBox(box)
        t = topo.copy().normalise()
        self.t = t
        self.bond_len_rb = np.zeros(max(t.n_bond, 1))
        self.angle_size_rb = np.zeros(max(t.n_angle, 1))
        self.type_off = np.concatenate([[0], np.cumsum(t.type_natom.astype(np.int64) ** 2)[:-1]]
                                       ).astype(np.int32) if t.n_type else np.zeros(1, np.int32)
        self.uf = np.zeros(max(self.ob.largest, 1), np.int32)
        s = OrcTopo()
        s.n_bond, s.n_angle, s.n_type = t.n_bond, t.n_angle, t.n_type
        s.max_intra_moves = int(t.max_intra_moves)
        I = lambda a: a.ctypes.data_as(_ip)
        D = lambda a: a.ctypes.data_as(_dp)
        for k in ("bond_a1", "bond_a2", "bond_var", "angle_a1", "angle_a2", "angle_mid",
                  "angle_var", "mol_bond_start", "mol_bond_count", "mol_angle_start",
                  "mol_angle_count", "mol_type", "type_natom"):
            setattr(s, k, I(getattr(t, k)))
        for k in ("bond_k", "bond_eq", "bond_len", "angle_k", "angle_eq", "angle_size"):
            setattr(s, k, D(getattr(t, k)))
        s.bond_len_rb, s.angle_size_rb = D(self.bond_len_rb), D(self.angle_size_rb)
        s.type_off, s.uf = I(self.type_off), I(self.uf)
        s.pair_code = t.pair_code.ctypes.data_as(C.POINTER(C.c_uint8))
        s.max_bond_delta, s.max_angle_delta = float(t.max_bond_delta), float(t.max_angle_delta)
        s.step_num = int(t.step_num)
        s.flex_bonds, s.flex_angles = int(t.flex_bonds), int(t.flex_angles)
        self.s = s

    @property
    def ref(self):
        return C.byref(self.s)

    def intra_energy(self, mol: int) -> float:
        return orc_lib().orc_intra_energy(self.ob.ref, self.ref, int(mol))

    def bond_energy(self, mol: int) -> float:
        return orc_lib().orc_bond_energy(self.ref, int(mol))

    def angle_energy(self, mol: int) -> float:
        return orc_lib().orc_angle_energy(self.ref, int(mol))

    def mol_energy(self, curr: int, start: int = 0) -> float:
        """SimulationStep::calcMoleculeEnergy with the intramolecular term."""
        return self.ob.mol_energy(curr, start) + self.intra_energy(curr)

    def system_energy(self) -> float:
        return orc_lib().orc_system_energy_intra(self.ob.ref, self.ref)

    def stretch_bond(self, mol: int, bond: int, dist: float) -> None:
        orc_lib().orc_stretch_bond(self.ob.ref, self.ref, int(mol), int(bond), float(dist))

    def expand_angle(self, mol: int, angle: int, deg: float) -> None:
        orc_lib().orc_expand_angle(self.ob.ref, self.ref, int(mol), int(angle), float(deg))

    def save(self, mol: int) -> None:
        orc_lib().orc_save_intra(self.ref, int(mol))

    def rollback(self, mol: int) -> None:
        """Coordinates, angle sizes and bond lengths back (rollback with
        ENABLE_INTRA)."""
        self.ob.rollback(mol)
        orc_lib().orc_rollback_intra(self.ref, int(mol))

    def intramolecular_move(self, mol: int) -> None:
        orc_lib().orc_intramolecular_move(self.ob.ref, self.ref, int(mol))

    def run_plain(self, steps: int, e0: float) -> tuple[float, int]:
        acc = C.c_int()
        e = orc_lib().orc_run_plain_intra(self.ob.ref, self.ref, int(steps), float(e0),
                                          C.byref(acc))
        return e, acc.value

    def state(self) -> dict:
        s = self.s
        return dict(bond_len=self.t.bond_len.copy(), angle_size=self.t.angle_size.copy(),
                    max_bond_delta=s.max_bond_delta, max_angle_delta=s.max_angle_delta,
                    step_num=s.step_num, bond_moves=s.bond_moves,
                    bond_accepted=s.bond_accepted, angle_moves=s.angle_moves,
                    angle_accepted=s.angle_accepted)

    def coords(self) -> np.ndarray:
        return self.ob.coords()


class OracleChain:
    """The device-resident chain form on the CPU: the same FP32 moves of the
    same fixed-point + FP32-offset state (bit for bit), FP64 energies with
    the reference's arithmetic on the state's FP64 rows."""

    def __init__(self, box, rot_mode: int):
        self.ob = OracleBox(box)
        b = self.ob.data
        self.A = np.zeros(3 * b.n_mol, dtype=np.uint32)
        self.q = np.zeros(4 * b.n_mol, dtype=np.float32)
        self.tpl = np.zeros(3 * b.n_atom, dtype=np.float32)
        self.off = np.zeros(3 * b.n_atom, dtype=np.float32)
        # largest molecule radius about its first primary atom, as the device
        # header holds it (FP32)
        rad = 0.0
        for m in range(b.n_mol):
            an = int(b.pidx[b.mol_pidx_start[m]])
            for a in range(int(b.mol_start[m]), int(b.mol_start[m] + b.mol_len[m])):
                dx, dy, dz = b.x[a] - b.x[an], b.y[a] - b.y[an], b.z[a] - b.z[an]
                rad = max(rad, math.sqrt(dx * dx + dy * dy + dz * dz))
        self.rad_max = float(np.float32(rad))
        fp = C.POINTER(C.c_float)
        self.s = OrcChainS(C.pointer(self.ob.s), self.A.ctypes.data_as(C.POINTER(C.c_uint32)),
                           self.q.ctypes.data_as(fp), self.tpl.ctypes.data_as(fp),
                           self.off.ctypes.data_as(fp), int(rot_mode))
        orc_lib().orc_fchain_init(C.byref(self.s))

    def draw(self, seed: int, chain: int, step: int) -> OrcMoveF:
        mv = OrcMoveF()
        orc_lib().orc_fchain_draw(C.byref(self.s), int(seed) & (2 ** 64 - 1), int(chain),
                                  int(step), C.byref(mv))
        return mv

    def run(self, seed: int, chain: int, n_steps: int, e0: float, step0: int = 0):
        tr = (OrcTrace * max(1, n_steps))()
        acc = C.c_longlong()
        e = orc_lib().orc_fchain_run(C.byref(self.s), int(seed) & (2 ** 64 - 1), int(chain),
                                     int(step0), int(n_steps), float(e0), tr, C.byref(acc))
        return e, acc.value, list(tr)[:n_steps]

    def run_window(self, seed: int, chain: int, n_steps: int, e0: float, window: int,
                   step0: int = 0, in_range_rule: bool = True):
        """run() in windows of `window` steps (orc_fchain_run_window): each
        step evaluated on its window's start state and again only when an
        earlier accepted step of the window moved its molecule or one in
        range of it (in_range_rule=False drops the latter: a planted
        mistake).  Returns (energy, accepted, trace, re-evaluated steps)."""
        tr = (OrcTrace * max(1, n_steps))()
        acc, redo = C.c_longlong(), C.c_longlong()
        e = orc_lib().orc_fchain_run_window(C.byref(self.s), int(seed) & (2 ** 64 - 1),
                                            int(chain), int(step0), int(n_steps), int(window),
                                            float(e0), tr, C.byref(acc), C.byref(redo),
                                            1 if in_range_rule else 0)
        return e, acc.value, list(tr)[:n_steps], redo.value

    def system_energy(self) -> float:
        return self.ob.system_energy()

    def coords(self) -> np.ndarray:
        return self.ob.coords()

    # 1 atm in kcal/mol/A^3 (101325 Pa * 1e-30 m^3/A^3 * N_A / 4184 J/kcal)
    ATM_KCAL = 101325 * 6.02214076e23 * 1e-30 / 4184

    def volume_move(self, seed: int, chain: int, step: int, pressure_atm: float,
                    max_dlnv: float, energy: float, lrc_v: float = 0.0) -> dict:
        """One isobaric ln V move at step count `step` (orc_fchain_volume);
        returns the outcome (1, 0, or -1 for rejected outright), both FP64
        energies, the draws and the energy after the decision."""
        e = C.c_double(energy)
        eo, en, dl, u = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        st = orc_lib().orc_fchain_volume(
            C.byref(self.s), int(seed) & (2 ** 64 - 1), int(chain), int(step),
            float(pressure_atm) * self.ATM_KCAL, float(max_dlnv), self.rad_max, float(lrc_v),
            C.byref(e),
            C.byref(eo), C.byref(en), C.byref(dl), C.byref(u))
        return {"status": st, "e_old": eo.value, "e_new": en.value, "dlnv": dl.value,
                "u": u.value, "energy": e.value, "edge": float(self.ob.s.size[0])}


def build_centres(seed: int, n: int, L: float, dmin: float) -> np.ndarray:
    """Molecule centres by random sequential addition (orc_build_centres):
    the same points as the product's input builder, without loading the
    product library (for the CPU baseline's workload)."""
    out = np.empty((n, 3), dtype=np.float64)
    rc = orc_lib().orc_build_centres(int(n), float(L), float(dmin), int(seed) & (2 ** 64 - 1),
                                     out.ctypes.data_as(_dp))
    if rc != 0:
        raise RuntimeError(f"could not place {n} centres at dmin {dmin} in L {L} (status {rc})")
    return out


def sincos_f32(x: float) -> tuple[float, float]:
    s, c = C.c_float(), C.c_float()
    orc_lib().orc_sincos_f32(float(x), C.byref(s), C.byref(c))
    return s.value, c.value


def philox(ctr, key) -> list[int]:
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (C.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (C.c_uint32 * 4)()
    orc_lib().orc_philox4x32_10(c, k, o)
    return list(o)


def chains_run_mt(boxes: list[OracleBox], seeds, n_steps: int, mode: int, threads: int,
                  step0: int = 0) -> int:
    """Advances every chain by n_steps (steps step0 .. step0 + n_steps - 1 of
    its Philox stream) on `threads` host threads; returns the moves made."""
    n = len(boxes)
    arr = (OrcBox * n)(*[b.s for b in boxes])
    sd = (C.c_uint64 * n)(*[int(s) & (2 ** 64 - 1) for s in seeds])
    moves = C.c_longlong()
    orc_lib().orc_chains_run_mt(arr, n, sd, int(step0), int(n_steps), int(mode), int(threads),
                                C.byref(moves))
    return moves.value


class RefHarness:
    """The reference's own CPU path (compiled from its sources) behind the
    white-box harness.  One global SimBox per process (the reference keeps
    its state in globals: SimCalcs::sb, GPUCopy's row tables, rand())."""

    def __init__(self):
        if not REF_SO.exists():
            raise FileNotFoundError(f"{REF_SO} not built (needs the reference sources)")
        L = C.CDLL(str(REF_SO))
        protos = {
            "ref_box_create": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                         _ip, _ip, _ip, _ip, _ip, _dp, C.c_double, C.c_double,
                                         C.c_double, C.c_double]),
            "ref_mol_energy": (C.c_double, [C.c_int, C.c_int]),
            "ref_system_energy": (C.c_double, []),
            "ref_apply_move": (None, [C.c_int, C.c_int] + [C.c_double] * 6),
            "ref_intermolecular_move": (None, [C.c_int]),
            "ref_rollback": (None, [C.c_int]),
            "ref_accept": (C.c_int, [C.c_double]),
            "ref_choose_molecule": (C.c_int, []),
            "ref_seed": (None, [C.c_int]),
            "ref_rand": (C.c_int, []),
            "ref_wrap_all": (None, []),
            "ref_get_coords": (None, [_dp, _dp, _dp]),
            "ref_run_plain": (C.c_double, [C.c_int, C.c_double, C.POINTER(C.c_int)]),
            "ref_load": (C.c_int, [C.c_char_p] + [C.POINTER(C.c_int)] * 3
                         + [C.POINTER(C.c_long)] * 2),
            "ref_load_rows": (None, [_dp] * 6 + [_ip] * 6 + [_dp, _dp]),
            "ref_load_lrc": (C.c_double, []),
            "ref_load_seed": (C.c_int, []),
            "ref_load_write_state": (None, [C.c_char_p, C.c_int]),
            "ref_load_set_coords": (None, [_dp, _dp, _dp]),
            "ref_load_activate": (None, []),
            "ref_topology_counts": (None, [C.POINTER(C.c_int)] * 3),
            "ref_topology_rows": (None, [_ip, _ip, _dp, _dp, _dp, _ip, _ip, _ip, _ip, _dp, _dp,
                                         _dp, _ip, _ip, _ip, _ip, _ip, _ip, _dp]),
            "ref_type_codes": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_uint8)]),
            "ref_set_topology": (None, [C.c_int, _ip, _ip, _dp, _dp, _dp, _ip,
                                        C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _ip,
                                        _ip, _ip, _ip, _ip, _ip, C.c_int, _ip,
                                        C.POINTER(C.c_uint8), C.c_double, C.c_double,
                                        C.c_int, C.c_int]),
            "ref_intra_energy": (C.c_double, [C.c_int]),
            "ref_bond_energy": (C.c_double, [C.c_int]),
            "ref_angle_energy": (C.c_double, [C.c_int]),
            "ref_stretch_bond": (None, [C.c_int, C.c_int, C.c_double]),
            "ref_expand_angle": (None, [C.c_int, C.c_int, C.c_double]),
            "ref_save_intra": (None, [C.c_int]),
            "ref_intramolecular_move": (None, [C.c_int]),
            "ref_intra_rollback": (None, [C.c_int]),
            "ref_mol_energy_intra": (C.c_double, [C.c_int, C.c_int]),
            "ref_system_energy_intra": (C.c_double, []),
            "ref_intra_state": (None, [_dp, _dp, _dp]),
            "ref_set_step": (None, [C.c_int]),
            "ref_run_plain_intra": (C.c_double, [C.c_int, C.c_double, C.POINTER(C.c_int)]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        self.L = L
        self.n_atom = 0

    def load(self, box) -> None:
        b = box.copy().normalise()
        self._keep = b
        size = np.ascontiguousarray(b.size, dtype=np.float64)
        self._size = size
        self.L.ref_box_create(b.n_mol, b.n_atom, b.n_pidx, *(getattr(b, k).ctypes.data_as(_dp)
                              for k in ("x", "y", "z", "sigma", "epsilon", "charge")),
                              *(getattr(b, k).ctypes.data_as(_ip) for k in
                                ("mol_start", "mol_len", "mol_pidx_start", "mol_pidx_count",
                                 "pidx")),
                              size.ctypes.data_as(_dp), b.cutoff, b.temperature,
                              b.max_translate, b.max_rotate)
        self.n_atom = b.n_atom

    def load_files(self, path: str) -> dict:
        """The reference's own loader on a .config or .state (run from the
        file's directory, as metrosim resolves the paths inside it):
        the SimBox rows it builds, its LRC, seed, start step and steps."""
        nm, na, npi = C.c_int(), C.c_int(), C.c_int()
        st, n = C.c_long(), C.c_long()
        cwd = os.getcwd()
        d, f = os.path.split(os.path.abspath(path))
        os.chdir(d)
        try:
            rc = self.L.ref_load(f.encode(), C.byref(nm), C.byref(na), C.byref(npi),
                                 C.byref(st), C.byref(n))
        finally:
            os.chdir(cwd)
        if rc:
            raise RuntimeError("the reference could not load " + path)
        na_, nm_ = na.value, nm.value
        out = {k: np.empty(na_) for k in ("x", "y", "z", "sigma", "epsilon", "charge")}
        out.update({k: np.empty(nm_, np.int32) for k in ("mol_start", "mol_len", "mol_type",
                                                         "mol_pidx_start", "mol_pidx_count")})
        out["pidx"] = np.empty(npi.value, np.int32)
        out["size"] = np.empty(3)
        out["params"] = np.empty(5)
        self.L.ref_load_rows(*(out[k].ctypes.data_as(_dp) for k in
                               ("x", "y", "z", "sigma", "epsilon", "charge")),
                             *(out[k].ctypes.data_as(_ip) for k in
                               ("mol_start", "mol_len", "mol_type", "mol_pidx_start",
                                "mol_pidx_count", "pidx")),
                             out["size"].ctypes.data_as(_dp), out["params"].ctypes.data_as(_dp))
        self._loaded_atoms = na_
        out["lrc"] = self.L.ref_load_lrc()
        out["seed"] = self.L.ref_load_seed()
        out["start_step"] = st.value
        out["steps"] = n.value
        return out

    def write_loaded_state(self, path: str, step: int, xyz=None) -> None:
        """StateScanner::outputState of the loaded box, at its own
        coordinates or at xyz (n_atom x 3)."""
        if xyz is not None:
            c = [np.ascontiguousarray(xyz[:, k], dtype=np.float64) for k in range(3)]
            self.L.ref_load_set_coords(*(v.ctypes.data_as(_dp) for v in c))
        self.L.ref_load_write_state(os.path.abspath(path).encode(), int(step))

    def activate_loaded(self) -> None:
        """Makes the SimBox of the last load_files the one the step functions
        act on (its rows, bonds, angles and exclusion lists as the
        reference's loader built them)."""
        self.L.ref_load_activate()
        self.n_atom = self._loaded_atoms

    def topology(self, type_natom) -> dict:
        """The current SimBox's bond/angle rows, per-molecule ranges and
        types, per-type pair codes (type_natom atoms each, as the
        reference's exclusion and fudge lists give them) and
        params = [maxBondDelta, maxAngleDelta, maxIntraMoves,
        hasFlexibleBonds, hasFlexibleAngles, stepNum]."""
        nb, na, nm = C.c_int(), C.c_int(), C.c_int()
        self.L.ref_topology_counts(C.byref(nb), C.byref(na), C.byref(nm))
        nb, na, nm = nb.value, na.value, nm.value
        o = {k: np.empty(nb, np.int32) for k in ("bond_a1", "bond_a2", "bond_var")}
        o.update({k: np.empty(nb) for k in ("bond_k", "bond_eq", "bond_len")})
        o.update({k: np.empty(na, np.int32) for k in ("angle_a1", "angle_a2", "angle_mid",
                                                      "angle_var")})
        o.update({k: np.empty(na) for k in ("angle_k", "angle_eq", "angle_size")})
        o.update({k: np.empty(nm, np.int32) for k in ("mol_bond_start", "mol_bond_count",
                                                      "mol_angle_start", "mol_angle_count",
                                                      "mol_type")})
        o["params"] = np.empty(6)
        I = lambda k: o[k].ctypes.data_as(_ip)
        D = lambda k: o[k].ctypes.data_as(_dp)
        self.L.ref_topology_rows(I("bond_a1"), I("bond_a2"), D("bond_k"), D("bond_eq"),
                                 D("bond_len"), I("bond_var"), I("angle_a1"), I("angle_a2"),
                                 I("angle_mid"), D("angle_k"), D("angle_eq"), D("angle_size"),
                                 I("angle_var"), I("mol_bond_start"), I("mol_bond_count"),
                                 I("mol_angle_start"), I("mol_angle_count"), I("mol_type"),
                                 D("params"))
        codes = []
        for t, n in enumerate(type_natom):
            c = np.zeros(int(n) * int(n), np.uint8)
            if n and self.L.ref_type_codes(t, int(n), c.ctypes.data_as(C.POINTER(C.c_uint8))):
                raise RuntimeError("type %d has no exclusion lists" % t)
            codes.append(c)
        o["pair_code"] = np.concatenate(codes) if codes else np.zeros(0, np.uint8)
        return o

    def set_topology(self, t) -> None:
        """Installs a Topology (mcgpu_gb300.workloads) on the current SimBox."""
        t = t.copy().normalise()
        self._topo = t
        I = lambda k: getattr(t, k).ctypes.data_as(_ip)
        D = lambda k: getattr(t, k).ctypes.data_as(_dp)
        self.L.ref_set_topology(t.n_bond, I("bond_a1"), I("bond_a2"), D("bond_k"), D("bond_eq"),
                                D("bond_len"), I("bond_var"), t.n_angle, I("angle_a1"),
                                I("angle_a2"), I("angle_mid"), D("angle_k"), D("angle_eq"),
                                D("angle_size"), I("angle_var"), I("mol_bond_start"),
                                I("mol_bond_count"), I("mol_angle_start"), I("mol_angle_count"),
                                I("mol_type"), t.n_type, I("type_natom"),
                                t.pair_code.ctypes.data_as(C.POINTER(C.c_uint8)),
                                float(t.max_bond_delta), float(t.max_angle_delta),
                                int(t.max_intra_moves), int(t.step_num))

    def intra_state(self, n_bond: int, n_angle: int) -> tuple:
        """(bond lengths, angle sizes, [maxBondDelta, maxAngleDelta, stepNum,
        numBondMoves, numAcceptedBondMoves, numAngleMoves,
        numAcceptedAngleMoves])."""
        bl, asz, out = np.empty(max(n_bond, 1)), np.empty(max(n_angle, 1)), np.empty(7)
        self.L.ref_intra_state(bl.ctypes.data_as(_dp), asz.ctypes.data_as(_dp),
                               out.ctypes.data_as(_dp))
        return bl[:n_bond], asz[:n_angle], out

    def coords(self) -> np.ndarray:
        x, y, z = np.empty(self.n_atom), np.empty(self.n_atom), np.empty(self.n_atom)
        self.L.ref_get_coords(x.ctypes.data_as(_dp), y.ctypes.data_as(_dp), z.ctypes.data_as(_dp))
        return np.stack([x, y, z], axis=1)

    def __getattr__(self, name):
        return getattr(self.L, "ref_" + name)
