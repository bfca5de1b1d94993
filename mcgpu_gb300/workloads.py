"""Synthetic boxes for the trial-move energy path.

``BoxData`` holds one box as the SimBox rows of the reference
(src/Metropolis/SimBox.h:120-149): FP64 coordinates, sigma/epsilon/charge,
molecule start/length/primary-index ranges and absolute primary indexes.

The generators build the workloads the path is measured on (seeded, so every
run gets the same inputs):

* ``water_box``     rigid 3-site TIP3P-like water (O q -0.834, sigma 3.1506,
                    eps 0.1521; H q +0.417, sigma = eps = 0; r_OH 0.9572 A,
                    HOH 104.52 deg), centres uniform with a rejection-resampled
                    minimum O-O distance, orientations uniform on SO(3).
* ``bicyclic_box``  rigid 16-atom planar fused 6+5 ring molecule (8 C, 1 N,
                    7 H at 1.08 A radially outward), seeded neutral charges.
* ``water_chains``  many independent water chains of log-uniform size at
                    1.0 g/cc with uneven temperatures.

Every box is wrapped by its first primary atom as Simulation::run does before
its loop (Simulation.cpp:70-72).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi

WATER_DENSITY = 0.03343          # molecules / A^3 (1.0 g/cc)
BICYCLIC_DENSITY = 4000 / 86.1 ** 3


@dataclass
class BoxData:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    sigma: np.ndarray
    epsilon: np.ndarray
    charge: np.ndarray
    mol_start: np.ndarray
    mol_len: np.ndarray
    mol_pidx_start: np.ndarray
    mol_pidx_count: np.ndarray
    pidx: np.ndarray
    size: np.ndarray
    cutoff: float
    temperature: float
    max_translate: float
    max_rotate: float
    name: str = ""
    _keep: list = field(default_factory=list, repr=False, compare=False)

    @property
    def n_mol(self) -> int:
        return int(self.mol_start.shape[0])

    @property
    def n_atom(self) -> int:
        return int(self.x.shape[0])

    @property
    def n_pidx(self) -> int:
        return int(self.pidx.shape[0])

    def copy(self) -> "BoxData":
        return BoxData(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                          for k, v in self.__dict__.items() if k != "_keep"})

    def normalise(self) -> "BoxData":
        f64 = ("x", "y", "z", "sigma", "epsilon", "charge", "size")
        i32 = ("mol_start", "mol_len", "mol_pidx_start", "mol_pidx_count", "pidx")
        for k in f64:
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64))
        for k in i32:
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32))
        return self

    def desc(self) -> _abi.BoxDesc:
        """A C descriptor pointing at this box's arrays (valid while self lives)."""
        self.normalise()
        d = _abi.BoxDesc()
        d.n_mol, d.n_atom, d.n_pidx = self.n_mol, self.n_atom, self.n_pidx
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        for k in ("x", "y", "z", "sigma", "epsilon", "charge"):
            setattr(d, k, getattr(self, k).ctypes.data_as(dp))
        for k in ("mol_start", "mol_len", "mol_pidx_start", "mol_pidx_count", "pidx"):
            setattr(d, k, getattr(self, k).ctypes.data_as(ip))
        for i in range(3):
            d.size[i] = float(self.size[i])
        d.cutoff = self.cutoff
        d.temperature = self.temperature
        d.max_translate = self.max_translate
        d.max_rotate = self.max_rotate
        return d

    def wrap(self) -> "BoxData":
        """keepMoleculeInBox for every molecule (SimulationStep.cpp:710-729):
        shift a molecule by one box edge when its first primary atom is
        below 0 or above L in that dimension."""
        p = self.pidx[self.mol_pidx_start]
        mol_of_atom = np.repeat(np.arange(self.n_mol), self.mol_len)
        atoms = np.concatenate([np.arange(s, s + n) for s, n in zip(self.mol_start, self.mol_len)]) \
            if self.n_mol else np.zeros(0, dtype=np.int64)
        for arr, L in ((self.x, self.size[0]), (self.y, self.size[1]), (self.z, self.size[2])):
            pv = arr[p]
            shift = np.where(pv < 0, L, np.where(pv > L, -L, 0.0))
            sh = shift[mol_of_atom]
            moved = sh != 0
            arr[atoms[moved]] += sh[moved]
        return self


# Pair codes of the intramolecular non-bonded terms: excluded (bonded or an
# angle's ends), scaled by 0.5 (three bonds apart), full.
PAIR_EXCLUDED, PAIR_FUDGE, PAIR_FULL = 0, 1, 2


@dataclass
class Topology:
    """The SimBox rows of flexible molecules (src/Metropolis/SimBox.h:160-300,
    filled by SimBoxBuilder.cpp:136-278): per bond its two atoms (box atom
    indexes), force constant, equilibrium and current length, variable flag;
    per angle its two ends and middle atom, force constant, equilibrium and
    current size (degrees), variable flag; per molecule its bond and angle
    ranges and type; per molecule type the intramolecular pair codes
    (``pair_code``: each type's natom x natom matrix, row-major,
    concatenated), built from the exclusion and fudge lists of the first
    molecule of the type.  ``max_bond_delta`` / ``max_angle_delta`` are the
    move widths, ``max_intra_moves`` the cap on bonds or angles moved at once
    (15 in the reference), ``step_num`` the simulation step the tuning
    counts from."""
    bond_a1: np.ndarray
    bond_a2: np.ndarray
    bond_k: np.ndarray
    bond_eq: np.ndarray
    bond_len: np.ndarray
    bond_var: np.ndarray
    angle_a1: np.ndarray
    angle_a2: np.ndarray
    angle_mid: np.ndarray
    angle_k: np.ndarray
    angle_eq: np.ndarray
    angle_size: np.ndarray
    angle_var: np.ndarray
    mol_bond_start: np.ndarray
    mol_bond_count: np.ndarray
    mol_angle_start: np.ndarray
    mol_angle_count: np.ndarray
    mol_type: np.ndarray
    type_natom: np.ndarray
    pair_code: np.ndarray
    max_bond_delta: float = 0.06
    max_angle_delta: float = 3.1
    max_intra_moves: int = 15
    step_num: int = 0

    @property
    def n_bond(self) -> int:
        return int(self.bond_a1.shape[0])

    @property
    def n_angle(self) -> int:
        return int(self.angle_a1.shape[0])

    @property
    def n_type(self) -> int:
        return int(self.type_natom.shape[0])

    @property
    def flex_bonds(self) -> bool:
        """SimBox::hasFlexibleBonds: some bond is variable."""
        return bool(np.any(self.bond_var != 0))

    @property
    def flex_angles(self) -> bool:
        """SimBox::hasFlexibleAngles: some angle is variable."""
        return bool(np.any(self.angle_var != 0))

    def copy(self) -> "Topology":
        return Topology(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                           for k, v in self.__dict__.items()})

    def normalise(self) -> "Topology":
        for k in ("bond_k", "bond_eq", "bond_len", "angle_k", "angle_eq", "angle_size"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64))
        for k in ("bond_a1", "bond_a2", "bond_var", "angle_a1", "angle_a2", "angle_mid",
                  "angle_var", "mol_bond_start", "mol_bond_count", "mol_angle_start",
                  "mol_angle_count", "mol_type", "type_natom"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32))
        self.pair_code = np.ascontiguousarray(self.pair_code, dtype=np.uint8)
        return self

    def type_codes(self, t: int) -> np.ndarray:
        """Type t's pair-code matrix."""
        off = int(np.sum(self.type_natom[:t].astype(np.int64) ** 2))
        n = int(self.type_natom[t])
        return self.pair_code[off:off + n * n].reshape(n, n)

    def desc(self) -> _abi.TopoDesc:
        """A C descriptor pointing at these rows (valid while self lives)."""
        self.normalise()
        d = _abi.TopoDesc()
        d.n_bond, d.n_angle, d.n_type = self.n_bond, self.n_angle, self.n_type
        d.max_intra_moves = int(self.max_intra_moves)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        for k in ("bond_k", "bond_eq", "bond_len", "angle_k", "angle_eq", "angle_size"):
            setattr(d, k, getattr(self, k).ctypes.data_as(dp))
        for k in ("bond_a1", "bond_a2", "bond_var", "angle_a1", "angle_a2", "angle_mid",
                  "angle_var", "mol_bond_start", "mol_bond_count", "mol_angle_start",
                  "mol_angle_count", "mol_type", "type_natom"):
            setattr(d, k, getattr(self, k).ctypes.data_as(ip))
        d.pair_code = self.pair_code.ctypes.data_as(C.POINTER(C.c_uint8))
        d.max_bond_delta = float(self.max_bond_delta)
        d.max_angle_delta = float(self.max_angle_delta)
        d.step_num = int(self.step_num)
        return d


# ---- geometry -----------------------------------------------------------------

def water_template() -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray, int]:
    """O at the origin, both H in the xy plane; returns xyz, sigma, eps, q, primary."""
    r, th = 0.9572, math.radians(104.52)
    xyz = np.array([[0.0, 0.0, 0.0], [r, 0.0, 0.0], [r * math.cos(th), r * math.sin(th), 0.0]])
    sig = np.array([3.1506, 0.0, 0.0])
    eps = np.array([0.1521, 0.0, 0.0])
    q = np.array([-0.834, 0.417, 0.417])
    return xyz, sig, eps, q, 0


def bicyclic_template(charge_seed: int = 7) -> tuple[np.ndarray, np.ndarray, np.ndarray,
                                                       np.ndarray, int]:
    """Planar fused 6+5 ring, 1.40 A bonds: a regular hexagon sharing one edge
    with a regular pentagon; N on the pentagon next to a fused atom, C
    elsewhere; H at 1.08 A radially outward from its ring centre on every
    unfused ring atom.  Origin at the heavy-atom centroid."""
    s = 1.40
    hexc = np.zeros(2)
    hexv = [s * np.array([math.cos(math.radians(60 * k + 30)), math.sin(math.radians(60 * k + 30))])
            for k in range(6)]
    rp = s / (2 * math.sin(math.radians(36)))
    pc = np.array([s * math.cos(math.radians(30)) + rp * math.cos(math.radians(36)), 0.0])
    penta = {a: pc + rp * np.array([math.cos(math.radians(a)), math.sin(math.radians(a))])
             for a in (72, 0, 288)}
    heavy = [penta[72], penta[0], penta[288], hexv[5], hexv[4], hexv[3], hexv[2], hexv[1], hexv[0]]
    centres = [pc, pc, pc, None, hexc, hexc, hexc, hexc, None]
    hs = []
    for p, c in zip(heavy, centres):
        if c is None:
            continue
        d = p - c
        hs.append(p + 1.08 * d / np.linalg.norm(d))
    pts = np.array(heavy + hs)
    xyz = np.zeros((16, 3))
    xyz[:, :2] = pts
    xyz[:9] -= 0  # keep layout explicit
    cen = xyz[:9].mean(axis=0)
    xyz -= cen
    sig = np.array([3.25] + [3.55] * 8 + [2.42] * 7)
    eps = np.array([0.17] + [0.07] * 8 + [0.03] * 7)
    rng = np.random.default_rng(charge_seed)
    q = rng.uniform(-0.3, 0.3, 16)
    q -= q.mean()
    return xyz, sig, eps, q, 0


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """n rotation matrices uniform on SO(3) (Shoemake's unit quaternions)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    qx, qy = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    qz, qw = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (qy * qy + qz * qz)
    R[:, 0, 1] = 2 * (qx * qy - qz * qw)
    R[:, 0, 2] = 2 * (qx * qz + qy * qw)
    R[:, 1, 0] = 2 * (qx * qy + qz * qw)
    R[:, 1, 1] = 1 - 2 * (qx * qx + qz * qz)
    R[:, 1, 2] = 2 * (qy * qz - qx * qw)
    R[:, 2, 0] = 2 * (qx * qz - qy * qw)
    R[:, 2, 1] = 2 * (qy * qz + qx * qw)
    R[:, 2, 2] = 1 - 2 * (qx * qx + qy * qy)
    return R


def rsa_centres(seed: int, n: int, L: float, dmin: float) -> np.ndarray:
    """n points uniform in [0, L)^3 with minimum-image separation >= dmin, by
    random sequential addition (every rejected candidate redrawn); native
    code in the library (mcgpu_build_centres)."""
    out = np.empty((n, 3), dtype=np.float64)
    rc = _abi.lib().mcgpu_build_centres(int(n), float(L), float(dmin),
                                        int(seed) & (2 ** 64 - 1),
                                        out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise RuntimeError(f"could not place {n} centres at dmin {dmin} in L {L} (status {rc})")
    return out


def fcc_centres(seed: int, n: int, L: float) -> np.ndarray:
    """n sites of a face-centred cubic lattice filling the cubic box: the
    smallest k with 4 k^3 >= n cells per edge, lattice constant L / k, a
    seeded random choice of n of the 4 k^3 sites (all of them when they
    match, e.g. 4000 molecules at k = 10).  The reference builds its boxes
    on such a lattice (FileUtilities.cpp:550-642)."""
    k = 1
    while 4 * k ** 3 < n:
        k += 1
    a = L / k
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cells = np.array([(i, j, l) for i in range(k) for j in range(k) for l in range(k)], float)
    sites = ((cells[:, None, :] + base[None]) * a + 0.25 * a).reshape(-1, 3)
    if sites.shape[0] > n:
        pick = np.sort(np.random.default_rng(seed).choice(sites.shape[0], n, replace=False))
        sites = sites[pick]
    return sites


def aligned_rotation(xyz: np.ndarray, a: float, seed: int, tries: int = 4096) -> np.ndarray:
    """One orientation for every molecule of an FCC lattice of constant a:
    among `tries` seeded uniform rotations, the one with the largest closest
    approach between a molecule's atoms and those of its 12 nearest lattice
    neighbours (farther shells are at least a apart)."""
    nb = []
    for v in ((0.5, 0.5, 0.0), (0.5, 0.0, 0.5), (0.0, 0.5, 0.5)):
        idx = [i for i in range(3) if v[i]]
        for s1 in (1.0, -1.0):
            for s2 in (1.0, -1.0):
                w = np.array(v) * a
                w[idx[0]] *= s1
                w[idx[1]] *= s2
                nb.append(w)
    nb = np.array(nb)
    R = random_rotations(np.random.default_rng(seed), tries)
    best, best_R = -1.0, R[0]
    for c in range(0, tries, 256):
        p = np.einsum("rij,aj->rai", R[c:c + 256], xyz)           # (r, atoms, 3)
        d = p[:, None, :, None, :] + nb[None, :, None, None, :] - p[:, None, None, :, :]
        m = np.sqrt(np.einsum("rnabk,rnabk->rnab", d, d)).min(axis=(1, 2, 3))
        k = int(np.argmax(m))
        if m[k] > best:
            best, best_R = float(m[k]), R[c + k]
    return best_R


def _close_atom_pairs(pos: np.ndarray, check: np.ndarray, L: float, dmin: float):
    """Molecule pairs (i, j), i in `check`, with an atom pair of different
    molecules closer than dmin (minimum image); pos is (n_mol, a, 3)."""
    n_mol, a, _ = pos.shape
    xyz = (pos.reshape(-1, 3) % L)
    mol = np.repeat(np.arange(n_mol), a)
    nc = max(1, int(L // dmin))
    cw = L / nc
    c3 = np.minimum((xyz / cw).astype(np.int64), nc - 1)
    cid = (c3[:, 0] * nc + c3[:, 1]) * nc + c3[:, 2]
    order = np.argsort(cid, kind="stable")
    counts = np.bincount(cid, minlength=nc ** 3)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    table = -np.ones((nc ** 3, int(counts.max())), dtype=np.int64)
    table[cid[order], np.arange(xyz.shape[0]) - starts[cid[order]]] = order
    sel = np.nonzero(np.isin(mol, check))[0]
    span = (-1, 0, 1) if nc >= 3 else (0,)
    offs = np.array([(i, j, k) for i in span for j in span for k in span])
    nb = (c3[sel][:, None, :] + offs[None]) % nc
    cand = table[(nb[..., 0] * nc + nb[..., 1]) * nc + nb[..., 2]].reshape(sel.size, -1)
    if nc < 3:
        cand = np.broadcast_to(np.arange(xyz.shape[0]), (sel.size, xyz.shape[0]))
    valid = cand >= 0
    cj = np.where(valid, cand, 0)
    valid &= mol[cj] != mol[sel][:, None]
    d = xyz[cj] - xyz[sel][:, None, :]
    d -= L * np.rint(d / L)
    close = valid & (np.einsum("bij,bij->bi", d, d) < dmin * dmin)
    ii, kk = np.nonzero(close)
    return mol[sel[ii]], mol[cj[ii, kk]]


def _place(xyz, R, centres):
    pos = np.empty((R.shape[0], xyz.shape[0], 3))
    for r in range(3):
        pos[:, :, r] = (R[:, r, 0, None] * xyz[None, :, 0] + R[:, r, 1, None] * xyz[None, :, 1]
                        + R[:, r, 2, None] * xyz[None, :, 2]) + centres[:, r, None]
    return pos


def build_box(template, n_mol: int, L: float, cutoff: float, temperature: float,
              max_translate: float, max_rotate: float, seed: int, dmin: float,
              name: str = "", atom_dmin: float = 0.0, overlap_rounds: int = 200,
              lattice: bool = False, centres=None) -> BoxData:
    """Places n_mol copies of a rigid template: centres by random sequential
    addition at minimum separation dmin and orientations uniform on SO(3),
    or (lattice=True) centres on an FCC lattice all in one orientation, the
    one keeping neighbouring molecules' atoms farthest apart.  With atom_dmin > 0, molecules with an atom closer than
    atom_dmin to another molecule's atom are re-oriented (and, off the
    lattice, re-centred after repeated failures) for up to overlap_rounds
    rounds; at liquid density some overlaps may remain, as in the
    reference's own lattice starts.  `centres(seed, n, L, dmin)` replaces
    the random-sequential-addition builder (it must place the same points)."""
    xyz, sig, eps, q, prim = template
    a = xyz.shape[0]
    rng = np.random.default_rng(seed)
    if lattice:
        centres = fcc_centres(seed, n_mol, L)
    else:
        centres = (centres or rsa_centres)(seed, n_mol, L, dmin)
    if lattice:
        k = 1
        while 4 * k ** 3 < n_mol:
            k += 1
        R = np.broadcast_to(aligned_rotation(xyz, L / k, seed), (n_mol, 3, 3)).copy()
    else:
        R = random_rotations(rng, n_mol)
    # pos[m, i, :] = R[m] @ xyz[i] + centre[m], elementwise (same bits on every host)
    pos = _place(xyz, R, centres)
    if atom_dmin > 0 and n_mol > 1:
        tries = np.zeros(n_mol, dtype=np.int64)
        check = np.arange(n_mol)
        for _ in range(overlap_rounds):
            i, j = _close_atom_pairs(pos, check, L, atom_dmin)
            if i.size == 0:
                break
            bad = np.unique(np.maximum(i, j))
            tries[bad] += 1
            R[bad] = random_rotations(rng, bad.size)
            recentre = bad[tries[bad] % 8 == 0] if not lattice else bad[:0]
            if recentre.size:
                centres[recentre] = rng.random((recentre.size, 3)) * L
            pos[bad] = _place(xyz, R[bad], centres[bad])
            check = bad
    box = BoxData(
        x=pos[:, :, 0].ravel().copy(), y=pos[:, :, 1].ravel().copy(), z=pos[:, :, 2].ravel().copy(),
        sigma=np.tile(sig, n_mol), epsilon=np.tile(eps, n_mol), charge=np.tile(q, n_mol),
        mol_start=np.arange(n_mol, dtype=np.int32) * a,
        mol_len=np.full(n_mol, a, dtype=np.int32),
        mol_pidx_start=np.arange(n_mol, dtype=np.int32),
        mol_pidx_count=np.ones(n_mol, dtype=np.int32),
        pidx=(np.arange(n_mol, dtype=np.int32) * a + prim).astype(np.int32),
        size=np.array([L, L, L], dtype=np.float64), cutoff=float(cutoff),
        temperature=float(temperature), max_translate=float(max_translate),
        max_rotate=float(max_rotate), name=name)
    return box.normalise().wrap()


def water_box(n_mol: int = 256, L: float | None = None, cutoff: float = 9.0,
              temperature: float = 298.15, max_translate: float = 0.15, max_rotate: float = 15.0,
              seed: int = 12345, dmin: float = 2.5, centres=None) -> BoxData:
    if L is None:
        L = (n_mol / WATER_DENSITY) ** (1.0 / 3.0)
    return build_box(water_template(), n_mol, L, cutoff, temperature, max_translate, max_rotate,
                     seed, dmin, name=f"water{n_mol}", centres=centres)


def bicyclic_box(n_mol: int = 4000, L: float | None = None, cutoff: float = 12.0,
                 temperature: float = 298.0, max_translate: float = 0.2, max_rotate: float = 10.0,
                 seed: int = 4000, dmin: float = 4.0, atom_dmin: float = 0.0,
                 lattice: bool = False) -> BoxData:
    """The 16-atom bicyclic liquid: random centres at a 4 A minimum centre
    distance, random orientations.  At this density ring atoms of
    neighbouring molecules overlap in the start (as in the reference's own
    lattice start of its 4000-indole example); atom_dmin > 0 re-orients
    overlapping molecules where the density allows."""
    if L is None:
        L = (n_mol / BICYCLIC_DENSITY) ** (1.0 / 3.0)
    return build_box(bicyclic_template(), n_mol, L, cutoff, temperature, max_translate,
                     max_rotate, seed, dmin, name=f"bicyclic{n_mol}", atom_dmin=atom_dmin,
                     lattice=lattice)


def water_chains(n_chains: int = 512, n_min: int = 64, n_max: int = 2048, seed: int = 2024,
                 t_range=(280.0, 360.0), max_translate: float = 0.15,
                 max_rotate: float = 15.0, centres=None) -> tuple[list[BoxData], np.ndarray]:
    """Independent water chains: N log-uniform in [n_min, n_max], L for
    1.0 g/cc, cutoff min(9, L/2), T uniform in t_range; returns the boxes and
    one 64-bit Philox key per chain.  `centres` replaces the centre builder
    (same signature as rsa_centres)."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_chains))).astype(int)
    temps = rng.uniform(t_range[0], t_range[1], n_chains)
    seeds = rng.integers(1, 2 ** 63 - 1, n_chains, dtype=np.int64).astype(np.uint64)
    boxes = []
    for c in range(n_chains):
        n = int(sizes[c])
        L = (n / WATER_DENSITY) ** (1.0 / 3.0)
        boxes.append(water_box(n, L=L, cutoff=min(9.0, L / 2), temperature=float(temps[c]),
                               max_translate=max_translate, max_rotate=max_rotate,
                               seed=int(seed * 100003 + c), centres=centres))
    return boxes, seeds


# ---- the measured workloads, by name --------------------------------------------
#
# One constructor per measured configuration, so the benchmark and the parity
# tests build bit-identical inputs.

def batch_water_512(seed: int = 2024, centres=None) -> tuple[list[BoxData], np.ndarray]:
    """512 independent NVT water chains, N log-uniform in [64, 2048] at
    1.0 g/cc, T uniform in [280, 360] K, cutoff min(9, L/2), +-0.15 A /
    +-15 deg moves: the batched headline workload."""
    return water_chains(512, n_min=64, n_max=2048, seed=seed, centres=centres)


def bicyclic_4000() -> BoxData:
    """4000 rigid 16-atom bicyclic molecules, L = 86.1 A, rc 12 A, 298 K,
    +-0.2 A / +-10 deg, on an FCC lattice (10^3 cells hold the 4000 centres
    exactly) in one common orientation: the single-chain workload."""
    return bicyclic_box(4000, L=86.1, seed=4000, lattice=True)


def flex_amine_water(n_mol: int = 512, files_dir=None):
    """The flexible-molecule workload: alternating flexible amine chains (9
    atoms: N, three C, five H; every bond and angle variable, so each move
    also stretches a random set of bonds and opens a random set of angles)
    and rigid 3-site waters, from the synthetic inputs flex.config / flex.z /
    synth.par / oplsaa.sb (tests/golden/files), with N molecules and the
    edge scaled to keep the configuration's density; built by the package's
    loader (FCC lattice, implied angles on).  Returns (BoxData, Topology)."""
    import os
    from pathlib import Path
    from . import files as F
    d = Path(files_dir) if files_dir else Path(__file__).resolve().parents[1] / "tests" / \
        "golden" / "files"
    edge = 19.0 * (n_mol / 48) ** (1 / 3)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        si = F.load("flex.config", implied_angles=True,
                    env={"n_molecules": int(n_mol), "x": edge, "y": edge, "z": edge})
    finally:
        os.chdir(cwd)
    return si.rows, si.topology


def water_32768() -> BoxData:
    """32,768 waters (98,304 atoms), L = 99.3 A, rc 12 A, 298 K: the large
    single system (NPT at 1 atm with Verlet lists in its measurement)."""
    return water_box(32768, L=99.3, cutoff=12.0, temperature=298.0, seed=32768)
