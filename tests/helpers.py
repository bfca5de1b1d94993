"""Shared helpers of the tests: golden fixtures and tolerances."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from mcgpu_gb300.workloads import BoxData

GOLDEN = Path(__file__).resolve().parent / "golden"
GOLDEN_NAMES = ["water256", "t3p64", "bicyclic100", "mixed", "water48_halfbox"]

# FP32 pair terms: |err| <= REL * max(|E|, FLOOR * sum_t k_t |t|), the sum over
# the pair terms of each term's magnitude times its condition number with
# respect to the pair distance (k = 12 for 4 eps s^12, 6 for 4 eps s^6, 1 for
# Coulomb; OracleBox.mol_energy_abs): FP32 positions carry a relative error of
# order 1e-7 that each term amplifies by k, so at close LJ contacts the plain
# sum of |terms| under-states the rounding scale twelvefold.
REL = 1e-5
FLOOR = 1e-3
# FP64 pair terms, different summation order only
REL64 = 1e-11


def load_golden(name: str) -> tuple[BoxData, dict]:
    z = dict(np.load(GOLDEN / f"{name}.npz"))
    s = z["box_scalars"]
    box = BoxData(x=z["box_x"], y=z["box_y"], z=z["box_z"], sigma=z["box_sigma"],
                  epsilon=z["box_epsilon"], charge=z["box_charge"], mol_start=z["box_mol_start"],
                  mol_len=z["box_mol_len"], mol_pidx_start=z["box_mol_pidx_start"],
                  mol_pidx_count=z["box_mol_pidx_count"], pidx=z["box_pidx"], size=z["box_size"],
                  cutoff=float(s[0]), temperature=float(s[1]), max_translate=float(s[2]),
                  max_rotate=float(s[3]), name=name).normalise()
    return box, z


def tol_mixed(ref: float, abs_sum: float) -> float:
    return REL * max(abs(ref), FLOOR * abs_sum)


def tol64(ref: float, abs_sum: float = 0.0) -> float:
    return REL64 * max(abs(ref), abs_sum, 1.0)


TOPO_KEYS = ("bond_a1", "bond_a2", "bond_k", "bond_eq", "bond_len", "bond_var", "angle_a1",
             "angle_a2", "angle_mid", "angle_k", "angle_eq", "angle_size", "angle_var",
             "mol_bond_start", "mol_bond_count", "mol_angle_start", "mol_angle_count",
             "mol_type", "type_natom", "pair_code")


def load_intra_golden():
    """tests/golden/intra_flex.npz: the box, its Topology and the vectors."""
    from mcgpu_gb300.workloads import Topology
    box, z = load_golden("intra_flex")
    s = z["topo_scalars"]
    topo = Topology(**{k: z[f"topo_{k}"] for k in TOPO_KEYS}, max_bond_delta=float(s[0]),
                    max_angle_delta=float(s[1]), max_intra_moves=int(s[2]),
                    step_num=int(s[3])).normalise()
    return box, topo, z


def random_flex_box(seed: int, n_mol: int = 12):
    """A small box of random flexible molecules for the live comparisons:
    trees of 4-9 atoms (1.5 A bonds) with one extra ring-closing bond in
    every third molecule, angles at every pair of bonds sharing an atom,
    plus per molecule one angle whose middle is an end (its expansion is
    undefined: zero normal) and one whose middle is another molecule's
    atom; random variable flags and parameters; exclusion codes from the
    bonds and angle ends, 0.5 for atoms three bonds apart.  One molecule
    type per molecule."""
    from mcgpu_gb300.workloads import BoxData, Topology
    rng = np.random.default_rng(seed)
    L = 30.0
    xs, sig, eps, q = [], [], [], []
    ms, ml = [], []
    b = {k: [] for k in ("a1", "a2", "k", "eq", "len", "var")}
    a = {k: [] for k in ("a1", "a2", "mid", "k", "eq", "size", "var")}
    mbs, mbc, mas, mac, natom, codes = [], [], [], [], [], []
    side = int(np.ceil(n_mol ** (1 / 3)))
    for m in range(n_mol):
        n = int(rng.integers(4, 10))
        start = len(xs)
        centre = (np.array([m % side, (m // side) % side, m // side ** 2]) + 0.5) * (L / side)
        parent = [-1] + [int(rng.integers(0, i)) for i in range(1, n)]
        pos = [centre]
        for i in range(1, n):
            d = rng.normal(size=3)
            pos.append(pos[parent[i]] + 1.5 * d / np.linalg.norm(d))
        xs.extend(pos)
        sig.extend(rng.uniform(1.0, 3.0, n))
        eps.extend(rng.uniform(0.01, 0.2, n))
        qq = rng.uniform(-0.3, 0.3, n)
        q.extend(qq - qq.mean())
        ms.append(start)
        ml.append(n)
        edges = [(i, parent[i]) for i in range(1, n)]
        if m % 3 == 0 and n > 3:
            edges.append((n - 1, 0) if parent[n - 1] != 0 else (n - 1, 1))
        mbs.append(len(b["a1"]))
        mbc.append(len(edges))
        for (i, j) in edges:
            b["a1"].append(start + i)
            b["a2"].append(start + j)
            b["k"].append(float(rng.uniform(200, 500)))
            b["eq"].append(1.5 + float(rng.uniform(-0.05, 0.05)))
            b["len"].append(float(np.linalg.norm(pos[i] - pos[j])))
            b["var"].append(int(rng.random() < 0.8))
        adj = [[] for _ in range(n)]
        for (i, j) in edges:
            adj[i].append(j)
            adj[j].append(i)
        trip = [(i, c, j) for c in range(n) for x, i in enumerate(adj[c]) for j in adj[c][x + 1:]]
        trip.append((1, 0, 0))                   # middle == an end
        mas.append(len(a["a1"]))
        for (i, c, j) in trip:
            a["a1"].append(start + i)
            a["a2"].append(start + j)
            a["mid"].append(start + c)
        a["a1"].append(start + n - 1)            # middle in molecule 0
        a["a2"].append(start + n - 2)
        a["mid"].append(0)
        for _ in range(len(trip) + 1):
            a["k"].append(float(rng.uniform(20, 60)))
            a["eq"].append(float(rng.uniform(100, 120)))
            a["size"].append(float(rng.uniform(100, 120)))
            a["var"].append(int(rng.random() < 0.8))
        mac.append(len(trip) + 1)
        dist = np.full((n, n), 99)
        for s0 in range(n):
            dist[s0, s0] = 0
            fr = [s0]
            while fr:
                nx = []
                for u in fr:
                    for v in adj[u]:
                        if dist[s0, v] == 99:
                            dist[s0, v] = dist[s0, u] + 1
                            nx.append(v)
                fr = nx
        c = np.full((n, n), 2, np.uint8)
        c[dist == 3] = 1
        for (i, j) in edges:
            c[i, j] = c[j, i] = 0
        for (i, _, j) in trip:
            c[i, j] = c[j, i] = 0
        natom.append(n)
        codes.append(c.ravel())
    xyz = np.array(xs)
    box = BoxData(x=xyz[:, 0].copy(), y=xyz[:, 1].copy(), z=xyz[:, 2].copy(),
                  sigma=np.array(sig), epsilon=np.array(eps), charge=np.array(q),
                  mol_start=np.array(ms), mol_len=np.array(ml), mol_pidx_start=np.arange(n_mol),
                  mol_pidx_count=np.ones(n_mol), pidx=np.array(ms), size=np.array([L, L, L]),
                  cutoff=10.0, temperature=300.0, max_translate=0.2, max_rotate=10.0,
                  name=f"flexrand{seed}").normalise().wrap()
    topo = Topology(bond_a1=b["a1"], bond_a2=b["a2"], bond_k=b["k"], bond_eq=b["eq"],
                    bond_len=b["len"], bond_var=b["var"], angle_a1=a["a1"], angle_a2=a["a2"],
                    angle_mid=a["mid"], angle_k=a["k"], angle_eq=a["eq"], angle_size=a["size"],
                    angle_var=a["var"], mol_bond_start=mbs, mol_bond_count=mbc,
                    mol_angle_start=mas, mol_angle_count=mac, mol_type=np.arange(n_mol),
                    type_natom=natom, pair_code=np.concatenate(codes), max_bond_delta=0.08,
                    max_angle_delta=5.0).normalise()
    return box, topo


def intra_abs(box, topo, xyz, mol, bond_len=None, angle_size=None) -> float:
    """Sum of the magnitudes of the intramolecular terms of molecule mol at
    coordinates xyz (n_atom x 3): the rounding scale of an FP64 sum of them
    taken in a different order."""
    s, n = int(box.mol_start[mol]), int(box.mol_len[mol])
    t = int(topo.mol_type[mol])
    code = topo.type_codes(t)
    L = box.size
    tot = 0.0
    bl = topo.bond_len if bond_len is None else bond_len
    asz = topo.angle_size if angle_size is None else angle_size
    for k in range(topo.mol_bond_start[mol], topo.mol_bond_start[mol] + topo.mol_bond_count[mol]):
        if topo.bond_var[k]:
            tot += abs(topo.bond_k[k]) * (topo.bond_eq[k] - bl[k]) ** 2
    for k in range(topo.mol_angle_start[mol],
                   topo.mol_angle_start[mol] + topo.mol_angle_count[mol]):
        if topo.angle_var[k]:
            tot += abs(topo.angle_k[k]) * (topo.angle_eq[k] - asz[k]) ** 2
    for i in range(n):
        for j in range(i + 1, n):
            c = code[i, j] if i < code.shape[0] and j < code.shape[0] else 2
            if c == 0:
                continue
            d = xyz[s + j] - xyz[s + i]
            d -= L * (d < -0.5 * L) - L * (d > 0.5 * L)
            r2 = float(d @ d)
            if r2 == 0:
                continue
            sg = np.sqrt(abs(box.sigma[s + i] * box.sigma[s + j]))
            ep = np.sqrt(abs(box.epsilon[s + i] * box.epsilon[s + j]))
            s6 = (sg * sg / r2) ** 3
            term = 4 * ep * (s6 * s6 + s6) + abs(box.charge[s + i] * box.charge[s + j]
                                                  * 332.06) / np.sqrt(r2)
            tot += (0.5 if c == 1 else 1.0) * term
    return tot
