"""Generates tests/golden/*.npz from the REFERENCE's own compiled CPU path.

Run in a checkout where the MCGPU sources are available (default
/root/reference, or $MCGPU_REFERENCE):

    make -C oracle ref && python tests/golden/gen_golden.py

Each fixture stores its full input box (so tests never regenerate inputs)
and the reference's outputs:

* ``sys_energy``                 SimulationStep::calcSystemEnergy
* ``me_curr/me_start/me_val``    BruteForceCalcs::calcMolecularEnergyContribution
                                 for sampled (currMol, startMol)
* ``mv_*``                       a sequence of injected trial moves applied
                                 through the reference's rotateAtom /
                                 translateAtom / keepMoleculeInBox, with the
                                 old and new molecule energies, an accept
                                 flag per move (rejected moves rolled back
                                 through SimCalcs::rollback) and the final
                                 coordinates
* ``traj_*`` (water256 only)     Simulation::run's NVT loop driven by the
                                 reference's own rand() from srand(seed):
                                 final energy, accepted count, coordinates
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mcgpu_gb300 import workloads as W  # noqa: E402
from oracle.pyoracle import RefHarness  # noqa: E402

OUT = Path(__file__).resolve().parent


def t3p_box(n_mol=64, seed=11):
    """TIP3P as the reference's t3p.z lays it out: O, two dummy sites with
    sigma = epsilon = -1 and zero charge (skipped by the pair loop), then
    the two H (resources/bossFiles/t3p.z, ZmatrixScanner.cpp:131-139)."""
    xyz, sig, eps, q, _ = W.water_template()
    t = (np.array([xyz[0], xyz[0] + [0.0, 0.0, 1.0], xyz[0] + [0.0, 1.0, 0.0], xyz[1], xyz[2]]),
         np.array([sig[0], -1.0, -1.0, sig[1], sig[2]]),
         np.array([eps[0], -1.0, -1.0, eps[1], eps[2]]),
         np.array([q[0], 0.0, 0.0, q[1], q[2]]), 0)
    L = (n_mol / W.WATER_DENSITY) ** (1 / 3)
    return W.build_box(t, n_mol, L, 9.0, 298.15, 0.15, 15.0, seed, 2.5, name="t3p64")


def mixed_box(seed=13):
    """Two molecule types in one box: 3-site water (one primary) and the
    16-atom bicyclic molecule with TWO primary indexes (N and the far ring
    carbon), so the any-primary-pair cutoff rule is exercised."""
    wb = W.water_box(120, L=24.0, seed=seed, dmin=2.6)
    bb = W.build_box(W.bicyclic_template(), 24, 24.0, 9.0, 298.15, 0.15, 15.0, seed + 1, 7.0,
                     atom_dmin=2.5)
    # move the bicyclic molecules into the water box, drop waters they overlap
    bxyz = np.stack([bb.x, bb.y, bb.z], 1)
    wo = np.stack([wb.x[wb.pidx], wb.y[wb.pidx], wb.z[wb.pidx]], 1)
    keep = []
    for m in range(wb.n_mol):
        d = bxyz - wo[m]
        d -= 24.0 * np.rint(d / 24.0)
        if np.min(np.einsum("ij,ij->i", d, d)) > 2.8 ** 2:
            keep.append(m)
    keep = np.array(keep)
    na_w = 3 * keep.size
    wx = np.concatenate([wb.x[3 * m:3 * m + 3] for m in keep])
    wy = np.concatenate([wb.y[3 * m:3 * m + 3] for m in keep])
    wz = np.concatenate([wb.z[3 * m:3 * m + 3] for m in keep])
    nb = bb.n_mol
    far = 4  # hexagon atom opposite the fused edge
    box = W.BoxData(
        x=np.concatenate([wx, bb.x]), y=np.concatenate([wy, bb.y]), z=np.concatenate([wz, bb.z]),
        sigma=np.concatenate([np.tile(wb.sigma[:3], keep.size), bb.sigma]),
        epsilon=np.concatenate([np.tile(wb.epsilon[:3], keep.size), bb.epsilon]),
        charge=np.concatenate([np.tile(wb.charge[:3], keep.size), bb.charge]),
        mol_start=np.concatenate([np.arange(keep.size) * 3, na_w + np.arange(nb) * 16]),
        mol_len=np.concatenate([np.full(keep.size, 3), np.full(nb, 16)]),
        mol_pidx_start=np.concatenate([np.arange(keep.size), keep.size + 2 * np.arange(nb)]),
        mol_pidx_count=np.concatenate([np.ones(keep.size), np.full(nb, 2)]),
        pidx=np.concatenate([np.arange(keep.size) * 3,
                             np.stack([na_w + np.arange(nb) * 16,
                                       na_w + np.arange(nb) * 16 + far], 1).ravel()]),
        size=np.array([24.0, 24.0, 24.0]), cutoff=9.0, temperature=298.15, max_translate=0.15,
        max_rotate=15.0, name="mixed")
    return box.normalise().wrap()


def boxes():
    return {
        "water256": W.water_box(256, L=19.71, seed=12345),
        "t3p64": t3p_box(),
        # a quarter of the liquid density, so no ring atoms overlap in the start
        "bicyclic100": W.build_box(W.bicyclic_template(), 100, 40.0, 12.0, 298.0, 0.2, 10.0, 4000,
                                   5.0, name="bicyclic100", atom_dmin=2.5),
        "mixed": mixed_box(),
        # cutoff at half the box edge: many atom pairs need their own image
        "water48_halfbox": W.water_box(48, cutoff=None or ((48 / W.WATER_DENSITY) ** (1 / 3)) / 2,
                                       seed=99),
    }


def box_arrays(b):
    return {f"box_{k}": getattr(b, k) for k in
            ("x", "y", "z", "sigma", "epsilon", "charge", "mol_start", "mol_len",
             "mol_pidx_start", "mol_pidx_count", "pidx", "size")} | {
        "box_scalars": np.array([b.cutoff, b.temperature, b.max_translate, b.max_rotate])}


def gen_one(name, b, ref: RefHarness, n_moves=150, seed=1):
    rng = np.random.default_rng(seed)
    ref.load(b)
    out = box_arrays(b)
    out["sys_energy"] = np.array([ref.system_energy()])
    cur = rng.integers(0, b.n_mol, 24)
    st = np.where(rng.random(24) < 0.5, 0, cur)
    out["me_curr"], out["me_start"] = cur.astype(np.int32), st.astype(np.int32)
    out["me_val"] = np.array([ref.mol_energy(int(c), int(s)) for c, s in zip(cur, st)])
    mols = rng.integers(0, b.n_mol, n_moves).astype(np.int32)
    verts = np.array([rng.integers(0, b.mol_len[m]) for m in mols], dtype=np.int32)
    d = rng.uniform(-b.max_translate, b.max_translate, (n_moves, 3))
    r = rng.uniform(-b.max_rotate, b.max_rotate, (n_moves, 3))
    acc = (rng.random(n_moves) < 0.6).astype(np.int32)
    eo, en = np.empty(n_moves), np.empty(n_moves)
    for k in range(n_moves):
        m = int(mols[k])
        eo[k] = ref.mol_energy(m, 0)
        ref.apply_move(m, int(verts[k]), *d[k], *r[k])
        en[k] = ref.mol_energy(m, 0)
        if not acc[k]:
            ref.rollback(m)
    out.update(mv_mol=mols, mv_vertex=verts, mv_d=d, mv_r=r, mv_accept=acc, mv_eold=eo,
               mv_enew=en, mv_final=ref.coords())
    return out


def gen_traj(b, ref: RefHarness, seed=42, steps=3000):
    ref.load(b)
    e0 = ref.system_energy()
    ref.seed(seed)
    import ctypes as C
    acc = C.c_int()
    e = ref.run_plain(steps, e0, C.byref(acc))
    return {"traj_seed": np.array([seed]), "traj_steps": np.array([steps]),
            "traj_e0": np.array([e0]), "traj_energy": np.array([e]),
            "traj_accepted": np.array([acc.value]), "traj_final": ref.coords()}


def main():
    ref = RefHarness()
    for name, b in boxes().items():
        out = gen_one(name, b, ref)
        if name == "water256":
            out.update(gen_traj(b, ref))
        np.savez_compressed(OUT / f"{name}.npz", **out)
        print(name, b.n_mol, "molecules", out["sys_energy"][0])


if __name__ == "__main__":
    main()
