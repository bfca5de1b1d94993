"""Generates tests/golden/intra_flex.npz from the REFERENCE's own compiled CPU
path, as it runs with ENABLE_INTRA true (its intramolecular functions are
compiled in; the harness composes them at the three call sites the flag
gates: molecule energy, change, rollback).

Input: tests/golden/files/flex.config (24 flexible amine chains with every
bond and angle variable, 24 rigid waters; our own synthetic parameter tables
synth.par and oplsaa.sb).  The SimBox rows come from the reference's own
loader; the bond / angle / exclusion rows are this package's loader's with the
implied angles on (files.load(..., implied_angles=True)), installed into the
reference's SimBox by the harness, because the reference's z-matrix scanner
starts its implied-angle flag uninitialised (ZmatrixScanner.h) and its loader
was seen to build either row set from one run to the next.  The loader's rows
are checked against the reference's for the flag value the reference took
(here, and in tests/test_intra_oracle.py).  Run where the MCGPU sources are
available:

    make -C oracle ref && python tests/golden/gen_intra_golden.py

Stored (``box_*``: the SimBox rows the reference's loader built; ``topo_*``:
the installed bond / angle / exclusion rows; so the tests never need the
reference):

* ``intra_e``, ``bond_e``, ``angle_e``  calcIntraMolecularEnergy, bondEnergy,
                                        angleEnergy of every molecule
* ``sys_energy``                        calcSystemEnergy with the intra term
* ``op_*``    60 trial moves with injected draws: the rigid move
              (rotateAtom / translateAtom / keepMoleculeInBox), saveBonds /
              saveAngles, one to four stretchBond / expandAngle with given
              amounts, the molecule energies before and after, rollback
              (coordinates, angle sizes, bond lengths) of the rejected ones;
              then the final coordinates, lengths and sizes
* ``im_*``    300 intramolecularMove calls drawing from rand() (seeded),
              with the step counter set to 1000 and 2000 on two of them (the
              width tuning), the intramolecular energy after each, the final
              coordinates, lengths, sizes, widths and counters
* ``traj_*``  Simulation::run's loop with the intramolecular term and move,
              2500 steps from srand(4321): initial and final energy, accepted
              count, coordinates, lengths, sizes, widths and counters
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mcgpu_gb300 import files as F  # noqa: E402
from mcgpu_gb300.workloads import BoxData, Topology  # noqa: E402
from oracle.pyoracle import RefHarness  # noqa: E402

OUT = Path(__file__).resolve().parent / "intra_flex.npz"
CONFIG = Path(__file__).resolve().parent / "files" / "flex.config"
TOPO_KEYS = ("bond_a1", "bond_a2", "bond_k", "bond_eq", "bond_len", "bond_var", "angle_a1",
             "angle_a2", "angle_mid", "angle_k", "angle_eq", "angle_size", "angle_var",
             "mol_bond_start", "mol_bond_count", "mol_angle_start", "mol_angle_count",
             "mol_type", "pair_code")


def package_topology(implied: bool) -> Topology:
    cwd = os.getcwd()
    os.chdir(CONFIG.parent)
    try:
        return F.load(CONFIG.name, implied_angles=implied).topology
    finally:
        os.chdir(cwd)


def check_loader(R: RefHarness, natom) -> bool:
    """The package loader's rows equal the reference loader's for the
    implied-angle flag the reference took; returns that flag."""
    ref = R.topology(natom)
    for implied in (False, True):
        t = package_topology(implied)
        if all(np.array_equal(getattr(t, k), ref[k]) for k in TOPO_KEYS):
            return implied
    raise AssertionError("the package loader's topology differs from the reference's")


def load(R: RefHarness):
    rows = R.load_files(str(CONFIG))
    R.activate_loaded()
    n_mol = rows["mol_start"].shape[0]
    # atoms of each type's first molecule
    natom = []
    for t in range(int(rows["mol_type"].max()) + 1):
        m = int(np.argmax(rows["mol_type"] == t))
        natom.append(int(rows["mol_len"][m]))
    flag = check_loader(R, np.array(natom, np.int32))
    print(f"reference loader: implied angles {'on' if flag else 'off'}; package rows equal")
    t = package_topology(True)
    R.set_topology(t)
    box = BoxData(x=rows["x"], y=rows["y"], z=rows["z"], sigma=rows["sigma"],
                  epsilon=rows["epsilon"], charge=rows["charge"], mol_start=rows["mol_start"],
                  mol_len=rows["mol_len"], mol_pidx_start=rows["mol_pidx_start"],
                  mol_pidx_count=rows["mol_pidx_count"], pidx=rows["pidx"], size=rows["size"],
                  cutoff=rows["params"][0], temperature=rows["params"][1],
                  max_translate=rows["params"][3], max_rotate=rows["params"][4],
                  name="flex").normalise()
    assert box.n_mol == n_mol
    return box, t


def arrays(box: BoxData, t: Topology) -> dict:
    out = {f"box_{k}": getattr(box, k) for k in
           ("x", "y", "z", "sigma", "epsilon", "charge", "mol_start", "mol_len",
            "mol_pidx_start", "mol_pidx_count", "pidx", "size")}
    out["box_scalars"] = np.array([box.cutoff, box.temperature, box.max_translate,
                                   box.max_rotate])
    out.update({f"topo_{k}": getattr(t, k) for k in TOPO_KEYS + ("type_natom",)})
    out["topo_scalars"] = np.array([t.max_bond_delta, t.max_angle_delta, t.max_intra_moves,
                                    t.step_num])
    return out


def state(R: RefHarness, t: Topology, prefix: str) -> dict:
    bl, asz, st = R.intra_state(t.n_bond, t.n_angle)
    return {f"{prefix}_coords": R.coords(), f"{prefix}_bond_len": bl.copy(),
            f"{prefix}_angle_size": asz.copy(), f"{prefix}_state": st.copy()}


def main() -> None:
    R = RefHarness()
    box, t = load(R)
    out = arrays(box, t)
    n = box.n_mol
    out["intra_e"] = np.array([R.L.ref_intra_energy(m) for m in range(n)])
    out["bond_e"] = np.array([R.L.ref_bond_energy(m) for m in range(n)])
    out["angle_e"] = np.array([R.L.ref_angle_energy(m) for m in range(n)])
    out["sys_energy"] = np.array([R.L.ref_system_energy_intra()])

    # injected trial moves
    rng = np.random.default_rng(77)
    n_moves = 60
    mols = rng.integers(0, n, n_moves).astype(np.int32)
    verts = np.array([rng.integers(0, box.mol_len[m]) for m in mols], np.int32)
    d = rng.uniform(-box.max_translate, box.max_translate, (n_moves, 3))
    r = rng.uniform(-box.max_rotate, box.max_rotate, (n_moves, 3))
    acc = (rng.random(n_moves) < 0.5).astype(np.int32)
    ops = []          # (move, kind 0 bond / 1 angle, index, amount)
    e_old, e_new, e_ops = np.empty(n_moves), np.empty(n_moves), []
    for k in range(n_moves):
        m = int(mols[k])
        e_old[k] = R.L.ref_mol_energy_intra(m, 0)
        R.L.ref_apply_move(m, int(verts[k]), *d[k], *r[k])
        R.L.ref_save_intra(m)
        for _ in range(int(rng.integers(1, 5))):
            if rng.random() < 0.5 and t.mol_bond_count[m]:
                i, amt = int(rng.integers(0, t.mol_bond_count[m])), float(rng.uniform(-0.08, 0.08))
                R.L.ref_stretch_bond(m, i, amt)
                ops.append((k, 0, i, amt))
            elif t.mol_angle_count[m]:
                i, amt = int(rng.integers(0, t.mol_angle_count[m])), float(rng.uniform(-6, 6))
                R.L.ref_expand_angle(m, i, amt)
                ops.append((k, 1, i, amt))
            e_ops.append(R.L.ref_intra_energy(m))
        e_new[k] = R.L.ref_mol_energy_intra(m, 0)
        if not acc[k]:
            R.L.ref_intra_rollback(m)
    op = np.array(ops)
    out.update(op_mol=mols, op_vertex=verts, op_d=d, op_r=r, op_accept=acc, op_eold=e_old,
               op_enew=e_new, op_move=op[:, 0].astype(np.int32), op_kind=op[:, 1].astype(np.int32),
               op_index=op[:, 2].astype(np.int32), op_amount=op[:, 3], op_eintra=np.array(e_ops))
    out.update(state(R, t, "op"))

    # rand()-driven intramolecular moves, from a fresh load
    box, t = load(R)
    R.L.ref_seed(99)
    im_mols = rng.integers(0, n, 300).astype(np.int32)
    im_steps = np.full(300, -1, np.int32)
    im_steps[120], im_steps[250] = 1000, 2000
    im_e = np.empty(300)
    for k, m in enumerate(im_mols):
        if im_steps[k] >= 0:
            R.L.ref_set_step(int(im_steps[k]))
        R.L.ref_intramolecular_move(int(m))
        im_e[k] = R.L.ref_intra_energy(int(m))
    out.update(im_seed=np.array([99]), im_mol=im_mols, im_step=im_steps, im_energy=im_e)
    out.update(state(R, t, "im"))

    # the reference's loop with the intramolecular term and move
    box, t = load(R)
    e0 = R.L.ref_system_energy_intra()
    R.L.ref_seed(4321)
    a = C.c_int()
    e = R.L.ref_run_plain_intra(2500, e0, C.byref(a))
    out.update(traj_seed=np.array([4321]), traj_steps=np.array([2500]), traj_e0=np.array([e0]),
               traj_energy=np.array([e]), traj_accepted=np.array([a.value]),
               traj_recompute=np.array([R.L.ref_system_energy_intra()]))
    out.update(state(R, t, "traj"))
    np.savez_compressed(OUT, **out)
    print(f"{OUT.name}: {n} molecules, {t.n_bond} bonds, {t.n_angle} angles, "
          f"E0 {e0:.6f}, after 2500 steps {e:.6f}, accepted {a.value}")


if __name__ == "__main__":
    cwd = os.getcwd()
    try:
        main()
    finally:
        os.chdir(cwd)
