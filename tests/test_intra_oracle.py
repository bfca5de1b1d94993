"""Flexible molecules (bond stretches, angle expansions, the intramolecular
energy) on the CPU: the `.sb` reader and the loader's bond / angle /
exclusion rows, and the oracle restatement against the reference's golden
vectors (tests/golden/intra_flex.npz, made by tests/golden/gen_intra_golden.py
from the compiled reference running its intramolecular code as with
ENABLE_INTRA true) -- bit for bit, NaN included.  Where the compiled
reference is present, the same against it live, on random topologies with
rings, a degenerate angle (middle == end: zero normal, NaN coordinates) and
middles in other molecules."""
import ctypes as C
import os
from pathlib import Path

import numpy as np
import pytest

from helpers import TOPO_KEYS, load_intra_golden, random_flex_box
from mcgpu_gb300 import files as F
from mcgpu_gb300.step import LibcRand
from oracle.pyoracle import REF_SO, OracleFlex

FILES = Path(__file__).resolve().parent / "golden" / "files"


def load_flex(implied=True):
    cwd = os.getcwd()
    os.chdir(FILES)
    try:
        return F.load("flex.config", implied_angles=implied)
    finally:
        os.chdir(cwd)


def test_sb_reader_rules(tmp_path):
    """SBScanner's rules: bond and angle lines by the sixth character, one-
    letter names padded, both orders stored, later lines overwrite, short
    lines skipped, the second end of an angle missing gives eq 0."""
    p = tmp_path / "oplsaa.sb"
    p.write_text("***** title\n"
                 "C -CT 317.       1.522        note\n"
                 "CT-HC 340.       1.090\n"
                 "CT-HC 331.       1.095\n"
                 "HC-CT-C   50.0   109.5\n"
                 "# comment\n"
                 "\"quoted\n"
                 "XY\n"
                 "\n")
    t = F.read_sb(str(p))
    assert t.k_bond("C", "CT") == 317.0 and t.eq_bond("CT", "C") == 1.522
    assert t.k_bond("HC", "CT") == 331.0 and t.eq_bond("CT", "HC") == 1.095
    assert t.k_angle("HC", "CT", "C") == 50.0 and t.eq_angle("C", "CT", "HC") == 109.5
    assert t.k_bond("C", "HC") == -1.0 and t.eq_bond("X", "Y") == -1.0
    assert t.k_angle("HC", "CT", "X") == -1.0
    assert t.eq_angle("HC", "CT", "X") == 0.0      # the reference's own value
    assert t.eq_angle("HC", "X", "C") == -1.0
    assert "XY" not in t.bonds and "X" not in t.bonds


def test_loader_rows_equal_golden():
    """The package loader on flex.config (implied angles on) gives the rows
    the golden vectors were made on."""
    box, topo, z = load_intra_golden()
    si = load_flex(True)
    for k in ("x", "y", "z", "sigma", "epsilon", "charge", "mol_start", "mol_len", "pidx"):
        assert np.array_equal(getattr(si.rows, k), getattr(box, k)), k
    for k in TOPO_KEYS:
        assert np.array_equal(getattr(si.topology, k), getattr(topo, k)), k
    assert si.topology.max_bond_delta == 0.05 and si.topology.max_angle_delta == 4.0
    assert si.topology.flex_bonds and si.topology.flex_angles


def test_loader_quirk_middle_atoms():
    """Without the implied angles the z-matrix angles keep middle 0 shifted
    by their copy's first atom (FileUtilities.cpp:508): the middle row of
    every angle of a copy set is that set's first atom."""
    si = load_flex(False)
    t, rows = si.topology, si.rows
    per = int(rows.mol_len[0] + rows.mol_len[1])
    for m in range(rows.n_mol):
        s, n = t.mol_angle_start[m], t.mol_angle_count[m]
        assert np.all(t.angle_mid[s:s + n] == (m // 2) * per)


def test_oracle_intra_energies_golden():
    box, topo, z = load_intra_golden()
    o = OracleFlex(box, topo)
    got = np.array([o.intra_energy(m) for m in range(box.n_mol)])
    assert np.array_equal(got, z["intra_e"])
    assert np.array_equal([o.bond_energy(m) for m in range(box.n_mol)], z["bond_e"])
    assert np.array_equal([o.angle_energy(m) for m in range(box.n_mol)], z["angle_e"])
    assert o.system_energy() == z["sys_energy"][0]


def test_oracle_injected_moves_golden():
    """Rigid move, save, stretches and expansions with given amounts,
    energies, rollbacks: the reference's values and final rows bit for bit."""
    box, topo, z = load_intra_golden()
    o = OracleFlex(box, topo)
    k_op = 0
    for k in range(len(z["op_mol"])):
        m = int(z["op_mol"][k])
        assert o.mol_energy(m, 0) == z["op_eold"][k]
        o.ob.apply_move(m, int(z["op_vertex"][k]), *z["op_d"][k], *z["op_r"][k])
        o.save(m)
        while k_op < len(z["op_move"]) and z["op_move"][k_op] == k:
            if z["op_kind"][k_op] == 0:
                o.stretch_bond(m, int(z["op_index"][k_op]), float(z["op_amount"][k_op]))
            else:
                o.expand_angle(m, int(z["op_index"][k_op]), float(z["op_amount"][k_op]))
            assert o.intra_energy(m) == z["op_eintra"][k_op]
            k_op += 1
        assert o.mol_energy(m, 0) == z["op_enew"][k]
        if not z["op_accept"][k]:
            o.rollback(m)
    assert np.array_equal(o.coords(), z["op_coords"])
    assert np.array_equal(o.t.bond_len, z["op_bond_len"])
    assert np.array_equal(o.t.angle_size, z["op_angle_size"])


def check_state(o: OracleFlex, z, prefix):
    st = o.state()
    ref = z[f"{prefix}_state"]
    assert np.array_equal(o.coords(), z[f"{prefix}_coords"])
    assert np.array_equal(st["bond_len"], z[f"{prefix}_bond_len"])
    assert np.array_equal(st["angle_size"], z[f"{prefix}_angle_size"])
    assert [st["max_bond_delta"], st["max_angle_delta"], st["step_num"], st["bond_moves"],
            st["bond_accepted"], st["angle_moves"], st["angle_accepted"]] == list(ref)


def test_oracle_intramolecular_moves_golden():
    """intramolecularMove drawing from rand(), with the width tuning at steps
    1000 and 2000."""
    box, topo, z = load_intra_golden()
    o = OracleFlex(box, topo)
    LibcRand(int(z["im_seed"][0]))
    for k, m in enumerate(z["im_mol"]):
        if z["im_step"][k] >= 0:
            o.s.step_num = int(z["im_step"][k])
        o.intramolecular_move(int(m))
        assert o.intra_energy(int(m)) == z["im_energy"][k]
    check_state(o, z, "im")


def test_oracle_plain_trajectory_golden():
    """Simulation::run's loop with the intramolecular term and move: the
    reference's energy, accepted count and final state bit for bit."""
    box, topo, z = load_intra_golden()
    o = OracleFlex(box, topo)
    e0 = o.system_energy()
    assert e0 == z["traj_e0"][0]
    LibcRand(int(z["traj_seed"][0]))
    e, acc = o.run_plain(int(z["traj_steps"][0]), e0)
    assert e == z["traj_energy"][0] and acc == z["traj_accepted"][0]
    check_state(o, z, "traj")
    assert o.system_energy() == z["traj_recompute"][0]


def test_topology_descriptor():
    """The C descriptor points at the rows the Topology holds."""
    _, topo, _ = load_intra_golden()
    d = topo.desc()
    assert d.n_bond == topo.n_bond and d.n_angle == topo.n_angle and d.n_type == 2
    assert d.bond_a1[5] == topo.bond_a1[5] and d.angle_mid[7] == topo.angle_mid[7]
    assert d.pair_code[10] == topo.pair_code[10] and d.max_angle_delta == 4.0


# ---- live, against the compiled reference --------------------------------------

live = pytest.mark.skipif(not REF_SO.exists(), reason="reference harness not built")


@pytest.fixture(scope="module")
def ref():
    from oracle.pyoracle import RefHarness
    return RefHarness()


@live
def test_loader_rows_match_reference_loader(ref):
    """The reference's SimBoxBuilder rows for flex.config and mixv.config
    equal the package loader's for the implied-angle setting the reference's
    uninitialised flag took in this process."""
    for name in ("flex.config", "mixv.config"):
        ref.load_files(str(FILES / name))
        ref.activate_loaded()
        cwd = os.getcwd()
        os.chdir(FILES)
        try:
            cands = [F.load(name, implied_angles=v).topology for v in (False, True)]
        finally:
            os.chdir(cwd)
        r = ref.topology(cands[0].type_natom)
        assert any(all(np.array_equal(getattr(t, k), r[k]) for k in TOPO_KEYS if k != "type_natom")
                   for t in cands), name


@live
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_topologies_vs_reference(ref, seed):
    """Random molecules: energies, stretches, expansions (rings left alone,
    the degenerate angle giving NaN), save / rollback, rand()-driven
    intramolecular moves and a short loop -- the reference's values bit
    for bit, NaN for NaN."""
    box, topo = random_flex_box(seed)
    ref.load(box)
    ref.set_topology(topo)
    o = OracleFlex(box, topo)
    same = lambda a, b: np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)
    for m in range(box.n_mol):
        assert same(o.intra_energy(m), ref.L.ref_intra_energy(m))
    rng = np.random.default_rng(seed)
    nan_seen = False
    for k in range(150):
        m = int(rng.integers(0, box.n_mol))
        if k % 10 == 0:
            o.save(m)
            ref.L.ref_save_intra(m)
        if rng.random() < 0.5:
            i, d = int(rng.integers(0, topo.mol_bond_count[m])), float(rng.uniform(-0.1, 0.1))
            o.stretch_bond(m, i, d)
            ref.L.ref_stretch_bond(m, i, d)
        else:
            i, d = int(rng.integers(0, topo.mol_angle_count[m])), float(rng.uniform(-6, 6))
            o.expand_angle(m, i, d)
            ref.L.ref_expand_angle(m, i, d)
        assert same(o.coords(), ref.coords()), k
        e = o.intra_energy(m)
        nan_seen |= bool(np.isnan(e))
        assert same(e, ref.L.ref_intra_energy(m)), k
        if k % 10 == 9:
            ref.L.ref_intra_rollback(m)
            o.rollback(m)
            # the rollback rows of the rigid move were never set: both
            # restore the same scratch
            assert same(o.coords(), ref.coords())
    assert nan_seen
    bl, asz, _ = ref.intra_state(topo.n_bond, topo.n_angle)
    assert same(bl, o.t.bond_len) and same(asz, o.t.angle_size)
    # rand()-driven moves and the loop from a fresh copy of both
    box, topo = random_flex_box(seed)
    ref.load(box)
    ref.set_topology(topo)
    o = OracleFlex(box, topo)
    e0 = o.system_energy()
    assert same(e0, ref.L.ref_system_energy_intra())
    LibcRand(seed)
    e, acc = o.run_plain(400, e0)
    ref.L.ref_seed(seed)
    a = C.c_int()
    er = ref.L.ref_run_plain_intra(400, e0, C.byref(a))
    assert same(e, er) and acc == a.value
    assert same(o.coords(), ref.coords())
    bl, asz, st = ref.intra_state(topo.n_bond, topo.n_angle)
    s = o.state()
    assert same(bl, s["bond_len"]) and same(asz, s["angle_size"])
    assert [s["max_bond_delta"], s["max_angle_delta"], s["step_num"]] == list(st[:3])


@live
@pytest.mark.parametrize("name", ["meoh500", "indole267"])
def test_reference_flexible_examples_live(tmp_path, ref, name):
    """The reference's own flexible examples (methanol: variable bonds 2-6,
    angles 3-6; indole: variable ranges too), where its sources are present:
    the package loader's bond / angle / exclusion rows equal the reference
    loader's (for the implied-angle setting its flag took), and the oracle's
    loop with the intramolecular term and move on the reference's rows equals
    the reference's own code run with ENABLE_INTRA's composition, 300 steps,
    bit for bit."""
    import shutil
    from mcgpu_gb300.workloads import BoxData, Topology
    from oracle.pyoracle import REFERENCE_SRC
    res = REFERENCE_SRC / "resources"
    if not res.is_dir():
        pytest.skip("reference resources not present")
    shutil.copytree(res, tmp_path / "resources")
    shutil.copy(res / "exampleFiles" / (name + ".config"), tmp_path / (name + ".config"))
    rows = ref.load_files(str(tmp_path / (name + ".config")))
    ref.activate_loaded()
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        cands = [F.load(name + ".config", implied_angles=v).topology for v in (False, True)]
    finally:
        os.chdir(cwd)
    r = ref.topology(cands[0].type_natom)
    keys = [k for k in TOPO_KEYS if k != "type_natom"]
    match = [t for t in cands if all(np.array_equal(getattr(t, k), r[k]) for k in keys)]
    assert match, name
    topo = match[0]
    assert topo.flex_bonds and topo.flex_angles
    p = r["params"]
    assert (topo.max_bond_delta, topo.max_angle_delta) == (p[0], p[1])
    box = BoxData(x=rows["x"], y=rows["y"], z=rows["z"], sigma=rows["sigma"],
                  epsilon=rows["epsilon"], charge=rows["charge"], mol_start=rows["mol_start"],
                  mol_len=rows["mol_len"], mol_pidx_start=rows["mol_pidx_start"],
                  mol_pidx_count=rows["mol_pidx_count"], pidx=rows["pidx"], size=rows["size"],
                  cutoff=rows["params"][0], temperature=rows["params"][1],
                  max_translate=rows["params"][3], max_rotate=rows["params"][4]).normalise()
    o = OracleFlex(box, topo)
    e0 = o.system_energy()
    same = lambda a, b: np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)
    assert same(e0, ref.L.ref_system_energy_intra())
    LibcRand(12345)
    e, acc = o.run_plain(300, e0)
    ref.L.ref_seed(12345)
    a = C.c_int()
    er = ref.L.ref_run_plain_intra(300, e0, C.byref(a))
    assert same(e, er) and acc == a.value
    assert same(o.coords(), ref.coords())
    bl, asz, st = ref.intra_state(topo.n_bond, topo.n_angle)
    s = o.state()
    assert same(bl, s["bond_len"]) and same(asz, s["angle_size"])
    print(f"{name}: {box.n_mol} molecules, {topo.n_bond} bonds, {topo.n_angle} angles, "
          f"accepted {acc}/300, E {e0:.4f} -> {e:.4f}")
