"""GPU parity of the flexible-molecule path (the reference's code behind
ENABLE_INTRA: intramolecular energy, bond stretches, angle expansions, the
intramolecular move with its rand() draws and width tuning, rollback of the
bond lengths and angle sizes) against the reference's golden vectors
(tests/golden/intra_flex.npz) and the oracle, through the C ABI.

Coordinates, bond lengths and angle sizes: bit for bit (the stages follow
the reference's FP64 operations with the C library's cosines and sines).
Energies: FP64 sums in another order, |err| <= 1e-11 * max(|E|, sum |terms|)
(mixed boxes: the intermolecular part within the FP32-pair rule).
Decisions and draws: equal."""
import numpy as np
import pytest

from helpers import (REL64, intra_abs, load_intra_golden, random_flex_box, tol64, tol_mixed)
from mcgpu_gb300 import PREC_FP64, PREC_MIXED, Context, GpuBox, GpuSimulationStep, LibcRand
from mcgpu_gb300 import run_plain
from mcgpu_gb300._abi import MCGPUError
from oracle.pyoracle import OracleBox, OracleFlex

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def flex_box(ctx, prec=PREC_FP64, intra=True):
    box, topo, z = load_intra_golden()
    g = GpuBox(ctx, box, prec)
    g.set_topology(topo)
    g.set_intra(intra)
    return g, box, topo, z


def coords(g):
    x, y, zz = g.download()
    return np.stack([x, y, zz], 1)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_intra_energies_golden(ctx, prec):
    g, box, topo, z = flex_box(ctx, prec)
    xyz = coords(g)
    for m in range(box.n_mol):
        e = g.intra_energy(m)
        ref = z["intra_e"][m]
        assert abs(e - ref) <= REL64 * max(abs(ref), intra_abs(box, topo, xyz, m), 1.0), (m, e, ref)
    # the system energy: intermolecular + intramolecular terms
    o = OracleBox(box)
    scale = sum(o.mol_energy_abs(m, m) + intra_abs(box, topo, xyz, m) for m in range(box.n_mol))
    e = g.system_energy()
    ref = z["sys_energy"][0]
    tol = tol64(ref, scale) if prec == PREC_FP64 else tol_mixed(ref, scale)
    assert abs(e - ref) <= tol, (e, ref)
    g.close()


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_injected_moves_golden(ctx, prec):
    """The golden sequence: rigid move, save, stretches and expansions with
    given amounts, molecule energies with the intramolecular term, rollback
    of the rejected moves (coordinates, sizes, lengths)."""
    g, box, topo, z = flex_box(ctx, prec)
    o = OracleFlex(box, topo)
    k_op = 0
    worst = 0.0
    for k in range(len(z["op_mol"])):
        m = int(z["op_mol"][k])
        mv = (int(z["op_vertex"][k]), *z["op_d"][k], *z["op_r"][k])
        eo = g.mol_energy(m, 0)
        so = o.ob.mol_energy_abs(m, 0) + intra_abs(box, topo, o.coords(), m, o.t.bond_len,
                                                   o.t.angle_size)
        g.set_intra(False)          # the rigid move alone; the ops below are injected
        g.change_molecule(m, *mv)
        g.set_intra(True)
        o.ob.apply_move(m, *mv)
        g.save_intra(m)
        o.save(m)
        while k_op < len(z["op_move"]) and z["op_move"][k_op] == k:
            i, a = int(z["op_index"][k_op]), float(z["op_amount"][k_op])
            if z["op_kind"][k_op] == 0:
                g.stretch_bond(m, i, a)
                o.stretch_bond(m, i, a)
            else:
                g.expand_angle(m, i, a)
                o.expand_angle(m, i, a)
            k_op += 1
        en = g.mol_energy(m, 0)
        sn = o.ob.mol_energy_abs(m, 0) + intra_abs(box, topo, o.coords(), m, o.t.bond_len,
                                                   o.t.angle_size)
        for got, ref, sc in ((eo, z["op_eold"][k], so), (en, z["op_enew"][k], sn)):
            t = tol64(ref, sc) if prec == PREC_FP64 else tol_mixed(ref, sc)
            assert abs(got - ref) <= t, (k, got, ref)
            worst = max(worst, abs(got - ref) / t)
        if not z["op_accept"][k]:
            g.rollback(m)
            o.rollback(m)
    assert np.array_equal(coords(g), z["op_coords"])
    st = g.intra_state()
    assert np.array_equal(st["bond_len"], z["op_bond_len"])
    assert np.array_equal(st["angle_size"], z["op_angle_size"])
    print(f"prec {prec}: worst energy error {worst:.3f} of the tolerance")
    g.close()


def check_state(g, z, prefix):
    st = g.intra_state()
    ref = z[f"{prefix}_state"]
    assert np.array_equal(coords(g), z[f"{prefix}_coords"])
    assert np.array_equal(st["bond_len"], z[f"{prefix}_bond_len"])
    assert np.array_equal(st["angle_size"], z[f"{prefix}_angle_size"])
    assert [st["max_bond_delta"], st["max_angle_delta"], st["step_num"], st["bond_moves"],
            st["bond_accepted"], st["angle_moves"], st["angle_accepted"]] == list(ref)


def test_intramolecular_moves_golden(ctx):
    """300 intramolecularMove calls with the C library's rand(), the width
    tuning at steps 1000 and 2000: the reference's final coordinates, rows,
    widths and counters."""
    g, box, topo, z = flex_box(ctx)
    LibcRand(int(z["im_seed"][0]))
    xyz = None
    for k, m in enumerate(z["im_mol"]):
        if z["im_step"][k] >= 0:
            g.set_step(int(z["im_step"][k]))
        g.intramolecular_move(int(m))
        e = g.intra_energy(int(m))
        ref = z["im_energy"][k]
        if k % 25 == 0:
            xyz = coords(g)
            st = g.intra_state()
            sc = intra_abs(box, topo, xyz, int(m), st["bond_len"], st["angle_size"])
            assert abs(e - ref) <= REL64 * max(abs(ref), sc, 1.0), (k, e, ref)
    # step is the last value set: the state's step_num is the reference's
    check_state(g, z, "im")
    g.close()


@pytest.mark.parametrize("native", [False, True])
def test_plain_trajectory_intra_golden(ctx, native):
    """Simulation::run's loop with the intramolecular term and move, 2500
    steps from srand(4321): the reference's accepted count, final energy,
    coordinates, bond lengths, angle sizes, tuned widths and counters (the
    Python loop over the contract calls, and the library's C++ loop)."""
    g, box, topo, z = flex_box(ctx)
    n, seed = int(z["traj_steps"][0]), int(z["traj_seed"][0])
    if native:
        st = g.run_plain_native(seed, n)
        e0, e, acc = st.energy0, st.energy, st.accepted
    else:
        res = run_plain(GpuSimulationStep(g, LibcRand(seed)), n)
        e0, e, acc = res.initial_energy, res.energy, res.accepted
    assert abs(e0 - z["traj_e0"][0]) <= 1e-11 * max(1.0, abs(z["traj_e0"][0]))
    assert acc == z["traj_accepted"][0]
    assert abs(e - z["traj_energy"][0]) <= 1e-8 * max(1.0, abs(z["traj_e0"][0]))
    check_state(g, z, "traj")
    assert abs(g.system_energy() - z["traj_recompute"][0]) <= 1e-9 * max(1.0, abs(e))
    g.close()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_topologies_vs_oracle(ctx, seed):
    """Random molecules with rings (stretches left alone), angles whose
    middle is an end (zero normal: NaN coordinates, as in the reference) and
    middles in other molecules: injected ops, rand()-driven intramolecular
    moves and a short loop equal to the oracle's (NaN for NaN)."""
    box, topo = random_flex_box(seed)
    g = GpuBox(ctx, box, PREC_FP64)
    g.set_topology(topo)
    g.set_intra(True)
    o = OracleFlex(box, topo)
    same = lambda a, b: np.array_equal(a, b, equal_nan=True)
    rng = np.random.default_rng(seed)
    nan_seen = False
    for k in range(120):
        m = int(rng.integers(0, box.n_mol))
        if rng.random() < 0.5:
            i, d = int(rng.integers(0, topo.mol_bond_count[m])), float(rng.uniform(-0.1, 0.1))
            g.stretch_bond(m, i, d)
            o.stretch_bond(m, i, d)
        else:
            i, d = int(rng.integers(0, topo.mol_angle_count[m])), float(rng.uniform(-6, 6))
            g.expand_angle(m, i, d)
            o.expand_angle(m, i, d)
        assert same(coords(g), o.coords()), k
        e, r = g.intra_energy(m), o.intra_energy(m)
        nan_seen |= bool(np.isnan(r))
        assert (np.isnan(e) and np.isnan(r)) or abs(e - r) <= REL64 * max(
            abs(r), intra_abs(box, topo, o.coords(), m, o.t.bond_len, o.t.angle_size), 1.0), k
    assert nan_seen
    st = g.intra_state()
    assert same(st["bond_len"], o.t.bond_len) and same(st["angle_size"], o.t.angle_size)
    g.close()
    # the loop from fresh copies (NaN placements are rejected on both)
    box, topo = random_flex_box(seed)
    g = GpuBox(ctx, box, PREC_FP64)
    g.set_topology(topo)
    g.set_intra(True)
    o = OracleFlex(box, topo)
    LibcRand(seed)
    e, acc = o.run_plain(400, o.system_energy())
    st = g.run_plain_native(seed, 400)
    assert st.accepted == acc
    assert abs(st.energy - e) <= 1e-8 * max(1.0, abs(e))
    assert same(coords(g), o.coords())
    s = g.intra_state()
    assert same(s["bond_len"], o.t.bond_len) and same(s["angle_size"], o.t.angle_size)
    g.close()


def test_intra_off_by_default_and_refusals(ctx):
    """Without set_intra the box is the rigid contract (energies without the
    intramolecular term, change_molecule rigid); with it on, the fused
    rigid-move call and the device-resident chain are refused; a topology
    whose bond leaves its molecule is refused."""
    g, box, topo, z = flex_box(ctx, intra=False)
    o = OracleBox(box)
    assert abs(g.mol_energy(3, 0) - o.mol_energy(3, 0)) <= tol64(o.mol_energy(3, 0),
                                                                  o.mol_energy_abs(3, 0))
    g.set_intra(True)
    with pytest.raises(MCGPUError):
        g.move_energies(3, 0, 0.1, 0.0, 0.0, 1.0, 2.0, 3.0)
    with pytest.raises(MCGPUError):
        g.chain_run(seed=1, n_steps=4)
    bad = topo.copy()
    bad.bond_a2[0] = int(box.mol_start[5])
    with pytest.raises(MCGPUError, match="outside molecule"):
        g.set_topology(bad)
    g.close()


# ---- the loop on the device (mcgpu_run_plain_device) ----------------------------


def test_device_loop_flexible_golden(ctx):
    """The reference's 2500-step flexible trajectory run entirely on the
    device (one CTA, the C library's generator restated there): the same
    accepted count, tuned widths and counters; bond lengths and angle sizes
    bit for bit (their updates are exact functions of the draws); energy
    within the FP64-sum tolerance; coordinates within 1e-9 A (device sin /
    cos in the rotations)."""
    g, box, topo, z = flex_box(ctx)
    n, seed = int(z["traj_steps"][0]), int(z["traj_seed"][0])
    st = g.run_plain_device(seed, n)
    assert st.accepted == z["traj_accepted"][0] and st.accepted + st.rejected == n
    assert abs(st.energy - z["traj_energy"][0]) <= 1e-8 * max(1.0, abs(z["traj_e0"][0]))
    s = g.intra_state()
    ref = z["traj_state"]
    assert [s["max_bond_delta"], s["max_angle_delta"], s["step_num"], s["bond_moves"],
            s["bond_accepted"], s["angle_moves"], s["angle_accepted"]] == list(ref)
    assert np.array_equal(s["bond_len"], z["traj_bond_len"])
    assert np.array_equal(s["angle_size"], z["traj_angle_size"])
    d = np.abs(coords(g) - z["traj_coords"]).max()
    assert d <= 1e-9, d
    print(f"device loop, flexible: max |coordinate - reference| {d:.2e} A")
    g.close()


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_device_loop_rigid_golden(ctx, prec):
    """The reference's 3000-step rigid trajectory of 256 waters on the device:
    the same accepted count and final energy; coordinates within 1e-9 A
    (FP64 pairs).  With FP32 pairs the decisions are taken on FP32-pair
    energies, so only the counts' closeness and a fresh FP64 recompute of
    the running energy are checked."""
    from helpers import load_golden
    box, z = load_golden("water256")
    g = GpuBox(ctx, box, prec)
    n, seed = int(z["traj_steps"][0]), int(z["traj_seed"][0])
    st = g.run_plain_device(seed, n)
    assert st.accepted + st.rejected == n
    if prec == PREC_FP64:
        assert st.accepted == z["traj_accepted"][0]
        assert abs(st.energy - z["traj_energy"][0]) <= 1e-8 * max(1.0, abs(z["traj_energy"][0]))
        d = np.abs(coords(g) - z["traj_final"]).max()
        assert d <= 1e-9, d
        print(f"device loop, rigid FP64: max |coordinate - reference| {d:.2e} A")
    else:
        assert abs(st.accepted - z["traj_accepted"][0]) <= 0.05 * n
        e = g.system_energy()
        assert abs(st.energy - e) <= 1e-5 * max(1.0, abs(e))
    g.close()


def test_device_loop_random_topologies(ctx):
    """Random flexible molecules (rings, degenerate angles giving NaN
    placements, which are rejected): the device loop takes the oracle's
    decisions over 400 steps (accepted count equal, rows bit for bit)."""
    box, topo = random_flex_box(2)
    g = GpuBox(ctx, box, PREC_FP64)
    g.set_topology(topo)
    g.set_intra(True)
    o = OracleFlex(box, topo)
    LibcRand(7)
    e, acc = o.run_plain(400, o.system_energy())
    st = g.run_plain_device(7, 400)
    assert st.accepted == acc
    assert abs(st.energy - e) <= 1e-8 * max(1.0, abs(e))
    s = g.intra_state()
    assert np.array_equal(s["bond_len"], o.t.bond_len, equal_nan=True)
    assert np.array_equal(s["angle_size"], o.t.angle_size, equal_nan=True)
    g.close()


def test_device_loop_many_boxes_equal_alone(ctx):
    """Several boxes in one launch (flexible and rigid, different seeds):
    each ends where it ends when run alone, the flexible golden box where the
    reference ends."""
    from helpers import load_golden
    from mcgpu_gb300 import run_plain_device_many
    def make():
        g1, box, topo, z = flex_box(ctx, PREC_FP64)
        wb, _ = load_golden("water256")
        g2 = GpuBox(ctx, wb, PREC_FP64)
        rb, rt = random_flex_box(3)
        g3 = GpuBox(ctx, rb, PREC_FP64)
        g3.set_topology(rt)
        g3.set_intra(True)
        return [g1, g2, g3], z
    seeds = [4321, 99, 5]
    boxes, z = make()
    many = run_plain_device_many(boxes, seeds, 2500)
    got = [coords(g) for g in boxes]
    for g in boxes:
        g.close()
    assert many[0].accepted == z["traj_accepted"][0]
    alone_boxes, _ = make()
    for k, (g, sd) in enumerate(zip(alone_boxes, seeds)):
        st = g.run_plain_device(sd, 2500)
        assert st.accepted == many[k].accepted and st.energy == many[k].energy, k
        assert np.array_equal(coords(g), got[k], equal_nan=True), k
        g.close()
