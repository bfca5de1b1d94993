"""GPU parity of isobaric (NPT) batches: ln V volume moves every `interval`
steps with full FP64 system energies at both volumes, replayed by the
oracle's mirror of the same chain state (orc_fchain_volume).

Bit-exact: the volume draws, the decisions, the scaled box edges and the
final coordinates.  FP64 energies of the volume moves: summation order only
(REL64).  Running energies: the FP32-pair tolerance since the last volume
move restarted them from an FP64 total."""
import numpy as np
import pytest

from helpers import load_golden
from mcgpu_gb300 import PREC_FP64, PREC_MIXED, ROT_AXIS, ChainBatch, Context
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleChain

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def npt_boxes():
    boxes, seeds = W.water_chains(5, n_min=64, n_max=300, seed=31)
    boxes.append(load_golden("bicyclic100")[0])
    return boxes, list(seeds) + [99]


def oracle_npt(box, seed, chain, n_steps, interval, pressure, max_dlnv, lrc_v=0.0):
    """The oracle run of one NPT chain: segments of `interval` steps, each
    followed by a volume move at the chain's step count."""
    oc = OracleChain(box, ROT_AXIS)
    e = oc.system_energy()
    steps, vols = [], []
    done = 0
    while done < n_steps:
        k = min(interval - done % interval, n_steps - done)
        e, _, tr = oc.run(seed, chain, k, e, step0=done)
        steps += tr
        done += k
        if done % interval == 0:
            r = oc.volume_move(seed, chain, done, pressure, max_dlnv, e, lrc_v)
            e = r["energy"]
            vols.append(r)
    return oc, e, steps, vols


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_npt_batch_replay(ctx, prec):
    """FP64 volume energies: equal to the oracle's up to summation order.
    Mixed (FP32 pairs, FP64 re-take near the threshold): the decisions and
    the boxes are still the oracle's exactly, the energies within the
    FP32-pair rule."""
    boxes, seeds = npt_boxes()
    pressures = [1.0, 1.0, 2000.0, 1.0, 0.0, 1.0]
    interval, steps, dl = 25, 200, 0.02
    bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    bt.set_tile(128, 1, 16)
    bt.set_npt(interval, pressures, dl, prec)
    tr, vtr = bt.run_traced(steps, volume=True)
    stats = bt.stats()
    n_acc = 0
    for c, b in enumerate(boxes):
        oc, e, otr, ovol = oracle_npt(b, seeds[c], c, steps, interval, pressures[c], dl)
        for s, (t, r) in enumerate(zip(tr[c], otr)):
            assert t.mol == r.mol and t.u == r.u, (c, s)
            assert bool(t.accepted) == bool(r.accepted), (c, s, t.de, r.de)
        assert len(vtr[c]) == len(ovol) == steps // interval
        for k, (t, r) in enumerate(zip(vtr[c], ovol)):
            assert t.step == (k + 1) * interval
            assert t.dlnv == r["dlnv"] and t.u == r["u"], (c, k)
            assert bool(t.evaluated) == (r["status"] != -1), (c, k)
            if t.evaluated:
                # fp64 1: both totals re-taken; 2: e_new re-taken in
                # double-float, e_old the running energy
                tight = 1e-11 * max(1.0, abs(r["e_old"]))
                loose = 2e-6 * max(abs(r["e_old"]), 1e-3 * scale_of(oc.ob, b))
                tol_old = tight if (prec == PREC_FP64 or t.fp64 == 1) else loose
                tol_new = tight if (prec == PREC_FP64 or t.fp64 in (1, 2)) else loose
                assert abs(t.e_old - r["e_old"]) <= tol_old, (c, k, t.e_old, r["e_old"])
                assert abs(t.e_new - r["e_new"]) <= tol_new, (c, k, t.e_new, r["e_new"])
            assert bool(t.accepted) == (r["status"] == 1), (c, k)
            assert t.edge == r["edge"], (c, k, t.edge, r["edge"])
            n_acc += t.accepted
        st = stats[c]
        assert st.vol_tried == steps // interval
        assert st.vol_accepted == sum(1 for r in ovol if r["status"] == 1)
        assert tuple(st.box) == tuple(oc.ob.s.size)
        x, y, z = bt.download(c)
        assert np.array_equal(np.stack([x, y, z], 1), oc.coords()), c
        scale = sum(oc.ob.mol_energy_abs(m, m) for m in range(b.n_mol))
        assert abs(st.energy - e) <= 1e-5 * max(abs(e), 1e-3 * scale) + interval * 1e-9 * scale
    assert 0 < n_acc < len(boxes) * (steps // interval)


def test_npt_lrc_term(ctx):
    """The long-range correction in the volume criterion: decisions, boxes
    and coordinates equal the oracle's with the term, and the term changes
    some decision (an exaggerated E_LRC * V so it matters every move)."""
    boxes, seeds = npt_boxes()
    interval, steps, dl = 25, 200, 0.02
    lrc = []
    for b in boxes:
        V = float(b.size[0] * b.size[1] * b.size[2])
        # E_LRC of one-site LJ water at this density is O(-0.1 N) kcal/mol
        lrc.append(-40.0 * b.n_mol * V)
    bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    bt.set_tile(128, 1, 16)
    bt.set_npt(interval, 1.0, dl, PREC_MIXED)
    bt.set_lrc(lrc)
    _, vtr = bt.run_traced(steps, volume=True)
    stats = bt.stats()
    differs = 0
    for c, b in enumerate(boxes):
        oc, e, _, ovol = oracle_npt(b, seeds[c], c, steps, interval, 1.0, dl, lrc[c])
        _, _, _, plain = oracle_npt(b, seeds[c], c, steps, interval, 1.0, dl, 0.0)
        for k, (t, r) in enumerate(zip(vtr[c], ovol)):
            assert bool(t.accepted) == (r["status"] == 1) and t.edge == r["edge"], (c, k)
        differs += sum(1 for p, q in zip(ovol, plain) if p["status"] != q["status"])
        assert tuple(stats[c].box) == tuple(oc.ob.s.size)
        x, y, z = bt.download(c)
        assert np.array_equal(np.stack([x, y, z], 1), oc.coords()), c
    assert differs > 0


def scale_of(ob, b):
    """Sum of the pair-term magnitudes of a box (the FP32 rounding scale)."""
    return sum(ob.mol_energy_abs(m, m) for m in range(b.n_mol))


def test_npt_graph_matches_traced(ctx):
    """The captured-graph NPT path (one graph per interval) gives the same
    chains as the traced direct launches."""
    boxes, seeds = npt_boxes()
    a = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    b = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    for bt in (a, b):
        bt.set_tile(128, 1, 16)
        bt.set_npt(20, 1.0, 0.02)
    a.run(160)
    b.run_traced(160)
    for sa, sb in zip(a.stats(), b.stats()):
        assert sa.accepted == sb.accepted and sa.vol_accepted == sb.vol_accepted
        assert tuple(sa.box) == tuple(sb.box)
        assert sa.energy == sb.energy


def test_npt_pressure_compresses(ctx):
    """A high pressure shrinks the boxes on average, zero pressure lets them
    grow: <V> responds to P in the right direction."""
    boxes, seeds = W.water_chains(16, n_min=64, n_max=128, seed=77)
    hi = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    lo = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    hi.set_npt(10, 20000.0, 0.03)
    lo.set_npt(10, 0.0, 0.03)
    hi.run(1000)
    lo.run(1000)
    v0 = np.array([b.size[0] ** 3 for b in boxes])
    vh = np.array([s.box[0] ** 3 for s in hi.stats()])
    vl = np.array([s.box[0] ** 3 for s in lo.stats()])
    assert np.mean(vh / v0) < np.mean(vl / v0)
