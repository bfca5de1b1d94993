"""GPU parity of the device-resident forms (Philox proposals, on-device
accept) against the oracle replaying the same proposals in FP64."""
import numpy as np
import pytest

from helpers import load_golden, tol_mixed
from mcgpu_gb300 import PREC_MIXED, ROT_AXIS, ROT_EULER, ChainBatch, Context, GpuBox
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleBox, philox

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def replay(box, seed, chain, trace, mode, e0):
    """Replays a device trace on the oracle: same Philox proposal, FP64
    energies, the device's decision applied (so both stay on one
    trajectory).  Checks every step's energies against the FP64 oracle
    (FP32-pair tolerance, or FP64 agreement for steps the device re-took in
    FP64) and that the device's decision equals the oracle's except where
    |-dE/kT - ln u| < 1e-6.  Returns the oracle box, the oracle running
    energy, the worst relative dE error and the count of FP64 re-takes."""
    o = OracleBox(box)
    kT = box.temperature * 0.00198717
    e = e0
    worst = 0.0
    retakes = 0
    for s, t in enumerate(trace):
        mv = o.philox_move(seed, chain, s, mode)
        assert t.mol == mv.mol, (s, t.mol, mv.mol)
        ro = o.mol_energy(mv.mol, 0)
        ao = o.mol_energy_abs(mv.mol, 0)
        o.apply_move(mv.mol, mv.vertex, mv.dx, mv.dy, mv.dz, mv.r0, mv.r1, mv.r2, mv.r3, mode)
        rn = o.mol_energy(mv.mol, 0)
        an = o.mol_energy_abs(mv.mol, 0)
        rde = rn - ro
        if t.fp64:
            retakes += 1
            tl = 1e-9 * max(1.0, ao + an)
            assert abs(t.e_old - ro) <= tl and abs(t.e_new - rn) <= tl, (s, t.e_old, ro, t.e_new, rn)
        else:
            assert abs(t.e_old - ro) <= tol_mixed(ro, ao), (s, t.e_old, ro)
            assert abs(t.e_new - rn) <= tol_mixed(rn, an), (s, t.e_new, rn)
        tl = tol_mixed(rde, ao + an)
        assert abs(t.de - rde) <= tl, (s, t.de, rde)
        worst = max(worst, abs(t.de - rde) / max(abs(rde), 1e-3 * (ao + an)))
        assert t.u == mv.u
        ok_ref = rde < 0 or np.exp(-rde / kT) >= mv.u
        if bool(t.accepted) != bool(ok_ref):
            assert rde >= 0 and abs(-rde / kT - np.log(mv.u)) < 1e-6, (s, rde, mv.u)
        if t.accepted:
            e += rde
        else:
            o.rollback(mv.mol)
    return o, e, worst, retakes


def test_philox_stream_matches_oracle(ctx):
    """The device draws the oracle's Philox proposals: molecule index per
    step identical over a long trace."""
    box = W.water_box(64, seed=3)
    g = GpuBox(ctx, box, PREC_MIXED)
    st, tr = g.chain_run(seed=0xDEADBEEF12345678, n_steps=400, chain_id=5, rotation=ROT_AXIS,
                         trace=True)
    o = OracleBox(box)
    for s, t in enumerate(tr):
        mv = o.philox_move(0xDEADBEEF12345678, 5, s, ROT_AXIS)
        assert t.mol == mv.mol and t.u == mv.u


def test_philox_avalanche():
    """Philox4x32-10 as restated: a one-bit counter change flips about half
    of the 128 output bits."""
    base = philox([1, 2, 3, 4], [5, 6])
    flips = []
    for bit in range(32):
        o = philox([1 ^ (1 << bit), 2, 3, 4], [5, 6])
        flips.append(sum(bin(a ^ b).count("1") for a, b in zip(base, o)))
    assert 50 < np.mean(flips) < 78


@pytest.mark.parametrize("mode", [ROT_EULER, ROT_AXIS])
@pytest.mark.parametrize("name", ["water256", "t3p64", "mixed", "water48_halfbox"])
def test_chain_run_replay(ctx, name, mode):
    box, z = load_golden(name)
    g = GpuBox(ctx, box, PREC_MIXED)
    seed, steps = 987654321, 600
    st, tr = g.chain_run(seed=seed, n_steps=steps, chain_id=0, rotation=mode, trace=True)
    assert st.steps == steps and st.error == 0
    e0 = OracleBox(box).system_energy()
    o, e, worst, retakes = replay(box, seed, 0, tr, mode, e0)
    x, y, zz = g.download()
    assert np.allclose(np.stack([x, y, zz], 1), o.coords(), rtol=0, atol=1e-8)
    assert st.accepted == sum(t.accepted for t in tr)
    # running total vs the oracle's running total and vs a fresh recompute
    scale = sum(o.mol_energy_abs(m, m) for m in range(box.n_mol))
    assert abs(st.energy - e) <= 1e-5 * max(abs(e), 1e-3 * scale) + steps * 1e-9 * scale
    assert abs(o.system_energy() - e) <= 1e-9 * max(1.0, scale)
    assert st.ties == retakes
    print(f"{name} mode {mode}: accepted {st.accepted}/{steps}, worst dE rel err {worst:.3e}, "
          f"FP64 re-takes {retakes}")


def test_batch_replay_uneven_chains(ctx):
    """A batch of uneven chains (sizes, temperatures, one 16-atom chain):
    every chain's trace replays on the oracle."""
    boxes, seeds = W.water_chains(6, n_min=40, n_max=300, seed=17)
    boxes.append(load_golden("bicyclic100")[0])
    seeds = list(seeds) + [4242]
    bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    bt.set_tile(128, 2, 8)
    steps = 200
    tr = bt.run_traced(steps)
    stats = bt.stats()
    for c, b in enumerate(boxes):
        o0 = OracleBox(b)
        e0 = o0.system_energy()
        o, e, worst, retakes = replay(b, int(seeds[c]), c, tr[c], ROT_AXIS, e0)
        assert stats[c].ties == retakes
        x, y, zz = bt.download(c)
        assert np.allclose(np.stack([x, y, zz], 1), o.coords(), rtol=0, atol=1e-8)
        assert stats[c].steps == steps
        scale = sum(o.mol_energy_abs(m, m) for m in range(b.n_mol))
        assert abs(stats[c].energy - e) <= 1e-5 * max(abs(e), 1e-3 * scale) + steps * 1e-9 * scale


@pytest.mark.parametrize("tile", [(64, 2, 4), (128, 1, 16), (256, 4, 32), (256, 8, 8)])
def test_batch_tiles_agree(ctx, tile):
    """Every tile shape gives the same trajectories (per-chain Philox streams
    make results independent of packing)."""
    boxes, seeds = W.water_chains(10, n_min=64, n_max=400, seed=5)
    ref = ChainBatch(ctx, boxes, seeds)
    ref.set_tile(128, 1, 16)
    ref.run(96)
    sref = ref.stats()
    bt = ChainBatch(ctx, boxes, seeds)
    bt.set_tile(*tile)
    bt.run(96)
    s = bt.stats()
    for a, b in zip(sref, s):
        assert a.accepted == b.accepted
        assert abs(a.energy - b.energy) <= 1e-9 * max(1.0, abs(a.energy))


def test_batch_graph_replay_and_drift(ctx):
    """Long run through the captured graph; the running totals agree with a
    full FP64 recompute (drift check)."""
    boxes, seeds = W.water_chains(32, seed=8)
    bt = ChainBatch(ctx, boxes, seeds)
    bt.set_tile(128, 1, 16)
    bt.run(16 * 40)
    st = bt.stats()
    full = bt.system_energies()
    for c, s in enumerate(st):
        assert s.steps == 640 and s.error == 0
        o = OracleBox(boxes[c])
        scale = sum(o.mol_energy_abs(m, m) for m in range(boxes[c].n_mol))
        assert abs(s.energy - full[c]) <= 1e-5 * max(abs(full[c]), 1e-3 * scale) + 640 * 1e-9 * scale
