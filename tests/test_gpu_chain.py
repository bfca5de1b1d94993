"""GPU parity of the device-resident forms (Philox proposals, on-device
accept) against the oracle replaying the same proposals in FP64."""
import numpy as np
import pytest

from helpers import load_golden, tol_mixed
from mcgpu_gb300 import PREC_MIXED, ROT_AXIS, ROT_EULER, ChainBatch, Context, GpuBox
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleBox, OracleChain, philox, sincos_f32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def replay(box, seed, chain, trace, mode):
    """Runs the chain form on the CPU oracle (same FP32 moves of the same
    state, FP64 energies, the reference's FP64 decision) and checks the
    device trace step by step: same molecule and uniform, same decision,
    energies within the FP32-pair tolerance (FP64 agreement for the steps
    the device re-took in FP64).  Returns the oracle chain, its running
    energy, the worst relative dE error and the count of FP64 re-takes."""
    oc = OracleChain(box, mode)
    e0 = oc.system_energy()
    e, acc, otr = oc.run(seed, chain, len(trace), e0)
    worst = 0.0
    retakes = 0
    for s, (t, r) in enumerate(zip(trace, otr)):
        assert t.mol == r.mol and t.u == r.u, (s, t.mol, r.mol)
        assert bool(t.accepted) == bool(r.accepted), (s, t.de, r.de, r.u)
        if t.fp64:
            retakes += 1
            tl = 1e-9 * max(1.0, abs(r.e_old) + abs(r.e_new))
            assert abs(t.e_old - r.e_old) <= tl and abs(t.e_new - r.e_new) <= tl, s
        else:
            # magnitudes from the oracle state at this step are not kept, so
            # the floor uses the energies' own scale plus the pair sums below
            pass
        worst = max(worst, abs(t.de - r.de))
    return oc, e, otr, worst, retakes


def check_energies(box, trace, otr, mode, seed, chain):
    """Per-step check of the FP32-pair steps: E_old within 1e-5 *
    max(|E|, 1e-3 * sum|pair terms|) and dE within the same rule with the
    term magnitudes of both placements (the new placement's are known to the
    oracle after an accepted step; for a rejected one the old placement's
    stand in for both, and a rejected step from a placement with no
    neighbours in range has its decision checked only).  Re-runs the oracle
    step by step to have each step's magnitudes."""
    oc = OracleChain(box, mode)
    worst = 0.0
    for s, (t, r) in enumerate(zip(trace, otr)):
        mv = oc.draw(seed, chain, s)
        ao = oc.ob.mol_energy_abs(mv.mol, 0)
        assert oc.ob.mol_energy(mv.mol, 0) == r.e_old
        oc.run(seed, chain, 1, 0.0, step0=s)
        an = oc.ob.mol_energy_abs(mv.mol, 0) if r.accepted else ao
        if not t.fp64:
            assert abs(t.e_old - r.e_old) <= tol_mixed(r.e_old, ao), (s, t.e_old, r.e_old)
            if ao + an > 0 or r.de == 0:
                assert abs(t.de - r.de) <= tol_mixed(r.de, ao + an), (s, t.de, r.de)
        worst = max(worst, abs(t.de - r.de) / max(abs(r.de), 1e-3 * (ao + an), 1e-300))
    return worst / 1.0


def test_philox_stream_matches_oracle(ctx):
    """The device draws the oracle's moves: molecule and uniform per step
    identical over a long trace."""
    box = W.water_box(64, seed=3)
    g = GpuBox(ctx, box, PREC_MIXED)
    st, tr = g.chain_run(seed=0xDEADBEEF12345678, n_steps=400, chain_id=5, rotation=ROT_AXIS,
                         trace=True)
    oc = OracleChain(box, ROT_AXIS)
    for s, t in enumerate(tr):
        mv = oc.draw(0xDEADBEEF12345678, 5, s)
        assert t.mol == mv.mol and t.u == mv.u


def test_sincos_f32_accuracy():
    """The FP32 sin/cos of the moves (Cody-Waite reduction + Taylor) is
    within a few ulp of the FP64 values over the angles moves use."""
    import math
    xs = np.linspace(-7.0, 7.0, 4001)
    worst = 0.0
    for x in xs:
        xf = float(np.float32(x))
        s, c = sincos_f32(xf)
        worst = max(worst, abs(s - math.sin(xf)), abs(c - math.cos(xf)))
    assert worst < 4e-7


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
@pytest.mark.parametrize("name", ["water256", "t3p64", "mixed", "water48_halfbox", "bicyclic100"])
def test_chain_run_replay(ctx, name, mode):
    box, z = load_golden(name)
    g = GpuBox(ctx, box, PREC_MIXED)
    seed, steps = 987654321, 600
    st, tr = g.chain_run(seed=seed, n_steps=steps, chain_id=0, rotation=mode, trace=True)
    assert st.steps == steps and st.error == 0
    oc, e, otr, _, retakes = replay(box, seed, 0, tr, mode)
    worst = check_energies(box, tr, otr, mode, seed, 0)
    # the device state is the oracle's state bit for bit
    x, y, zz = g.download()
    assert np.array_equal(np.stack([x, y, zz], 1), oc.coords())
    assert st.accepted == sum(t.accepted for t in tr)
    assert st.ties == retakes
    scale = sum(oc.ob.mol_energy_abs(m, m) for m in range(box.n_mol))
    assert abs(st.energy - e) <= 1e-5 * max(abs(e), 1e-3 * scale) + steps * 1e-9 * scale
    print(f"{name} mode {mode}: accepted {st.accepted}/{steps}, worst dE rel err {worst:.3e}, "
          f"FP64 re-takes {retakes}")


@pytest.mark.parametrize("verlet", [0.0, 1.5])
def test_wide_group_chain_replay(ctx, verlet):
    """A chain of 2600 molecules runs as one group of 10 warps (the 512-thread
    kernel): the oracle's trajectory bit for bit, with and without Verlet lists."""
    box = W.water_box(2600, seed=61)
    g = GpuBox(ctx, box, PREC_MIXED)
    if verlet:
        g.set_verlet(verlet)
    st, tr = g.chain_run(seed=4321, n_steps=400, rotation=ROT_AXIS, trace=True)
    assert st.error == 0
    oc, e, _, _, retakes = replay(box, 4321, 0, tr, ROT_AXIS)
    x, y, z = g.download()
    assert np.array_equal(np.stack([x, y, z], 1), oc.coords())
    assert st.ties == retakes
    g.close()


def test_batch_replay_uneven_chains(ctx):
    """A batch of uneven chains (sizes, temperatures, one 16-atom chain):
    every chain's trace equals the oracle's run of the same chain."""
    boxes, seeds = W.water_chains(6, n_min=40, n_max=300, seed=17)
    boxes.append(load_golden("bicyclic100")[0])
    seeds = list(seeds) + [4242]
    bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    bt.set_tile(128, 2, 8)
    steps = 200
    tr = bt.run_traced(steps)
    stats = bt.stats()
    for c, b in enumerate(boxes):
        oc, e, otr, _, retakes = replay(b, int(seeds[c]), c, tr[c], ROT_AXIS)
        assert stats[c].ties == retakes
        x, y, zz = bt.download(c)
        assert np.array_equal(np.stack([x, y, zz], 1), oc.coords())
        assert stats[c].steps == steps
        scale = sum(oc.ob.mol_energy_abs(m, m) for m in range(b.n_mol))
        assert abs(stats[c].energy - e) <= 1e-5 * max(abs(e), 1e-3 * scale) + steps * 1e-9 * scale


@pytest.mark.parametrize("tile", [(64, 2, 4), (128, 1, 16), (256, 4, 32), (256, 8, 8),
                                  (512, 1, 16), (512, 4, 16)])
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


def big_molecule_box(n_mol=40, n_atom=40, seed=5):
    """Rigid molecules of n_atom sites (more than the 32 bits of a lane
    mask): a seeded blob of radius ~2.5 A, every site with LJ and a charge,
    net neutral."""
    rng = np.random.default_rng(seed)
    xyz = rng.normal(size=(n_atom, 3))
    xyz *= 2.5 / np.linalg.norm(xyz, axis=1).max()
    xyz -= xyz[0]
    sig = rng.uniform(2.0, 3.5, n_atom)
    eps = rng.uniform(0.02, 0.2, n_atom)
    q = rng.uniform(-0.3, 0.3, n_atom)
    q -= q.mean()
    L = 46.0
    return W.build_box((xyz, sig, eps, q, 0), n_mol, L, 12.0, 300.0, 0.2, 10.0, seed, 8.5,
                       name=f"big{n_atom}")


def test_chain_replay_molecules_over_32_atoms(ctx):
    """40-site molecules through the general pair path (teams of lanes per
    neighbour, compensated displacements): the oracle's trajectory bit for
    bit, every step's energies within the FP32-pair rule."""
    box = big_molecule_box()
    g = GpuBox(ctx, box, PREC_MIXED)
    st, tr = g.chain_run(seed=777, n_steps=300, rotation=ROT_AXIS, trace=True)
    assert st.error == 0
    oc, e, otr, _, retakes = replay(box, 777, 0, tr, ROT_AXIS)
    worst = check_energies(box, tr, otr, ROT_AXIS, 777, 0)
    x, y, z = g.download()
    assert np.array_equal(np.stack([x, y, z], 1), oc.coords())
    assert st.ties == retakes
    print(f"40-site molecules: accepted {st.accepted}/300, worst dE error {worst:.3e}")
    g.close()
