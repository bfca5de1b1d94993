"""GPU parity of the windowed chain kernel: a chain advanced in windows of K
consecutive steps by a thread-block cluster of K CTAs (each window's moves
evaluated at once, one per CTA, then decided in step order; a step whose
molecule an earlier accepted step of the window moved, or came within range
of, is evaluated again on the current state).

Checked against the oracle (the reference's FP64 decisions on the same
draws, Simulation.cpp:219-264, BruteForceStep.cpp:15-79) and against the
one-step kernel on the same draws: the same molecule, uniform and decision
at every step, coordinates bit for bit, the same accepted counts.  Small
boxes make nearly every step of a window depend on the one before (the
re-evaluation path); large ones make that rare (the speculative path)."""
import numpy as np
import pytest

from helpers import load_golden
from mcgpu_gb300 import (PREC_FP64, PREC_MIXED, ROT_AXIS, ROT_EULER, ChainBatch, Context, GpuBox,
                         MCGPUError)
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleChain

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def set_window(obj, k):
    """obj.set_window(k); a 16-CTA cluster (a non-portable size) is skipped
    where the device places none."""
    try:
        obj.set_window(k)
    except MCGPUError as e:
        if k == 16 and e.status == 4:
            pytest.skip(f"no 16-CTA cluster fits: {e}")
        raise


def oracle_check(box, seed, chain, trace, mode, coords, accepted):
    """The oracle's run of the same chain: every step's molecule, uniform and
    decision; FP64 energies of the steps taken with FP64 pairs; the final
    coordinates bit for bit and the accepted count."""
    oc = OracleChain(box, mode)
    e0 = oc.system_energy()
    e, acc, otr = oc.run(seed, chain, len(trace), e0)
    for s, (t, r) in enumerate(zip(trace, otr)):
        assert t.mol == r.mol and t.u == r.u, (s, t.mol, r.mol)
        assert bool(t.accepted) == bool(r.accepted), (s, t.de, r.de, r.u)
        if t.fp64:
            tl = 1e-9 * max(1.0, abs(r.e_old) + abs(r.e_new))
            assert abs(t.e_old - r.e_old) <= tl and abs(t.e_new - r.e_new) <= tl, s
    assert np.array_equal(coords, oc.coords())
    assert accepted == acc
    return e


def same_run(tr_a, tr_b, tol_rel=1e-5):
    """Two traces of one chain: same draws and decisions, energies within the
    FP32 summation-order difference."""
    assert len(tr_a) == len(tr_b)
    for s, (a, b) in enumerate(zip(tr_a, tr_b)):
        assert a.mol == b.mol and a.u == b.u, s
        assert a.accepted == b.accepted, (s, a.de, b.de)
        tl = tol_rel * max(1.0, abs(b.e_old) + abs(b.e_new))
        assert abs(a.e_old - b.e_old) <= tl and abs(a.e_new - b.e_new) <= tl, s


@pytest.mark.parametrize("window", [2, 4, 8, 16])
@pytest.mark.parametrize("name,mode", [("water256", ROT_AXIS), ("water48_halfbox", ROT_EULER),
                                       ("mixed", ROT_AXIS), ("bicyclic100", ROT_AXIS)])
def test_window_small_boxes_replay(ctx, name, mode, window):
    """Golden boxes small enough that most steps of a window see the one
    before (cutoff near half the edge): 600 steps equal to the oracle, most
    of them re-evaluated in their window."""
    box, _ = load_golden(name)
    g = GpuBox(ctx, box, PREC_MIXED)
    set_window(g, window)
    seed, steps = 987654321, 600
    st, tr = g.chain_run(seed=seed, n_steps=steps, chain_id=0, rotation=mode, trace=True)
    assert st.steps == steps and st.error == 0
    x, y, z = g.download()
    oracle_check(box, seed, 0, tr, mode, np.stack([x, y, z], 1), st.accepted)
    assert st.window_redo > 0
    g.close()
    print(f"{name} window {window}: accepted {st.accepted}/{steps}, re-evaluated "
          f"{st.window_redo}, FP64 re-takes {st.ties}")


@pytest.mark.parametrize("window", [2, 4, 8, 16])
@pytest.mark.parametrize("skin", [0.0, 1.5])
def test_window_equals_one_step_kernel(ctx, window, skin):
    """3000 waters (L = 44.8 A, rc 9 A), 1024 steps with and without Verlet
    lists: the windowed run takes the one-step kernel's decisions on the same
    draws and ends on the same coordinates bit for bit; the first 256 steps
    are also replayed by the oracle."""
    box = W.water_box(3000, seed=71)
    runs = {}
    for k in (1, window):
        g = GpuBox(ctx, box, PREC_MIXED)
        if skin:
            g.set_verlet(skin)
        set_window(g, k)
        st, tr = g.chain_run(seed=2468, n_steps=1024, rotation=ROT_AXIS, trace=True)
        assert st.error == 0 and st.steps == 1024
        x, y, z = g.download()
        runs[k] = (st, tr, np.stack([x, y, z], 1))
        g.close()
    (s1, t1, c1), (sk, tk, ck) = runs[1], runs[window]
    same_run(tk, t1)
    assert np.array_equal(ck, c1)
    assert sk.accepted == s1.accepted
    # a list-screened and a fully scanned evaluation of one step round
    # differently, so a step near the threshold may take FP64 in one run only
    assert abs(sk.ties - s1.ties) <= 2
    assert abs(sk.energy - s1.energy) <= 1e-6 * abs(s1.energy)
    assert s1.window_redo == 0
    g = GpuBox(ctx, box, PREC_MIXED)
    if skin:
        g.set_verlet(skin)
    g.set_window(window)
    st, tr = g.chain_run(seed=2468, n_steps=256, rotation=ROT_AXIS, trace=True)
    x, y, z = g.download()
    oracle_check(box, 2468, 0, tr, ROT_AXIS, np.stack([x, y, z], 1), st.accepted)
    g.close()
    print(f"water3000 skin {skin} window {window}: accepted {sk.accepted}/1024, "
          f"re-evaluated {sk.window_redo}")


@pytest.mark.parametrize("window", [8, 16])
def test_window_fp64_pairs_batch(ctx, window):
    """A 2000-water chain with FP64 pair terms at every step (the FP64 arm of
    the precision sweep), windows of 8 and 16 against one step at a time: the
    same decisions and coordinates, FP64 energies equal to 1e-12."""
    box = W.water_box(2000, seed=19)
    runs = {}
    for k in (1, window):
        bt = ChainBatch(ctx, [box], [0xC0FFEE], rotation=ROT_AXIS)
        bt.set_tile(512, 1, 64)
        set_window(bt, k)
        bt.set_verlet(1.5)
        bt.set_precision(PREC_FP64)
        tr = bt.run_traced(512)[0]
        st = bt.stats()[0]
        assert st.error == 0 and st.ties == 512
        runs[k] = (st, tr, np.stack(bt.download(0), 1))
        bt.close()
    (s1, t1, c1), (s8, t8, c8) = runs[1], runs[window]
    same_run(t8, t1, tol_rel=1e-12)
    assert np.array_equal(c8, c1)
    assert s8.accepted == s1.accepted
    assert abs(s8.energy - s1.energy) <= 1e-11 * abs(s1.energy)


def test_window_batch_more_chains_than_clusters(ctx):
    """96 uneven water chains in windows of 8 (more chain tasks than clusters
    of 8 CTAs that fit at once, so clusters take several in turn): every
    chain equals its one-step run, and three of them the oracle's."""
    boxes, seeds = W.water_chains(96, n_min=40, n_max=300, seed=23)
    out = {}
    for k in (1, 8):
        bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
        bt.set_tile(256, 1, 32)
        bt.set_window(k)
        tr = bt.run_traced(256)
        st = bt.stats()
        out[k] = (tr, st, [np.stack(bt.download(c), 1) for c in range(len(boxes))])
        bt.close()
    (t1, s1, c1), (t8, s8, c8) = out[1], out[8]
    for c in range(len(boxes)):
        assert s8[c].error == 0 and s8[c].steps == 256
        same_run(t8[c], t1[c])
        assert np.array_equal(c8[c], c1[c]), c
        assert s8[c].accepted == s1[c].accepted, c
    for c in (0, 47, 95):
        oracle_check(boxes[c], int(seeds[c]), c, t8[c], ROT_AXIS, c8[c], s8[c].accepted)


def test_window_refusals(ctx):
    """Window sizes other than 1, 2, 4, 8; tiles the window cannot use; the
    tile search (it times one-step kernels)."""
    box = W.water_box(300, seed=3)
    g = GpuBox(ctx, box, PREC_MIXED)
    for k in (0, 3, 12, 32, -1):
        with pytest.raises(MCGPUError):
            g.set_window(k)
    g.close()
    bt = ChainBatch(ctx, [box, box], [1, 2], rotation=ROT_AXIS)
    bt.set_tile(256, 2, 32)
    with pytest.raises(MCGPUError):
        bt.set_window(2)                 # two chains per CTA
    bt.set_tile(128, 1, 32)
    with pytest.raises(MCGPUError):
        bt.set_window(8)                 # 4 warps for 8 staged steps
    bt.set_window(4)
    with pytest.raises(MCGPUError):
        bt.set_tile(256, 2, 32, 0)       # the window needs one chain per CTA
    with pytest.raises(MCGPUError):
        bt.autotune(16)
    assert bt.tile == (128, 1, 32, 0)
    bt.set_window(1)
    bt.set_tile(256, 2, 32, 0)
    bt.close()
