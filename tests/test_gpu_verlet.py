"""Verlet neighbour lists of the device-resident chains (cell-list build on
the GPU, skin/2 displacement trigger): the chains screened through the
lists follow the oracle's full-scan trajectories exactly (same molecules,
uniforms and decisions, bit-identical coordinates), also across forced
rebuilds, volume moves and 16-atom molecules."""
import numpy as np
import pytest

from mcgpu_gb300 import PREC_MIXED, ROT_AXIS, ChainBatch, Context, GpuBox
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleChain
from test_gpu_chain import replay

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("skin,max_t", [(1.5, 0.15), (0.4, 0.6)])
def test_verlet_chain_replay(ctx, skin, max_t):
    box = W.water_box(1500, max_translate=max_t, seed=41)
    g = GpuBox(ctx, box, PREC_MIXED)
    g.set_verlet(skin)
    steps = 1500
    st, tr = g.chain_run(seed=2718, n_steps=steps, rotation=ROT_AXIS, trace=True)
    oc, e, _, _, retakes = replay(box, 2718, 0, tr, ROT_AXIS)
    assert st.ties == retakes and st.error == 0
    x, y, z = g.download()
    assert np.array_equal(np.stack([x, y, z], 1), oc.coords())
    assert st.nl_builds >= 1
    if max_t > 0.5:
        assert st.nl_builds >= 2          # displacements beyond skin/2 force rebuilds
    else:
        assert st.nl_full_scans < steps // 2
    g.close()


def test_verlet_bicyclic_chain(ctx):
    box = W.bicyclic_box(800, seed=12, atom_dmin=2.5)
    g = GpuBox(ctx, box, PREC_MIXED)
    g.set_verlet(1.5)
    st, tr = g.chain_run(seed=99, n_steps=400, rotation=ROT_AXIS, trace=True)
    oc, e, _, _, _ = replay(box, 99, 0, tr, ROT_AXIS)
    x, y, z = g.download()
    assert np.array_equal(np.stack([x, y, z], 1), oc.coords())
    assert st.nl_builds >= 1
    g.close()


def test_verlet_batch_equals_full_scan(ctx):
    """A batch with lists and the same batch without: same decisions and
    coordinates; energies equal within the FP32 summation-order rule."""
    boxes, seeds = W.water_chains(8, n_min=300, n_max=1200, seed=13)
    a = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    b = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    for bt in (a, b):
        bt.set_tile(128, 1, 16)
    b.set_verlet(1.0)
    a.run(800)
    b.run(800)
    for c, (sa, sb) in enumerate(zip(a.stats(), b.stats())):
        assert sa.accepted == sb.accepted and sa.steps == sb.steps
        assert sb.nl_builds >= 1
        assert abs(sa.energy - sb.energy) <= 1e-6 * max(1.0, abs(sa.energy))
        xa, ya, za = a.download(c)
        xb, yb, zb = b.download(c)
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb) and np.array_equal(za, zb)


def test_verlet_with_volume_moves(ctx):
    """Accepted volume moves rescale every centre and force a rebuild; the
    NPT chains still replay the oracle exactly."""
    from test_gpu_npt import oracle_npt
    boxes, seeds = W.water_chains(3, n_min=400, n_max=700, seed=19)
    bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    bt.set_tile(128, 1, 16)
    bt.set_npt(20, 1.0, 0.02)
    bt.set_verlet(1.2)
    tr, vtr = bt.run_traced(200, volume=True)
    stats = bt.stats()
    for c, b in enumerate(boxes):
        oc, e, otr, ovol = oracle_npt(b, seeds[c], c, 200, 20, 1.0, 0.02)
        for s, (t, r) in enumerate(zip(tr[c], otr)):
            assert t.mol == r.mol and bool(t.accepted) == bool(r.accepted), (c, s)
        x, y, z = bt.download(c)
        assert np.array_equal(np.stack([x, y, z], 1), oc.coords())
        assert stats[c].nl_builds >= 1 + stats[c].vol_accepted - 1
