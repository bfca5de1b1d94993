"""GPU: the FP64-pair form of the device-resident chains
(mcgpu_batch_set_precision(MCGPU_PREC_FP64)) against the oracle and against
the FP32-pair form.

Every step's energies are the reference's FP64 pair arithmetic
(BruteForceStep.cpp:48-79) on the chain state: equal to the oracle's up to
summation order (1e-9 relative); the decisions, and so the coordinates, are
the oracle's bit for bit, with and without Verlet lists (the FP64 path then
screens the list), and the same as the FP32-pair form's."""
import numpy as np
import pytest

from mcgpu_gb300 import PREC_FP64, PREC_MIXED, ROT_AXIS, ChainBatch, Context
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleChain

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("skin", [0.0, 1.5])
def test_fp64_pair_chains_replay(ctx, skin):
    boxes, seeds = W.water_chains(5, n_min=300, n_max=900, seed=71)
    steps = 300
    runs = {}
    for prec in (PREC_FP64, PREC_MIXED):
        bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
        bt.set_tile(256, 1, 32)
        if skin:
            bt.set_verlet(skin)
        bt.set_precision(prec)
        tr = bt.run_traced(steps)
        runs[prec] = (tr, bt.stats(), bt.download_all())
        bt.close()
    tr64, st64, xyz64 = runs[PREC_FP64]
    tr32, st32, xyz32 = runs[PREC_MIXED]
    for c, b in enumerate(boxes):
        oc = OracleChain(b, ROT_AXIS)
        e0 = oc.system_energy()
        e, acc, otr = oc.run(int(seeds[c]), c, steps, e0)
        for s, (t, r) in enumerate(zip(tr64[c], otr)):
            assert t.fp64 == 1
            assert t.mol == r.mol and t.u == r.u and bool(t.accepted) == bool(r.accepted), (c, s)
            tol = 1e-9 * max(1.0, abs(r.e_old) + abs(r.e_new))
            assert abs(t.e_old - r.e_old) <= tol and abs(t.e_new - r.e_new) <= tol, (c, s)
        x, y, z = xyz64[c]
        assert np.array_equal(np.stack([x, y, z], 1), oc.coords())
        assert all(np.array_equal(a, b2) for a, b2 in zip(xyz64[c], xyz32[c]))
        assert st64[c].accepted == st32[c].accepted == acc
        assert st64[c].ties == steps
        # the running energy: the oracle's, up to the error bound of the
        # FP32-pair total the batch starts from (1e-6 of the sum of |terms|)
        scale = sum(oc.ob.mol_energy_abs(m, m) for m in range(b.n_mol))
        assert abs(st64[c].energy - e) <= 1e-6 * scale + 1e-9 * abs(e), (c, st64[c].energy, e)
        if skin:
            assert st64[c].nl_builds >= 1
