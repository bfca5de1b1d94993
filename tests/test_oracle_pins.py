"""The oracle restatement against the LIVE reference (its own sources
compiled by oracle/Makefile into oracle/_ref/), on fresh random cases.
Skipped where the reference could not be compiled (e.g. a host without its
sources)."""
import numpy as np
import pytest

from oracle.pyoracle import REF_SO, OracleBox, RefHarness
from mcgpu_gb300 import workloads as W

pytestmark = pytest.mark.skipif(not REF_SO.exists(), reason="reference harness not built")


@pytest.fixture(scope="module")
def ref():
    return RefHarness()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_moves_bit_exact(ref, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(20, 120))
    box = W.water_box(n, seed=seed, cutoff=float(rng.uniform(5.0, 9.0)))
    o = OracleBox(box)
    ref.load(box)
    assert o.system_energy() == ref.system_energy()
    for _ in range(60):
        m = int(rng.integers(n))
        v = int(rng.integers(3))
        d = rng.uniform(-0.3, 0.3, 3)
        a = rng.uniform(-40, 40, 3)
        assert o.mol_energy(m, 0) == ref.mol_energy(m, 0)
        o.apply_move(m, v, *d, *a)
        ref.apply_move(m, v, *d, *a)
        assert o.mol_energy(m, 0) == ref.mol_energy(m, 0)
        if rng.random() < 0.5:
            o.rollback(m)
            ref.rollback(m)
    assert np.array_equal(o.coords(), ref.coords())


def test_rand_stream_matches(ref):
    """The host driver's LibcRand is the reference's seed()/rand()."""
    from mcgpu_gb300.step import LibcRand
    ref.seed(77)
    a = [ref.rand() for _ in range(50)]
    r = LibcRand(77)
    assert a == [r.rand() for _ in range(50)]


def test_reference_intermolecular_move_draw_order(ref):
    """SimCalcs::intermolecularMove draws vertex, dx, dy, dz, rx, ry, rz; the
    host step object draws the same values in the same order."""
    from mcgpu_gb300.step import LibcRand
    box = W.water_box(32, seed=5)
    ref.load(box)
    o = OracleBox(box)
    ref.seed(9)
    ref.intermolecular_move(3)
    r = LibcRand(9)
    n = int(box.mol_len[3])
    v = min(int(r.random_real(0, n)), n - 1)
    t, rr = box.max_translate, box.max_rotate
    d = [r.random_real(-t, t) for _ in range(3)]
    a = [r.random_real(-rr, rr) for _ in range(3)]
    o.apply_move(3, v, *d, *a)
    assert np.array_equal(o.coords(), ref.coords())
