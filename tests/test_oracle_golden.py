"""The oracle restatement against the reference's own golden vectors
(tests/golden/*.npz, made by tests/golden/gen_golden.py from the compiled
reference).  Bit-exact: same arithmetic, same order."""
import numpy as np
import pytest

from helpers import GOLDEN_NAMES, load_golden
from oracle.pyoracle import OracleBox


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_system_energy(name):
    box, z = load_golden(name)
    assert OracleBox(box).system_energy() == z["sys_energy"][0]


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_mol_energy(name):
    box, z = load_golden(name)
    o = OracleBox(box)
    got = [o.mol_energy(int(c), int(s)) for c, s in zip(z["me_curr"], z["me_start"])]
    assert np.array_equal(np.array(got), z["me_val"])


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_move_sequence(name):
    box, z = load_golden(name)
    o = OracleBox(box)
    for k in range(len(z["mv_mol"])):
        m = int(z["mv_mol"][k])
        assert o.mol_energy(m, 0) == z["mv_eold"][k]
        o.apply_move(m, int(z["mv_vertex"][k]), *z["mv_d"][k], *z["mv_r"][k])
        assert o.mol_energy(m, 0) == z["mv_enew"][k]
        if not z["mv_accept"][k]:
            o.rollback(m)
    assert np.array_equal(o.coords(), z["mv_final"])


def test_dummy_sites_are_skipped():
    """t3p64 carries two sigma = epsilon = -1 sites per water
    (BruteForceStep.cpp:64-65): removing them leaves every energy unchanged."""
    box, z = load_golden("t3p64")
    keep = np.ones(box.n_atom, bool)
    for m in range(box.n_mol):
        keep[box.mol_start[m] + 1: box.mol_start[m] + 3] = False
    from mcgpu_gb300.workloads import BoxData
    nb = BoxData(x=box.x[keep], y=box.y[keep], z=box.z[keep], sigma=box.sigma[keep],
                 epsilon=box.epsilon[keep], charge=box.charge[keep],
                 mol_start=np.arange(box.n_mol) * 3, mol_len=np.full(box.n_mol, 3),
                 mol_pidx_start=np.arange(box.n_mol), mol_pidx_count=np.ones(box.n_mol),
                 pidx=np.arange(box.n_mol) * 3, size=box.size, cutoff=box.cutoff,
                 temperature=box.temperature, max_translate=box.max_translate,
                 max_rotate=box.max_rotate).normalise()
    assert abs(OracleBox(nb).system_energy() - z["sys_energy"][0]) < 1e-9 * abs(z["sys_energy"][0])


def test_plain_trajectory_libc_rand():
    """Simulation::run's loop with the reference's rand() stream, restated:
    the oracle with the same srand seed ends where the reference ended."""
    from mcgpu_gb300.step import LibcRand
    box, z = load_golden("water256")
    o = OracleBox(box)
    rng = LibcRand(int(z["traj_seed"][0]))
    e = o.system_energy()
    assert e == z["traj_e0"][0]
    acc = 0
    kT = box.temperature * 0.00198717
    for _ in range(int(z["traj_steps"][0])):
        idx = min(int(rng.random_real(0, box.n_mol)), box.n_mol - 1)
        old = o.mol_energy(idx, 0)
        n = int(box.mol_len[idx])
        v = min(int(rng.random_real(0, n)), n - 1)
        t, r = box.max_translate, box.max_rotate
        d = [rng.random_real(-t, t) for _ in range(3)]
        a = [rng.random_real(-r, r) for _ in range(3)]
        o.apply_move(idx, v, *d, *a)
        new = o.mol_energy(idx, 0)
        de = new - old
        ok = de < 0 or np.exp(-de / kT) >= rng.random_real(0.0, 1.0)
        if ok:
            acc += 1
            e += de
        else:
            o.rollback(idx)
    assert acc == z["traj_accepted"][0]
    assert e == z["traj_energy"][0]
    assert np.array_equal(o.coords(), z["traj_final"])
