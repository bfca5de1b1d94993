"""GPU parity of the plain single-chain path (the SimulationStep contract)
against the reference's golden vectors and the oracle, through the C ABI.

FP64 pairs: equal to the reference up to summation order (REL64).
FP32 pairs (mixed): |err| <= 1e-5 * max(|E_ref|, 1e-3 * sum|pair terms|)."""
import numpy as np
import pytest

from helpers import GOLDEN_NAMES, load_golden, tol64, tol_mixed
from mcgpu_gb300 import PREC_FP64, PREC_MIXED, Context, GpuBox, GpuSimulationStep, LibcRand
from mcgpu_gb300 import run_plain
from oracle.pyoracle import OracleBox

pytestmark = pytest.mark.gpu
PRECS = [PREC_FP64, PREC_MIXED]


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def tol(prec, ref, abs_sum):
    return tol64(ref, abs_sum) if prec == PREC_FP64 else tol_mixed(ref, abs_sum)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_system_energy(ctx, name, prec):
    box, z = load_golden(name)
    o = OracleBox(box)
    abs_sum = sum(o.mol_energy_abs(m, m) for m in range(box.n_mol))
    e = GpuBox(ctx, box, prec).system_energy()
    ref = z["sys_energy"][0]
    assert abs(e - ref) <= tol(prec, ref, abs_sum), (e, ref)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_mol_energy(ctx, name, prec):
    box, z = load_golden(name)
    o = OracleBox(box)
    g = GpuBox(ctx, box, prec)
    for c, s, ref in zip(z["me_curr"], z["me_start"], z["me_val"]):
        e = g.mol_energy(int(c), int(s))
        assert abs(e - ref) <= tol(prec, ref, o.mol_energy_abs(int(c), int(s))), (c, s, e, ref)


@pytest.mark.parametrize("fused", [False, True])
@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_move_sequence(ctx, name, prec, fused):
    """The reference's injected move sequence: old/new energies per move,
    rollbacks, and the final coordinates."""
    box, z = load_golden(name)
    o = OracleBox(box)
    g = GpuBox(ctx, box, prec)
    worst = 0.0
    for k in range(len(z["mv_mol"])):
        m, v = int(z["mv_mol"][k]), int(z["mv_vertex"][k])
        mv = (v, *z["mv_d"][k], *z["mv_r"][k])
        ao = o.mol_energy_abs(m, 0)
        if fused:
            eo, _ = None, None
            eo, en = g.move_energies(m, *mv)
        else:
            eo = g.mol_energy(m, 0)
            g.change_molecule(m, *mv)
            en = g.mol_energy(m, 0)
        o.apply_move(m, *mv)
        an = o.mol_energy_abs(m, 0)
        ro, rn = z["mv_eold"][k], z["mv_enew"][k]
        assert abs(eo - ro) <= tol(prec, ro, ao), (k, eo, ro)
        assert abs(en - rn) <= tol(prec, rn, an), (k, en, rn)
        de, rde = en - eo, rn - ro
        assert abs(de - rde) <= tol(prec, rde, ao + an), (k, de, rde)
        worst = max(worst, abs(de - rde) / max(abs(rde), 1e-3 * (ao + an)))
        if not z["mv_accept"][k]:
            g.rollback(m)
            o.rollback(m)
    x, y, zz = g.download()
    got = np.stack([x, y, zz], 1)
    assert np.allclose(got, z["mv_final"], rtol=0, atol=1e-9), np.abs(got - z["mv_final"]).max()
    print(f"{name} prec={prec} fused={fused}: worst dE rel err {worst:.3e}")


@pytest.mark.parametrize("fused", [False, True])
def test_plain_trajectory_fp64_matches_reference(ctx, fused):
    """Simulation::run's loop on the GPU, FP64 pairs, proposals from the C
    library's rand() in the reference's draw order: the same accepted count,
    final energy and coordinates as the reference's own run."""
    box, z = load_golden("water256")
    g = GpuBox(ctx, box, PREC_FP64)
    step = GpuSimulationStep(g, LibcRand(int(z["traj_seed"][0])))
    res = run_plain(step, int(z["traj_steps"][0]), fused=fused)
    assert abs(res.initial_energy - z["traj_e0"][0]) <= tol64(z["traj_e0"][0])
    assert res.accepted == z["traj_accepted"][0]
    assert abs(res.energy - z["traj_energy"][0]) <= 1e-8 * max(1.0, abs(z["traj_energy"][0]))
    x, y, zz = g.download()
    # the rotation's cosines and sines come from the C library on the host,
    # as in the reference: the coordinates are the reference's bit for bit
    assert np.array_equal(np.stack([x, y, zz], 1), z["traj_final"])


@pytest.mark.parametrize("fused", [False, True])
def test_native_plain_loop_matches_reference(ctx, fused):
    """The C++ loop of the library (mcgpu_run_plain: Simulation::run's NVT
    loop over the contract calls, the C library's rand() in the reference's
    draw order): the reference's own run's accepted count, final energy and
    coordinates (bit for bit), and a device pair count of two evaluations per
    step."""
    box, z = load_golden("water256")
    g = GpuBox(ctx, box, PREC_FP64)
    n = int(z["traj_steps"][0])
    st = g.run_plain_native(int(z["traj_seed"][0]), n, fused=fused)
    assert abs(st.energy0 - z["traj_e0"][0]) <= tol64(z["traj_e0"][0])
    assert st.accepted == z["traj_accepted"][0] and st.accepted + st.rejected == n
    assert abs(st.energy - z["traj_energy"][0]) <= 1e-8 * max(1.0, abs(z["traj_energy"][0]))
    x, y, zz = g.download()
    got = np.stack([x, y, zz], 1)
    assert np.array_equal(got, z["traj_final"])
    # 256 waters, rc 9: about a hundred in-range neighbours of 9 pairs, twice a step
    assert 500 * n < st.pairs < 3000 * n
    print(f"native loop fused={fused}: max |coordinate - reference| "
          f"{np.abs(got - z['traj_final']).max():.3e} A, energy difference "
          f"{abs(st.energy - z['traj_energy'][0]):.3e}")
    g.close()


def test_plain_trajectory_mixed_lockstep(ctx):
    """FP32 pairs driven in lockstep with the FP64 oracle on the reference's
    rand() proposals: every dE within tolerance, the oracle's decision applied
    to both; decisions the GPU dE would flip lie inside the tolerance band."""
    box, z = load_golden("water256")
    g = GpuBox(ctx, box, PREC_MIXED)
    o = OracleBox(box)
    rng = LibcRand(1234)
    step = GpuSimulationStep(g, rng)
    kT = box.temperature * 0.00198717
    flips = 0
    errs = []
    for _ in range(1500):
        idx = step.choose_molecule()
        mv = step.draw_move(idx)
        eo, en = g.move_energies(idx, *mv)
        ro = o.mol_energy(idx, 0)
        ao = o.mol_energy_abs(idx, 0)
        o.apply_move(idx, *mv)
        rn = o.mol_energy(idx, 0)
        an = o.mol_energy_abs(idx, 0)
        rde, de = rn - ro, en - eo
        t = tol_mixed(rde, ao + an)
        assert abs(de - rde) <= t
        errs.append(abs(de - rde) / max(abs(rde), 1e-3 * (ao + an)))
        if rde < 0:
            ok = True
        else:
            u = rng.random_real(0.0, 1.0)
            ok = np.exp(-rde / kT) >= u
            ok_gpu = de < 0 or np.exp(-de / kT) >= u
            if ok != ok_gpu:
                flips += 1
                assert abs(-rde / kT - np.log(u)) <= t / kT + 1e-12
        if not ok:
            g.rollback(idx)
            o.rollback(idx)
    x, y, zz = g.download()
    assert np.allclose(np.stack([x, y, zz], 1), o.coords(), rtol=0, atol=1e-9)
    print(f"mixed lockstep: max dE rel err {max(errs):.3e}, median {np.median(errs):.3e}, "
          f"decision flips {flips}")
