"""Ensemble averages of the device-resident chains against FP64 CPU chains.

* Ideal gas (every interaction off), NPT: the GPU volume moves, with FP64
  and with mixed volume energies, give <V> = (N + 1) kT / P, the exact mean
  of the isobaric ensemble, within two standard errors.
* 64 waters, NVT: <U>/N of mixed-precision GPU chains (FP32 pairs) against
  FP64 chains over independent streams, within two standard errors, for
  each proposal family: Euler X->Y->Z rotations about a random vertex
  against the reference's own algorithm (the oracle's restatement,
  BruteForceStep.cpp:15-79 and SimulationStep.cpp:520-566, 794-803), and
  random-axis rotations against the oracle's FP64 chain form.  (The two
  families rotate by different amounts per move, so their chains relax at
  different rates; each is compared with its own kind.)
* 64 waters, NPT at 1 atm: <U>/N and <V> of mixed-precision GPU chains (FP32
  volume energies with the threshold re-takes) against the oracle's FP64
  chain form with its restated volume move, independent streams: within two
  standard errors.
Standard errors come from the spread of independent chains' means; energies
on the GPU side are FP64 recomputes (mcgpu_batch_system_energy)."""
import math

import numpy as np
import pytest

from mcgpu_gb300 import PREC_FP64, PREC_MIXED, ROT_AXIS, ROT_EULER, ChainBatch, Context
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import KBOLTZ, OracleBox, OracleChain
from test_ensemble_oracle import ideal_water_box

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def mean_se(chain_means) -> tuple[float, float]:
    a = np.asarray(chain_means, np.float64)
    return float(a.mean()), float(a.std(ddof=1) / math.sqrt(len(a)))


def agree(a, b, label):
    (ma, sa), (mb, sb) = a, b
    z = abs(ma - mb) / math.sqrt(sa * sa + sb * sb)
    print(f"{label}: GPU {ma:.5f} +- {sa:.5f}, FP64 {mb:.5f} +- {sb:.5f}, |z| = {z:.2f}")
    assert z <= 2.0, (label, ma, sa, mb, sb)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_ideal_gas_volume_mean(ctx, prec):
    n, p_atm, T, chains = 16, 1000.0, 298.0, 32
    box, v_exact = ideal_water_box(n, p_atm, T, seed=3)
    seeds = [0xA11CE + 7919 * c for c in range(chains)]
    bt = ChainBatch(ctx, [box] * chains, seeds, rotation=ROT_AXIS)
    bt.set_tile(128, 1, 16)
    bt.set_npt(1, p_atm, 0.1, prec)
    bt.run(1000)                                    # burn-in: 1000 volume moves
    samples = []
    for _ in range(60):
        bt.run(100)
        samples.append([s.box[0] ** 3 for s in bt.stats()])
    v = np.array(samples)                           # (samples, chains)
    assert all(s.error == 0 for s in bt.stats())
    m, se = mean_se(v.mean(axis=0))
    print(f"ideal gas prec {prec}: <V> {m:.2f} +- {se:.2f}, exact {v_exact:.2f}; "
          f"var {v.var():.0f}, exact {(n + 1) * (v_exact / (n + 1)) ** 2:.0f}")
    assert abs(m - v_exact) <= 2 * se
    assert 2 * se < v_exact / (n + 1)
    bt.close()


def water64():
    return W.water_box(64, L=(64 / W.WATER_DENSITY) ** (1 / 3), cutoff=6.0, temperature=298.0,
                       seed=640)


def gpu_nvt_means(ctx, box, rotation, seeds, burn, seg, n_seg):
    """Per-chain <U>/N of GPU chains (FP64 recomputes of the sampled states)."""
    bt = ChainBatch(ctx, [box] * len(seeds), seeds, rotation=rotation)
    bt.set_tile(128, 1, 16)
    bt.run(burn)
    u = []
    for _ in range(n_seg):
        bt.run(seg)
        u.append(bt.system_energies() / box.n_mol)
    assert all(s.error == 0 for s in bt.stats())
    bt.close()
    return np.array(u).mean(axis=0)


NVT_BURN, NVT_SEG, NVT_NSEG = 30000, 500, 80


@pytest.mark.parametrize("rotation", [ROT_EULER, ROT_AXIS], ids=["euler", "axis"])
def test_nvt_energy_mean_vs_fp64(ctx, rotation):
    """Same proposal family on both sides, so the comparison isolates the
    arithmetic: Euler moves against the reference's own algorithm in FP64
    (the oracle's restatement of its loop); random-axis moves against the
    oracle's FP64 chain form."""
    box = water64()
    n = box.n_mol
    seeds = [0xE115 + 104729 * c for c in range(32)]
    gpu = mean_se(gpu_nvt_means(ctx, box, rotation, seeds, NVT_BURN, NVT_SEG, NVT_NSEG))
    cpu_means = []
    for c in range(8):
        seed = 0xC0FFEE + 31337 * c
        vals = []
        if rotation == ROT_EULER:
            ob = OracleBox(box)
            e = ob.system_energy()
            e, _, _ = ob.chain_run(seed, c, NVT_BURN, ROT_EULER, e)
            for k in range(NVT_NSEG):
                e, _, _ = ob.chain_run(seed, c, NVT_SEG, ROT_EULER, e,
                                       step0=NVT_BURN + k * NVT_SEG)
                vals.append(e / n)
            # the running FP64 total agrees with a recompute
            assert abs(e - ob.system_energy()) <= 1e-9 * max(1.0, abs(e))
        else:
            oc = OracleChain(box, ROT_AXIS)
            e = oc.system_energy()
            e, _, _ = oc.run(seed, c, NVT_BURN, e)
            for k in range(NVT_NSEG):
                e, _, _ = oc.run(seed, c, NVT_SEG, e, step0=NVT_BURN + k * NVT_SEG)
                vals.append(e / n)
        cpu_means.append(np.mean(vals))
    agree(gpu, mean_se(cpu_means), f"NVT <U>/N (kcal/mol), rotation {rotation}")


def test_npt_energy_and_volume_means_vs_fp64(ctx):
    box = water64()
    n = box.n_mol
    interval, dl, p_atm = 50, 0.02, 1.0
    burn, seg, n_seg = 20000, 500, 80
    chains = 32
    seeds = [0x5EA + 6007 * c for c in range(chains)]
    bt = ChainBatch(ctx, [box] * chains, seeds, rotation=ROT_AXIS)
    bt.set_tile(128, 1, 16)
    bt.set_npt(interval, p_atm, dl, PREC_MIXED)
    bt.run(burn)
    u, v = [], []
    for _ in range(n_seg):
        bt.run(seg)
        u.append(bt.system_energies() / n)
        v.append([s.box[0] ** 3 for s in bt.stats()])
    st = bt.stats()
    assert all(s.error == 0 for s in st)
    g_u = mean_se(np.array(u).mean(axis=0))
    g_v = mean_se(np.array(v).mean(axis=0))
    bt.close()
    cu, cv = [], []
    for c in range(8):
        oc = OracleChain(box, ROT_AXIS)
        e = oc.system_energy()
        seed = 0xFEED + 7717 * c
        done, us, vs = 0, [], []
        while done < burn + seg * n_seg:
            e, _, _ = oc.run(seed, c, interval, e, step0=done)
            done += interval
            e = oc.volume_move(seed, c, done, p_atm, dl, e)["energy"]
            if done > burn and done % seg == 0:
                us.append(e / n)
                vs.append(oc.ob.s.size[0] ** 3)
        cu.append(np.mean(us))
        cv.append(np.mean(vs))
    agree(g_u, mean_se(cu), "NPT <U>/N (kcal/mol)")
    agree(g_v, mean_se(cv), "NPT <V> (A^3)")
