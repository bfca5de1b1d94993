"""An analytic pin of the restated isobaric move, on the CPU oracle.

The reference's own NPT path is not a valid ensemble (Ensemble.cpp:9-23,
SimulationStep.cpp:476-518: a fixed 1.1 scale applied to every move), so the
ln V move is a restatement with no reference output to pin it.  An ideal gas
pins it instead: with every sigma, epsilon and charge zero the energies
vanish, and ln V moves accepted by exp(-beta P dV + (N + 1) dlnV) >= u sample
p(V) ~ V^N exp(-beta P V), whose mean is exactly (N + 1) kT / P and whose
variance is (N + 1) (kT / P)^2.  Block averages of the oracle's volume-move
chain must match both within two standard errors."""
import math

import numpy as np

from mcgpu_gb300 import ROT_AXIS
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import KBOLTZ, OracleChain


def ideal_water_box(n: int, pressure_atm: float, temperature: float, seed: int):
    """n waters with every interaction switched off, in the box of the
    ideal-gas mean volume."""
    kT = temperature * KBOLTZ
    v = (n + 1) * kT / (pressure_atm * OracleChain.ATM_KCAL)
    box = W.water_box(n, L=v ** (1.0 / 3.0), temperature=temperature, seed=seed, dmin=0.0)
    box.sigma[:] = 0.0
    box.epsilon[:] = 0.0
    box.charge[:] = 0.0
    return box, v


def block_stats(x: np.ndarray, n_blocks: int) -> tuple[float, float]:
    """Mean and its standard error from n_blocks contiguous block means."""
    b = x[: len(x) - len(x) % n_blocks].reshape(n_blocks, -1).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / math.sqrt(n_blocks))


def test_oracle_ideal_gas_volume_distribution():
    n, p_atm, T = 16, 1000.0, 298.0
    box, v_exact = ideal_water_box(n, p_atm, T, seed=3)
    oc = OracleChain(box, ROT_AXIS)
    seed, dl, n_moves = 0x1DEA1, 0.1, 60000
    vols = np.empty(n_moves)
    e = 0.0
    for k in range(n_moves):
        r = oc.volume_move(seed, 0, k + 1, p_atm, dl, e)
        assert r["energy"] == 0.0 and r["status"] in (0, 1)
        vols[k] = r["edge"] ** 3
    v = vols[2000:]
    mean, se = block_stats(v, 100)
    var = float(v.var())
    var_exact = (n + 1) * (v_exact / (n + 1)) ** 2
    var_b, var_se = block_stats((v - v.mean()) ** 2, 100)
    print(f"<V> {mean:.2f} +- {se:.2f} (exact {v_exact:.2f}); var {var:.1f} +- {var_se:.1f} "
          f"(exact {var_exact:.1f})")
    assert abs(mean - v_exact) <= 2 * se
    assert abs(var_b - var_exact) <= 2 * var_se
    # (N + 1) is what the move must use: N or N + 2 would shift <V> by 1/(N + 1)
    assert 2 * se < v_exact / (n + 1)
