"""The windowed chain loop's rule, checked on the CPU with the oracle.

The device's windowed kernel evaluates the K steps of a window at once on
the state at the window's start and, taking them in order, evaluates a step
again only when an earlier accepted step of the window moved its molecule or
moved a molecule in range of it (the reference's test,
SimulationStep.cpp:317-342, at either placement of either molecule).  The
oracle restates that loop (orc_fchain_run_window); with the exact in-range
test as the rule, every step that is not evaluated again sums the same
in-range molecules in the same order as the sequential loop
(Simulation.cpp:219-264, BruteForceStep.cpp:15-46), so the windowed loop is
the sequential one bit for bit: energies, decisions, state.  The device's
rule flags a superset of these steps (the screen's outer guard radius).
Dropping the in-range half of the rule (a mistake planted in the oracle)
breaks the equality on dense boxes."""
import pytest

from helpers import load_golden
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleChain

SEED, CHAIN, STEPS = 2024, 5, 900


def boxes():
    out = [(n, load_golden(n)[0]) for n in ("water256", "water48_halfbox", "mixed",
                                           "bicyclic100")]
    out.append(("water1500", W.water_box(1500, seed=77)))
    return out


BOXES = boxes()


def trace_key(tr):
    return [(t.mol, t.accepted, t.e_old, t.e_new, t.u) for t in tr]


@pytest.mark.parametrize("window", [2, 4, 8, 16])
@pytest.mark.parametrize("name,box", BOXES, ids=[n for n, _ in BOXES])
@pytest.mark.parametrize("mode", [0, 1])
def test_window_loop_equals_sequential_loop(name, box, window, mode):
    seq = OracleChain(box, mode)
    e0 = seq.system_energy()
    e_s, acc_s, tr_s = seq.run(SEED, CHAIN, STEPS, e0)
    win = OracleChain(box, mode)
    e_w, acc_w, tr_w, redo = win.run_window(SEED, CHAIN, STEPS, e0, window)
    assert trace_key(tr_w) == trace_key(tr_s)
    assert e_w == e_s and acc_w == acc_s
    assert (win.coords() == seq.coords()).all()
    assert (win.A == seq.A).all() and (win.q == seq.q).all() and (win.off == seq.off).all()
    if name != "water1500":
        assert redo > 0                  # dense boxes: the rule is exercised
    assert redo <= STEPS


def test_window_rule_is_needed():
    """With only same-molecule steps evaluated again (a planted mistake), the
    dense boxes leave the sequential trajectory."""
    broken = 0
    for name, box in BOXES[:4]:
        seq = OracleChain(box, 1)
        e0 = seq.system_energy()
        _, _, tr_s = seq.run(SEED, CHAIN, STEPS, e0)
        win = OracleChain(box, 1)
        _, _, tr_w, _ = win.run_window(SEED, CHAIN, STEPS, e0, 8, in_range_rule=False)
        broken += trace_key(tr_w) != trace_key(tr_s)
    assert broken == 4


def test_window_of_one_is_the_loop():
    name, box = BOXES[0]
    a, b = OracleChain(box, 1), OracleChain(box, 1)
    e0 = a.system_energy()
    e_s, acc_s, tr_s = a.run(SEED, CHAIN, 300, e0)
    e_w, acc_w, tr_w, redo = b.run_window(SEED, CHAIN, 300, e0, 1)
    assert trace_key(tr_w) == trace_key(tr_s) and e_w == e_s and redo == 0
