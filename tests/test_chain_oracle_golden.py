"""The oracle's device-resident chain form (orc_fchain_run) against its
frozen output (tests/golden/chain_oracle.npz, made by
tests/golden/gen_chain_golden.py): 400 steps of two golden boxes in both
rotation forms, every step's molecule, decision and FP64 energies and the
final coordinates bit for bit.  The GPU chain kernels are checked against
this oracle step by step, so the pin keeps that reference point fixed."""
from pathlib import Path

import numpy as np
import pytest

from helpers import load_golden
from oracle.pyoracle import OracleChain

FIX = np.load(Path(__file__).parent / "golden" / "chain_oracle.npz")
SEED, CHAIN, STEPS = 0x5EED, 7, 400


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", ["water256", "bicyclic100"])
def test_chain_oracle_reproduces_fixture(name, mode):
    k = f"{name}_m{mode}_"
    box, _ = load_golden(name)
    oc = OracleChain(box, mode)
    e0 = oc.system_energy()
    assert e0 == FIX[k + "e0"]
    e, acc, tr = oc.run(SEED, CHAIN, STEPS, e0)
    assert e == FIX[k + "e"] and acc == FIX[k + "acc"]
    assert np.array_equal([t.mol for t in tr], FIX[k + "mol"])
    assert np.array_equal([t.accepted for t in tr], FIX[k + "accepted"])
    assert np.array_equal([t.e_old for t in tr], FIX[k + "e_old"])
    assert np.array_equal([t.e_new for t in tr], FIX[k + "e_new"])
    assert np.array_equal(oc.coords(), FIX[k + "coords"])
