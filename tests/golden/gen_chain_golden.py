"""Generates tests/golden/chain_oracle.npz: a regression pin of the oracle's
device-resident chain form (orc_fchain_run: Philox proposals, FP32 moves of
the fixed-point + FP32-offset state, FP64 energies and decisions).

The chain form has no counterpart in the reference (its loop draws from
rand() and moves FP64 rows), so this fixture is not an independent pin: it
freezes the oracle's own output, which the GPU tests match bit for bit
(coordinates) and step by step (decisions).  tests/test_chain_oracle_golden.py
reproduces it on any host; a change of the oracle that moves any bit of it
fails there.

    python tests/golden/gen_chain_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from helpers import load_golden  # noqa: E402
from oracle.pyoracle import OracleChain  # noqa: E402

SEED, CHAIN, STEPS = 0x5EED, 7, 400
BOXES = ("water256", "bicyclic100")


def run(name: str, mode: int):
    box, _ = load_golden(name)
    oc = OracleChain(box, mode)
    e0 = oc.system_energy()
    e, acc, tr = oc.run(SEED, CHAIN, STEPS, e0)
    return dict(e0=e0, e=e, acc=acc, mol=np.array([t.mol for t in tr], np.int32),
                accepted=np.array([t.accepted for t in tr], np.int32),
                e_old=np.array([t.e_old for t in tr]), e_new=np.array([t.e_new for t in tr]),
                coords=oc.coords())


def main() -> None:
    out = {}
    for name in BOXES:
        for mode in (0, 1):
            for k, v in run(name, mode).items():
                out[f"{name}_m{mode}_{k}"] = np.asarray(v)
    np.savez_compressed(Path(__file__).with_name("chain_oracle.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
