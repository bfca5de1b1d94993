"""Shared helpers of the tests: golden fixtures and tolerances."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from mcgpu_gb300.workloads import BoxData

GOLDEN = Path(__file__).resolve().parent / "golden"
GOLDEN_NAMES = ["water256", "t3p64", "bicyclic100", "mixed", "water48_halfbox"]

# FP32 pair terms: |err| <= REL * max(|E|, FLOOR * sum_t k_t |t|), the sum over
# the pair terms of each term's magnitude times its condition number with
# respect to the pair distance (k = 12 for 4 eps s^12, 6 for 4 eps s^6, 1 for
# Coulomb; OracleBox.mol_energy_abs): FP32 positions carry a relative error of
# order 1e-7 that each term amplifies by k, so at close LJ contacts the plain
# sum of |terms| under-states the rounding scale twelvefold.
REL = 1e-5
FLOOR = 1e-3
# FP64 pair terms, different summation order only
REL64 = 1e-11


def load_golden(name: str) -> tuple[BoxData, dict]:
    z = dict(np.load(GOLDEN / f"{name}.npz"))
    s = z["box_scalars"]
    box = BoxData(x=z["box_x"], y=z["box_y"], z=z["box_z"], sigma=z["box_sigma"],
                  epsilon=z["box_epsilon"], charge=z["box_charge"], mol_start=z["box_mol_start"],
                  mol_len=z["box_mol_len"], mol_pidx_start=z["box_mol_pidx_start"],
                  mol_pidx_count=z["box_mol_pidx_count"], pidx=z["box_pidx"], size=z["box_size"],
                  cutoff=float(s[0]), temperature=float(s[1]), max_translate=float(s[2]),
                  max_rotate=float(s[3]), name=name).normalise()
    return box, z


def tol_mixed(ref: float, abs_sum: float) -> float:
    return REL * max(abs(ref), FLOOR * abs_sum)


def tol64(ref: float, abs_sum: float = 0.0) -> float:
    return REL64 * max(abs(ref), abs_sum, 1.0)
