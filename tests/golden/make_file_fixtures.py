"""Generates the reference outputs under tests/golden/files/ref/ from the
synthetic inputs beside this script (synth.par, *.z, *.config).

It runs the reference itself, compiled from its sources by ``make -C oracle
ref``: the ``metrosim`` program (its outputs: ``.state``, ``.pdb``, the final
energy, long-range correction and move counts it prints) and the white-box
harness (the SimBox rows its loader builds, its LRC, and the full-precision
coordinates of the same trajectory).  Only this container has the reference
sources; the committed outputs are what the tests compare against anywhere.

    python tests/golden/make_file_fixtures.py
"""
from __future__ import annotations

import ctypes as C
import os
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent / "files"
REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from mcgpu_gb300 import files as F  # noqa: E402
from oracle.pyoracle import REF_BIN, RefHarness  # noqa: E402

OUT = HERE / "ref"
INPUTS = ["synth.par", "oplsaa.sb", "wat4.z", "mix.z", "mixv.z", "trip.z", "tri3.z",
          "wat.config", "mix.config", "mixp.config", "mixv.config", "trip.config",
          "tri3.config"]
# The reference's program runs wat.config and its resume; on the two-template
# mixture it did not finish (busy for minutes) after some step counts (60,
# 199, 200) though its own loop code run through the harness completes the
# same trajectory in milliseconds.  The mixtures' outputs therefore come from
# the harness: the reference's loader, loop code and StateScanner.
# mixv.config carries variable-geometry markers (loader only).
ROW_KEYS = ("x", "y", "z", "sigma", "epsilon", "charge", "mol_start", "mol_len", "mol_type",
            "mol_pidx_start", "mol_pidx_count", "pidx", "size", "params")
# (name, input, extra metrosim arguments, steps)
RUNS = [("wat", "wat.config", [], 300),
        ("watres", "wat_300.state", ["--name", "watres"], 100)]
# (name, config, steps) run through the harness
HARNESS_RUNS = [("mix", 200), ("mixp", 200)]


def metrosim(work: Path, args: list[str]) -> dict:
    p = subprocess.run([str(REF_BIN)] + args + ["-s"], cwd=work, capture_output=True, text=True,
                       check=True, timeout=120)
    pat = {"final": r"Final Energy: (\S+)", "lrc": r"Energy Long-range Correction: (\S+)",
           "accepted": r"Accepted Moves: (\d+)", "rejected": r"Rejected Moves: (\d+)"}
    return {k: float(re.search(v, p.stdout).group(1)) for k, v in pat.items()}


def same_state(a: str, b: str, resumed: bool) -> bool:
    """Equal .state texts; after a resume the seed field (last of line 1) is
    whatever the reference's parser found in freed memory (0 or 1 seen)."""
    if not resumed:
        return a == b
    la, lb = a.split("\n", 1), b.split("\n", 1)
    return la[1] == lb[1] and la[0].split()[:-1] == lb[0].split()[:-1]


def harness_run(R: RefHarness, rows, seed: int, steps: int):
    """The reference's loop on the same rows (harness), for the final
    coordinates at full precision."""
    R.load(rows)
    R.L.ref_seed(seed)
    e0 = R.L.ref_system_energy()
    acc = C.c_int()
    e = R.L.ref_run_plain(steps, e0, C.byref(acc))
    return e0, e, acc.value, R.coords()


def main() -> None:
    if not REF_BIN.exists():
        sys.exit("build the reference first: make -C oracle ref")
    OUT.mkdir(exist_ok=True)
    R = RefHarness()
    for cfg in ("wat", "mix", "mixp", "mixv", "trip", "tri3"):
        ref = R.load_files(str(HERE / (cfg + ".config")))
        np.savez_compressed(OUT / (cfg + "_rows.npz"), **{k: ref[k] for k in ROW_KEYS},
                 lrc=np.float64(ref["lrc"]) if cfg == "wat" else np.float64(np.nan),
                 seed=np.int64(ref["seed"]))
    with tempfile.TemporaryDirectory() as td:
        work = Path(td)
        for f in INPUTS:
            shutil.copy(HERE / f, work / f)
        for name, inp, extra, steps in RUNS:
            out = metrosim(work, [inp, "-n", str(steps)] + extra)
            start = 300 if inp.endswith(".state") else 0
            state = "%s_%d.state" % (name, start + steps)
            shutil.copy(work / state, OUT / state)
            shutil.copy(work / (name + ".pdb"), OUT / (name + ".pdb"))
            cwd = os.getcwd()
            os.chdir(work)
            try:
                si = F.load(inp)
            finally:
                os.chdir(cwd)
            e0, e, acc, xyz = harness_run(R, si.rows, si.box.env.random_seed, steps)
            assert acc == int(out["accepted"]), (name, acc, out)
            coords = (xyz[:, 0], xyz[:, 1], xyz[:, 2])
            # the restated writers reproduce the reference's files from the
            # reference's own coordinates
            ours = F.format_state(si.box.env, si.box.molecules, start + steps, coords)
            assert same_state(ours, (OUT / state).read_text(), resumed=start > 0), name
            assert F.format_pdb(si.box.env, si.box.molecules, coords) == \
                (OUT / (name + ".pdb")).read_text(), name
            np.savez_compressed(OUT / (name + "_run.npz"), xyz=xyz, e0=np.float64(e0), e=np.float64(e),
                     accepted=np.int64(acc), steps=np.int64(steps), start=np.int64(start),
                     final=np.float64(out["final"]), lrc_printed=np.float64(out["lrc"]))
            print(name, out, "pair energy %.6f" % e)
            if name == "wat":
                ref = R.load_files(str(OUT / state))
                np.savez_compressed(OUT / "wat300_rows.npz", **{k: ref[k] for k in ROW_KEYS},
                                    start_step=np.int64(ref["start_step"]))
    for name, steps in HARNESS_RUNS:
        ref = R.load_files(str(HERE / (name + ".config")))
        cwd = os.getcwd()
        os.chdir(HERE)
        try:
            si = F.load(name + ".config")
        finally:
            os.chdir(cwd)
        e0, e, acc, xyz = harness_run(R, si.rows, int(ref["seed"]), steps)
        R.load_files(str(HERE / (name + ".config")))
        state = "%s_%d.state" % (name, steps)
        R.write_loaded_state(str(OUT / state), steps, xyz)
        # the harness's z-matrix scanner starts with its uninitialised
        # implied-angle flag in some state: record which one it had
        text = (OUT / state).read_text()
        coords = (xyz[:, 0], xyz[:, 1], xyz[:, 2])
        flag = None
        for implied in (False, True):
            os.chdir(HERE)
            try:
                sj = F.load(name + ".config", implied_angles=implied)
            finally:
                os.chdir(cwd)
            if F.format_state(sj.box.env, sj.box.molecules, steps, coords) == text:
                flag = implied
        assert flag is not None, name
        np.savez_compressed(OUT / (name + "_run.npz"), xyz=xyz, e0=np.float64(e0),
                            e=np.float64(e), accepted=np.int64(acc), steps=np.int64(steps),
                            start=np.int64(0), implied_angles=np.bool_(flag))
        print(name, "accepted", acc, "pair energy %.6f" % e)


if __name__ == "__main__":
    main()
