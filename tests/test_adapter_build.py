"""The reference-side drop-in (mcgpu_gb300/adapter/GpuBruteForceStep) compiles
against the reference's own headers and links with the reference's objects
and the CUDA library: the build a maintainer would do.  Needs the reference
sources (skipped elsewhere)."""
import subprocess
from pathlib import Path

import pytest

from oracle.pyoracle import REF_SO, REFERENCE_SRC

ROOT = Path(__file__).resolve().parents[1]
pytestmark = pytest.mark.skipif(not (REF_SO.exists() and REFERENCE_SRC.is_dir()),
                                reason="reference sources / objects not available")


def test_adapter_compiles_and_links(tmp_path):
    obj = tmp_path / "GpuBruteForceStep.o"
    subprocess.run(["g++", "-std=c++11", "-O2", "-fPIC", "-w", f"-I{REFERENCE_SRC}",
                    f"-I{REFERENCE_SRC / 'src'}", f"-I{ROOT / 'include'}",
                    "-c", str(ROOT / "mcgpu_gb300/adapter/GpuBruteForceStep.cpp"), "-o", str(obj)],
                   check=True)
    ref_objs = [str(p) for p in (ROOT / "oracle/_ref/obj").rglob("*.o")
                if p.name not in ("Program.o", "ref_harness.o")]
    so = tmp_path / "libdropin.so"
    subprocess.run(["g++", "-shared", "-o", str(so), str(obj)] + ref_objs +
                   [f"-L{ROOT / 'mcgpu_gb300'}", "-lmcgpu_gb300", "-lgomp",
                    f"-Wl,-rpath,{ROOT / 'mcgpu_gb300'}"], check=True)
    syms = subprocess.run(["nm", "-C", "-D", "--defined-only", str(so)], capture_output=True,
                          text=True, check=True).stdout
    assert "vtable for GpuBruteForceStep" in syms
    assert "GpuBruteForceStep::calcMolecularEnergyContribution(int, int)" in syms
