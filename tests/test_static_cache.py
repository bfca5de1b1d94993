"""The scratch-address cache of mcgpu_system_energy_static, on the CPU: a
cached device address is reused only in the context it was looked up in, so
a device reset or a new primary context makes the next call look it up
again (tests/static_cache_check.cpp with fake lookups)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_scratch_address_refreshed_after_context_change(tmp_path):
    exe = tmp_path / "static_cache_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "mcgpu_gb300/csrc"),
                    str(ROOT / "tests/static_cache_check.cpp"), "-o", str(exe), "-lpthread"],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
