"""Host-side pieces of bench.py that need no GPU: the clock summary of the
nvidia-smi samples (median SM clock, throttle reasons) and the DRAM-traffic
lookup by tile."""
import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("bench_host", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_clock_summary():
    b = _bench()
    cs = b.ClockSampler(0)
    cs.lines = [
        "0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = cs.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    cs.lines = []
    assert cs.summary()["samples"] == 0


def test_chain_traffic_lookup():
    """A capture is reported only for its own tile and kernel version."""
    b = _bench()
    for tile, (v, ver) in b.CHAIN_TRAFFIC_BYTES.items():
        got, note = b.chain_traffic(tile)
        assert (got == v) == (ver == b.CHAIN_KERNEL_VERSION), (tile, note)
    got, note = b.chain_traffic((192, 1, 64, 0))
    assert got is None and "no ncu capture" in note
    b.CHAIN_TRAFFIC_BYTES[(96, 1, 64, 0)] = (1.0, "an older kernel")
    got, note = b.chain_traffic((96, 1, 64, 0))
    assert got is None and "predates" in note
