"""mcgpu_system_energy_static, the system energy that allocates nothing,
through the C ABI, against the oracle: the golden system energies that the
compiled reference produced, and the oracle's restatement of
SimulationStep::calcSystemEnergy on the same rows (OracleBox).

The caller owns every device buffer (here torch tensors stand in for an
offload program's own device rows); the entry point gets device pointers and
writes one device double.  Same FP64 pair terms, different summation order:
agreement within REL64.  The file is named to be collected last so that it
also runs after every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

from helpers import load_golden, tol64
from mcgpu_gb300 import Context, _abi
from mcgpu_gb300.workloads import water_box
from oracle.pyoracle import OracleBox

pytestmark = pytest.mark.gpu

MAX_MOL = 32768


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


class DeviceRows:
    """SimBox rows in caller-owned device memory and a descriptor over them."""

    def __init__(self, box):
        import torch
        dev = torch.device("cuda:0")
        f64 = lambda a: torch.tensor(np.ascontiguousarray(a, np.float64), device=dev)
        i32 = lambda a: torch.tensor(np.ascontiguousarray(a, np.int32), device=dev)
        self.t = [f64(box.x), f64(box.y), f64(box.z), f64(box.sigma), f64(box.epsilon),
                  f64(box.charge), i32(box.mol_start), i32(box.mol_len),
                  i32(box.mol_pidx_start), i32(box.mol_pidx_count), i32(box.pidx)]
        self.out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        d = _abi.BoxDesc()
        d.n_mol, d.n_atom, d.n_pidx = box.n_mol, box.n_atom, len(box.pidx)
        names = ["x", "y", "z", "sigma", "epsilon", "charge", "mol_start", "mol_len",
                 "mol_pidx_start", "mol_pidx_count", "pidx"]
        for n, t in zip(names, self.t):
            ptype = _abi._dp if t.dtype == torch.float64 else _abi._ip
            setattr(d, n, C.cast(C.c_void_p(t.data_ptr()), ptype))
        for k in range(3):
            d.size[k] = float(box.size[k])
        d.cutoff = float(box.cutoff)
        self.desc = d

    def energy(self) -> float:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
        st = _abi.lib().mcgpu_system_energy_static(C.byref(self.desc),
                                                   C.c_void_p(self.out.data_ptr()),
                                                   C.c_void_p(stream))
        _abi.check(st)
        torch.cuda.synchronize()
        return float(self.out.item())


def reference_energy(box) -> float:
    """The oracle's FP64 restatement of calcSystemEnergy on the same rows."""
    return OracleBox(box).system_energy()


GOLDEN = ["water256", "t3p64", "bicyclic100", "mixed", "water48_halfbox"]


def test_static_energy_matches_golden_and_oracle(ctx):
    """Every golden box: the compiled reference's system energy (fixture)
    and the oracle's, to summation order."""
    for name in GOLDEN:
        box, z = load_golden(name)
        gold = float(z["sys_energy"][0])
        assert reference_energy(box) == gold, name      # the oracle is pinned to the fixture
        e = DeviceRows(box).energy()
        assert abs(e - gold) <= tol64(gold), (name, e, gold)


def test_static_energy_two_calls_in_a_row(ctx):
    """Two boxes of different sizes back to back, then the first again: the
    scratch left by one call does not leak into the next."""
    boxes = [load_golden("water256")[0], load_golden("t3p64")[0], load_golden("bicyclic100")[0]]
    refs = [reference_energy(b) for b in boxes]
    rows = [DeviceRows(b) for b in boxes]
    for i in (0, 1, 0, 2, 1):
        e = rows[i].energy()
        assert abs(e - refs[i]) <= tol64(refs[i]), (boxes[i].name, e, refs[i])
    e1, e2 = rows[0].energy(), rows[0].energy()
    assert e1 == e2


def test_static_energy_zero_primary_molecule(ctx):
    """A molecule without primary indexes is never in range
    (moleculesInRange, SimulationStep.cpp:317-330) and contributes nothing,
    as in the oracle."""
    box, _ = load_golden("water256")
    box = box.copy()
    box.mol_pidx_count[17] = 0
    box.mol_pidx_count[200] = 0
    ref = reference_energy(box)
    assert ref != reference_energy(load_golden("water256")[0])
    e = DeviceRows(box).energy()
    assert abs(e - ref) <= tol64(ref), (e, ref)


def test_static_energy_out_of_range_rows_give_nan(ctx):
    """Rows that index past the arrays are caught by the kernel's own range
    checks (the bad index is never dereferenced): the result is NaN, and the
    next valid call is exact again."""
    box, z = load_golden("t3p64")
    gold = float(z["sys_energy"][0])
    bad_start = box.copy()
    bad_start.mol_start[5] = box.n_atom            # molecule 5 starts past the atoms
    bad_pidx = box.copy()
    bad_pidx.pidx[3] = box.n_atom + 7              # a primary index past the atoms
    bad_count = box.copy()
    bad_count.mol_pidx_count[box.n_mol - 1] = 2    # runs past the primary table
    for b in (bad_start, bad_pidx, bad_count):
        assert np.isnan(DeviceRows(b).energy())
    e = DeviceRows(box).energy()
    assert abs(e - gold) <= tol64(gold)


def test_static_energy_allocates_nothing_after_setup(ctx):
    import torch
    box = water_box(1000, seed=5)
    ref = reference_energy(box)
    rows = DeviceRows(box)
    assert abs(rows.energy() - ref) <= tol64(ref)      # first call: address lookup
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        assert abs(rows.energy() - ref) <= tol64(ref)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0


def test_static_energy_captures_into_a_graph(ctx):
    """After the first call, a call captures into a CUDA graph (stream
    capture refuses allocations and host synchronisation, so the capture
    itself shows the call does neither) and the graph's replays give the
    oracle's energy without changing the device's free memory."""
    import torch
    box = water_box(1000, seed=5)
    ref = reference_energy(box)
    rows = DeviceRows(box)
    assert abs(rows.energy() - ref) <= tol64(ref)      # first call: address lookup
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        st = _abi.lib().mcgpu_system_energy_static(
            C.byref(rows.desc), C.c_void_p(rows.out.data_ptr()),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        rows.out.fill_(float("nan"))
        graph.replay()
        torch.cuda.synchronize()
        assert abs(float(rows.out.item()) - ref) <= tol64(ref)
    assert torch.cuda.mem_get_info(0)[0] == free0


def test_static_energy_rejects_oversized_box():
    import torch
    d = _abi.BoxDesc()
    d.n_mol, d.n_atom, d.n_pidx = MAX_MOL + 1, 3 * (MAX_MOL + 1), MAX_MOL + 1
    buf_out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    out = C.c_void_p(buf_out.data_ptr())
    st = _abi.lib().mcgpu_system_energy_static(C.byref(d), out, None)
    assert st == 4   # MCGPU_ERR_UNSUPPORTED, before any device access
    buf = C.create_string_buffer(256)
    _abi.lib().mcgpu_last_error(None, buf, 256)
    assert b"32768" in buf.value
    assert _abi.lib().mcgpu_system_energy_static(None, out, None) == 1
