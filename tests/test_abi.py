"""The C-ABI library loads and exports every entry point its header
declares; calls that need no GPU behave (no compute runs here)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from mcgpu_gb300 import _abi

HEADERS = sorted((Path(__file__).resolve().parents[1] / "include").glob("*.h"))


def declared():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(mcgpu_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared()
    assert "mcgpu_mol_energy" in names and "mcgpu_batch_run" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = _abi.lib()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared()) <= set(_abi.exported_symbols())


def test_version_string():
    assert b"sm_103a" in _abi.lib().mcgpu_version()


def test_errors_are_status_codes_without_gpu():
    lib = _abi.lib()
    h = C.c_void_p()
    st = lib.mcgpu_ctx_create(C.byref(h), 0)
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert st in (2, 4)
    buf = C.create_string_buffer(256)
    assert lib.mcgpu_last_error(None, buf, 256) == 0
    assert buf.value


def test_null_arguments_rejected():
    lib = _abi.lib()
    assert lib.mcgpu_ctx_create(None, 0) == 1
    assert lib.mcgpu_box_upload(None, None, 0, None) == 1
    assert lib.mcgpu_mol_energy(None, 0, 0, None) == 1
    assert lib.mcgpu_batch_run(None, 1, 1) == 1
    assert lib.mcgpu_chain_set_window(None, 8) == 1
    assert lib.mcgpu_batch_set_window(None, 8) == 1


def test_build_centres_min_distance():
    out = np.empty((500, 3))
    rc = _abi.lib().mcgpu_build_centres(500, 25.0, 2.5, 123, out.ctypes.data_as(
        C.POINTER(C.c_double)))
    assert rc == 0
    assert out.min() >= 0 and out.max() < 25.0
    d = out[:, None] - out[None]
    d -= 25.0 * np.rint(d / 25.0)
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, 99)
    assert r.min() >= 2.5


def test_batch_descriptor_rows():
    """The batch descriptor record matches mcgpu_box_desc field for field, and
    the row addresses it takes are the arrays' own (converted copies only
    for rows that are not contiguous FP64 / int32, kept alive by the caller)."""
    from mcgpu_gb300 import batch as B
    dt = B._desc_dtype()
    assert dt.itemsize == C.sizeof(_abi.BoxDesc)
    for name, _ in _abi.BoxDesc._fields_:
        assert dt.fields[name][1] == getattr(_abi.BoxDesc, name).offset
    f64, i32 = np.dtype(np.float64), np.dtype(np.int32)
    a = np.arange(12.0)
    keep = []
    assert B._row_address(a, f64, keep) == a.ctypes.data and keep == []
    ro = np.arange(6.0)
    ro.flags.writeable = False
    assert B._row_address(ro, f64, keep) == ro.ctypes.data and keep == []
    empty = np.zeros(0)
    assert B._row_address(empty, f64, keep) == empty.ctypes.data and keep == []
    strided = np.arange(20.0)[::2]
    addr = B._row_address(strided, f64, keep)
    assert len(keep) == 1 and addr == keep[0].ctypes.data
    assert np.array_equal(keep[0], strided) and keep[0].flags.c_contiguous
    addr = B._row_address([1, 2, 3], i32, keep)
    assert len(keep) == 2 and keep[1].dtype == i32 and addr == keep[1].ctypes.data
    ints64 = np.arange(4, dtype=np.int64)
    B._row_address(ints64, i32, keep)
    assert keep[2].dtype == i32 and np.array_equal(keep[2], ints64)


@pytest.mark.parametrize("seed", [0, 1, 42, 4321, 2147483647, 2147483648, 4294967295])
def test_restated_rand_stream_equals_c_library(seed):
    """The device loop's generator (the C library's rand() restated, seeded
    as srand seeds it) gives the C library's own numbers, here on the host."""
    from mcgpu_gb300.step import LibcRand
    n = 20000
    out = np.empty(n, np.int32)
    assert _abi.lib().mcgpu_rand_stream(seed, n, out.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    r = LibcRand(seed)
    assert all(int(out[k]) == r.rand() for k in range(n))
