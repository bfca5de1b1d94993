"""Batched device-resident chains: many independent Metropolis chains of
uneven size and temperature advanced by one persistent kernel, replayed as a
captured CUDA graph, with autotuned tiles (mcgpu_batch_* in the C ABI)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .step import Context
from .workloads import BoxData


_F64 = ("x", "y", "z", "sigma", "epsilon", "charge")
_I32 = ("mol_start", "mol_len", "mol_pidx_start", "mol_pidx_count", "pidx")
_ROWS = tuple((k, np.dtype(np.float64)) for k in _F64) + \
    tuple((k, np.dtype(np.int32)) for k in _I32)


def _row_address(a, dt: np.dtype, keep: list) -> int:
    """Address of row a as a C-contiguous array of dt (converted, and kept
    alive in keep, only where it is not one already)."""
    if not (type(a) is np.ndarray and a.dtype == dt and a.flags.c_contiguous):
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
    if a.flags.writeable and a.size:
        return C.addressof(C.c_char.from_buffer(a))   # the cheaper route
    return a.ctypes.data


def _desc_dtype() -> np.dtype:
    """mcgpu_box_desc as a numpy record (pointers as 64-bit addresses)."""
    names, formats, offsets = [], [], []
    for name, ctype in _abi.BoxDesc._fields_:
        names.append(name)
        offsets.append(getattr(_abi.BoxDesc, name).offset)
        if ctype is C.c_int32:
            formats.append(np.int32)
        elif ctype is C.c_double:
            formats.append(np.float64)
        elif ctype is C.c_double * 3:
            formats.append((np.float64, 3))
        else:
            assert C.sizeof(ctype) == 8
            formats.append(np.uint64)
    return np.dtype({"names": names, "formats": formats, "offsets": offsets,
                     "itemsize": C.sizeof(_abi.BoxDesc)})


class ChainBatch:
    def __init__(self, ctx: Context, boxes: list[BoxData], seeds, rotation: int = _abi.ROT_AXIS):
        """Uploads the boxes as one pool (their rows are copied by the
        library).  The descriptors are filled as one numpy record array that
        points at the boxes' own arrays (converted only where they are not
        contiguous FP64 / int32 already)."""
        self.ctx = ctx
        n = len(boxes)
        self.n_chains = n
        self.n_atom = np.array([b.n_atom for b in boxes], np.int64)
        self._atom0 = np.concatenate([[0], np.cumsum(self.n_atom)])
        d = np.zeros(n, _desc_dtype())
        d["n_mol"] = [b.n_mol for b in boxes]
        d["n_atom"] = self.n_atom
        d["n_pidx"] = [b.n_pidx for b in boxes]
        keep: list = []
        addr = np.array([[_row_address(getattr(b, k), dt, keep) for k, dt in _ROWS]
                         for b in boxes], np.uint64).reshape(n, len(_ROWS))
        for f, (k, _) in enumerate(_ROWS):
            d[k] = addr[:, f]
        d["size"] = np.array([np.asarray(b.size, np.float64)[:3] for b in boxes]).reshape(n, 3)
        d["cutoff"] = [float(b.cutoff) for b in boxes]
        d["temperature"] = [float(b.temperature) for b in boxes]
        d["max_translate"] = [float(b.max_translate) for b in boxes]
        d["max_rotate"] = [float(b.max_rotate) for b in boxes]
        self._seeds = (C.c_uint64 * n)(*[int(s) & (2 ** 64 - 1) for s in seeds])
        self._h = C.c_void_p()
        _abi.check(_abi.lib().mcgpu_batch_create(
            ctx.handle, n, C.cast(d.ctypes.data, C.POINTER(_abi.BoxDesc)), self._seeds,
            int(rotation), C.byref(self._h)), ctx.handle)
        del keep        # the pool holds its own copy now
        ctx.adopt(self)

    def _check(self, st: int) -> None:
        _abi.check(st, self.ctx.handle)

    def close(self) -> None:
        if self._h:
            _abi.lib().mcgpu_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, n_steps: int, sync: bool = True) -> None:
        self._check(_abi.lib().mcgpu_batch_run(self._h, int(n_steps), 1 if sync else 0))

    def run_traced(self, n_steps: int, volume: bool = False):
        """Runs n_steps and returns, per chain, the list of step records;
        with volume=True also, per chain, the volume-move records of an NPT
        batch (as a second list)."""
        arr = (_abi.Trace * (n_steps * self.n_chains))()
        vs = n_steps // self.vol_interval + 1 if (volume and self.vol_interval > 0) else 0
        varr = (_abi.VolTrace * max(1, vs * self.n_chains))() if vs else None
        self._check(_abi.lib().mcgpu_batch_run_traced(self._h, int(n_steps), arr, varr))
        flat = list(arr)
        steps = [flat[c * n_steps:(c + 1) * n_steps] for c in range(self.n_chains)]
        if not volume:
            return steps
        vols = []
        for c in range(self.n_chains):
            recs = list(varr[c * vs:(c + 1) * vs]) if vs else []
            vols.append([r for r in recs if r.step > 0])
        return steps, vols

    vol_interval = 0

    def set_verlet(self, skin: float) -> None:
        """Verlet neighbour lists with this skin (Angstrom); <= 0 turns them off."""
        self._check(_abi.lib().mcgpu_batch_set_verlet(self._h, float(skin)))

    def set_npt(self, interval: int, pressure_atm, max_dlnv,
                precision: int = _abi.PREC_FP64) -> None:
        """Isobaric volume moves every `interval` steps (0 = NVT again);
        pressure_atm and max_dlnv are scalars or one value per chain;
        precision of the two system energies: PREC_FP64 or PREC_MIXED."""
        n = self.n_chains
        p = np.broadcast_to(np.asarray(pressure_atm, np.float64), (n,)).copy()
        d = np.broadcast_to(np.asarray(max_dlnv, np.float64), (n,)).copy()
        dp = C.POINTER(C.c_double)
        self._check(_abi.lib().mcgpu_batch_set_npt(self._h, int(interval), p.ctypes.data_as(dp),
                                                   d.ctypes.data_as(dp), int(precision)))
        self.vol_interval = int(interval)

    def set_precision(self, precision: int) -> None:
        """Pair arithmetic of the steps: PREC_MIXED (default) or PREC_FP64
        (every step with FP64 pairs; same decisions, FP64-rounded energies)."""
        self._check(_abi.lib().mcgpu_batch_set_precision(self._h, int(precision)))

    def set_lrc(self, lrc_v) -> None:
        """Long-range LJ correction in the volume-move criterion: E_LRC * V
        per chain (scalar or one per chain, kcal/mol * A^3; 0 = none)."""
        v = np.broadcast_to(np.asarray(lrc_v, np.float64), (self.n_chains,)).copy()
        self._check(_abi.lib().mcgpu_batch_set_lrc(self._h, v.ctypes.data_as(
            C.POINTER(C.c_double))))

    def sync(self) -> None:
        self._check(_abi.lib().mcgpu_batch_sync(self._h))

    def autotune(self, trial_steps: int = 64) -> tuple[int, int, int, int]:
        self._check(_abi.lib().mcgpu_batch_autotune(self._h, int(trial_steps)))
        return self.tile

    def set_tile(self, threads: int, chains_per_cta: int, steps_per_launch: int,
                 lanes_per_molecule: int = 0) -> None:
        self._check(_abi.lib().mcgpu_batch_set_tile(self._h, threads, chains_per_cta,
                                                    steps_per_launch, lanes_per_molecule))

    def set_window(self, k: int) -> None:
        """Windows of k steps (1, 2, 4, 8): one cluster of k CTAs per chain,
        the window's moves evaluated at once and decided in step order
        (mcgpu_batch_set_window); results equal k = 1."""
        self._check(_abi.lib().mcgpu_batch_set_window(self._h, int(k)))

    @property
    def tile(self) -> tuple[int, int, int, int]:
        """(threads per CTA, chains per CTA, steps per launch, lanes cap)."""
        t, c, s, l = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        self._check(_abi.lib().mcgpu_batch_get_tile(self._h, C.byref(t), C.byref(c), C.byref(s),
                                                    C.byref(l)))
        return t.value, c.value, s.value, l.value

    def stats(self) -> list[_abi.ChainStats]:
        arr = (_abi.ChainStats * self.n_chains)()
        self._check(_abi.lib().mcgpu_batch_stats(self._h, arr))
        return list(arr)

    def download(self, chain: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = int(self.n_atom[chain])
        x, y, z = np.empty(n), np.empty(n), np.empty(n)
        dp = C.POINTER(C.c_double)
        self._check(_abi.lib().mcgpu_batch_download(self._h, int(chain), x.ctypes.data_as(dp),
                                                    y.ctypes.data_as(dp), z.ctypes.data_as(dp)))
        return x, y, z

    def download_all(self) -> list:
        """Coordinates of every chain, (x, y, z) per chain, in three copies."""
        tot = int(self._atom0[-1])
        x, y, z = np.empty(tot), np.empty(tot), np.empty(tot)
        dp = C.POINTER(C.c_double)
        self._check(_abi.lib().mcgpu_batch_download_all(self._h, x.ctypes.data_as(dp),
                                                        y.ctypes.data_as(dp),
                                                        z.ctypes.data_as(dp)))
        a = self._atom0
        return [(x[a[c]:a[c + 1]], y[a[c]:a[c + 1]], z[a[c]:a[c + 1]])
                for c in range(self.n_chains)]

    def checkpoint(self) -> bytes:
        """The batch's resumable device state (chain states with their
        Philox counters, coordinates, Verlet lists, NPT phase) as bytes."""
        n = C.c_size_t()
        self._check(_abi.lib().mcgpu_batch_checkpoint(self._h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._check(_abi.lib().mcgpu_batch_checkpoint(self._h, buf, n, C.byref(n)))
        return buf.raw[:n.value]

    def restore(self, blob: bytes) -> None:
        """Continues from a checkpoint of a batch built from the same boxes
        (set the same Verlet skin and NPT interval first)."""
        buf = C.create_string_buffer(bytes(blob), len(blob))
        self._check(_abi.lib().mcgpu_batch_restore(self._h, buf, len(blob)))

    def system_energies(self) -> np.ndarray:
        out = np.empty(self.n_chains)
        self._check(_abi.lib().mcgpu_batch_system_energy(
            self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out
