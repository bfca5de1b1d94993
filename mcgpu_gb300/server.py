"""Serving: continuous batching of simulation jobs on one GPU
(mcgpu_server_* in the C ABI).  Jobs are queued with submit(), admitted
between rounds as slots and HBM budget free up, advanced together by the
persistent chain kernel, and retired with their coordinates and counters;
step() runs one round, drain() runs until every job has finished."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .step import Context
from .workloads import BoxData


@dataclass
class JobOutput:
    """A finished job: the C result record plus its final coordinates."""
    result: _abi.JobResult
    coords: np.ndarray | None = None

    @property
    def latency(self) -> float:
        return self.result.t_done - self.result.t_submit


@dataclass
class _Pending:
    box: BoxData
    desc: _abi.BoxDesc
    xyz: tuple | None
    keep: list = field(default_factory=list)


class JobServer:
    def __init__(self, ctx: Context, hbm_budget_bytes: int, max_slots: int = 256,
                 round_steps: int = 100, max_mol_atoms: int = 16, rotation: int = _abi.ROT_AXIS,
                 max_atoms: int = 0, max_molecules: int = 0, tile=(256, 1, 0)):
        self.ctx = ctx
        cfg = _abi.ServerConfig()
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_atoms = int(max_atoms)
        cfg.max_molecules = int(max_molecules)
        cfg.max_slots = int(max_slots)
        cfg.round_steps = int(round_steps)
        cfg.max_mol_atoms = int(max_mol_atoms)
        cfg.rotation = int(rotation)
        cfg.threads, cfg.chains_per_cta, cfg.lanes_per_molecule = (int(v) for v in tile)
        self._h = C.c_void_p()
        _abi.check(_abi.lib().mcgpu_server_create(ctx.handle, C.byref(cfg), C.byref(self._h)),
                   ctx.handle)
        self._pending: dict[int, _Pending] = {}
        ctx.adopt(self)

    def _check(self, st: int) -> None:
        _abi.check(st, self.ctx.handle)

    def close(self) -> None:
        if self._h:
            _abi.lib().mcgpu_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, box: BoxData, seed: int, n_steps: int, chain_id: int = 0,
               npt: bool = False, pressure_atm: float = 1.0, max_dlnv: float = 0.01,
               want_coords: bool = True, vol_precision: int = _abi.PREC_FP64,
               lrc_v: float = 0.0) -> int:
        b = box.copy().normalise()
        d = b.desc()
        jd = _abi.JobDesc()
        jd.box = C.pointer(d)
        jd.seed = int(seed) & (2 ** 64 - 1)
        jd.chain_id = int(chain_id)
        jd.npt = 1 if npt else 0
        jd.vol_precision = int(vol_precision)
        jd.n_steps = int(n_steps)
        jd.pressure_atm = float(pressure_atm)
        jd.max_dlnv = float(max_dlnv)
        jd.lrc_v = float(lrc_v)
        xyz = None
        if want_coords:
            xyz = tuple(np.empty(b.n_atom) for _ in range(3))
            dp = C.POINTER(C.c_double)
            jd.x_out, jd.y_out, jd.z_out = (a.ctypes.data_as(dp) for a in xyz)
        jid = C.c_int64()
        self._check(_abi.lib().mcgpu_server_submit(self._h, C.byref(jd), C.byref(jid)))
        self._pending[jid.value] = _Pending(b, d, xyz)
        return jid.value

    def step(self) -> None:
        self._check(_abi.lib().mcgpu_server_step(self._h))

    def drain(self) -> None:
        self._check(_abi.lib().mcgpu_server_drain(self._h))

    def status(self) -> dict:
        r, q = C.c_int32(), C.c_int32()
        f, b = C.c_int64(), C.c_uint64()
        self._check(_abi.lib().mcgpu_server_status(self._h, C.byref(r), C.byref(q), C.byref(f),
                                                   C.byref(b)))
        return {"running": r.value, "queued": q.value, "finished": f.value,
                "bytes_in_use": b.value}

    def results(self) -> dict[int, JobOutput]:
        out = {}
        arr = (_abi.JobResult * 256)()
        while True:
            n = C.c_int32()
            self._check(_abi.lib().mcgpu_server_results(self._h, arr, 256, C.byref(n)))
            for i in range(n.value):
                r = _abi.JobResult.from_buffer_copy(arr[i])
                p = self._pending.pop(r.job_id, None)
                coords = np.stack(p.xyz, 1) if (p and p.xyz) else None
                out[r.job_id] = JobOutput(r, coords)
            if n.value < 256:
                return out

    def clock(self) -> float:
        return float(_abi.lib().mcgpu_server_clock(self._h))

    def counters(self) -> dict:
        """Device-counted atom pairs of the retired jobs, GPU seconds and
        number of the completed rounds (mcgpu_server_counters)."""
        pairs, rounds, gs = C.c_int64(), C.c_int64(), C.c_double()
        self._check(_abi.lib().mcgpu_server_counters(self._h, C.byref(pairs), C.byref(gs),
                                                     C.byref(rounds)))
        return {"pairs": pairs.value, "gpu_seconds": gs.value, "rounds": rounds.value}
