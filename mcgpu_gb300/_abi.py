"""ctypes binding of the C ABI in ``include/mcgpu_gb300.h``.

The shared library is built in-tree (``mcgpu_gb300/libmcgpu_gb300.so``) by
``mcgpu_gb300/build.py``.  There is no fallback: if the library is missing or
fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmcgpu_gb300.so"

MCGPU_OK = 0
STATUS_NAMES = {
    0: "MCGPU_OK", 1: "MCGPU_ERR_INVALID", 2: "MCGPU_ERR_CUDA", 3: "MCGPU_ERR_NOMEM",
    4: "MCGPU_ERR_UNSUPPORTED", 5: "MCGPU_ERR_DEVICE", 6: "MCGPU_ERR_CAPACITY",
}
PREC_FP64 = 0
PREC_MIXED = 1
ROT_EULER = 0
ROT_AXIS = 1
MAX_MOL_ATOMS = 64
MAX_MOL_PIDX = 8

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class BoxDesc(C.Structure):
    _fields_ = [
        ("n_mol", C.c_int32), ("n_atom", C.c_int32), ("n_pidx", C.c_int32), ("pad0", C.c_int32),
        ("x", _dp), ("y", _dp), ("z", _dp),
        ("sigma", _dp), ("epsilon", _dp), ("charge", _dp),
        ("mol_start", _ip), ("mol_len", _ip),
        ("mol_pidx_start", _ip), ("mol_pidx_count", _ip),
        ("pidx", _ip),
        ("size", C.c_double * 3),
        ("cutoff", C.c_double), ("temperature", C.c_double),
        ("max_translate", C.c_double), ("max_rotate", C.c_double),
    ]


class TopoDesc(C.Structure):
    _fields_ = [
        ("n_bond", C.c_int32), ("n_angle", C.c_int32), ("n_type", C.c_int32),
        ("max_intra_moves", C.c_int32),
        ("bond_a1", _ip), ("bond_a2", _ip), ("bond_var", _ip),
        ("bond_k", _dp), ("bond_eq", _dp), ("bond_len", _dp),
        ("angle_a1", _ip), ("angle_a2", _ip), ("angle_mid", _ip), ("angle_var", _ip),
        ("angle_k", _dp), ("angle_eq", _dp), ("angle_size", _dp),
        ("mol_bond_start", _ip), ("mol_bond_count", _ip),
        ("mol_angle_start", _ip), ("mol_angle_count", _ip), ("mol_type", _ip),
        ("type_natom", _ip), ("pair_code", C.POINTER(C.c_uint8)),
        ("max_bond_delta", C.c_double), ("max_angle_delta", C.c_double),
        ("step_num", C.c_int64),
    ]


class IntraState(C.Structure):
    _fields_ = [("max_bond_delta", C.c_double), ("max_angle_delta", C.c_double),
                ("step_num", C.c_int64), ("bond_moves", C.c_int64),
                ("bond_accepted", C.c_int64), ("angle_moves", C.c_int64),
                ("angle_accepted", C.c_int64)]


class Move(C.Structure):
    _fields_ = [("vertex", C.c_int32), ("pad0", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("rx", C.c_double), ("ry", C.c_double), ("rz", C.c_double)]


class ChainStats(C.Structure):
    _fields_ = [("energy", C.c_double), ("steps", C.c_int64), ("accepted", C.c_int64),
                ("pairs", C.c_int64), ("error", C.c_int32), ("ties", C.c_int32),
                ("box", C.c_double * 3), ("vol_tried", C.c_int32), ("vol_accepted", C.c_int32),
                ("nl_builds", C.c_int32), ("nl_full_scans", C.c_int32),
                ("window_redo", C.c_int32), ("pad0", C.c_int32)]


class VolTrace(C.Structure):
    _fields_ = [("step", C.c_int64), ("accepted", C.c_int32), ("evaluated", C.c_int32),
                ("e_old", C.c_double), ("e_new", C.c_double), ("dlnv", C.c_double),
                ("u", C.c_double), ("edge", C.c_double), ("fp64", C.c_int32),
                ("pad0", C.c_int32)]


class Trace(C.Structure):
    _fields_ = [("mol", C.c_int32), ("accepted", C.c_int32), ("e_old", C.c_double),
                ("e_new", C.c_double), ("de", C.c_double), ("u", C.c_double),
                ("fp64", C.c_int32), ("pad0", C.c_int32)]


class PlainStats(C.Structure):
    _fields_ = [("energy0", C.c_double), ("energy", C.c_double), ("accepted", C.c_int64),
                ("rejected", C.c_int64), ("pairs", C.c_int64)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_atoms", C.c_int64),
                ("max_molecules", C.c_int64), ("max_slots", C.c_int32),
                ("round_steps", C.c_int32), ("max_mol_atoms", C.c_int32),
                ("rotation", C.c_int32), ("threads", C.c_int32), ("chains_per_cta", C.c_int32),
                ("lanes_per_molecule", C.c_int32), ("pad0", C.c_int32)]


class JobDesc(C.Structure):
    _fields_ = [("box", C.POINTER(BoxDesc)), ("seed", C.c_uint64), ("chain_id", C.c_uint32),
                ("npt", C.c_int32), ("vol_precision", C.c_int32), ("pad1", C.c_int32),
                ("n_steps", C.c_int64), ("pressure_atm", C.c_double),
                ("max_dlnv", C.c_double), ("x_out", _dp), ("y_out", _dp), ("z_out", _dp),
                ("lrc_v", C.c_double)]


class JobResult(C.Structure):
    _fields_ = [("job_id", C.c_int64), ("energy", C.c_double), ("steps", C.c_int64),
                ("accepted", C.c_int64), ("vol_tried", C.c_int32), ("vol_accepted", C.c_int32),
                ("box", C.c_double * 3), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("footprint_bytes", C.c_int64), ("error", C.c_int32),
                ("ties", C.c_int32)]


_vp = C.c_void_p
_PROTOS = {
    "mcgpu_version": (C.c_char_p, []),
    "mcgpu_ctx_create": (C.c_int, [C.POINTER(_vp), C.c_int]),
    "mcgpu_ctx_destroy": (C.c_int, [_vp]),
    "mcgpu_ctx_set_stream": (C.c_int, [_vp, _vp]),
    "mcgpu_last_error": (C.c_int, [_vp, C.c_char_p, C.c_size_t]),
    "mcgpu_box_upload": (C.c_int, [_vp, C.POINTER(BoxDesc), C.c_int, C.POINTER(_vp)]),
    "mcgpu_box_destroy": (C.c_int, [_vp]),
    "mcgpu_box_download": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "mcgpu_mol_energy": (C.c_int, [_vp, C.c_int, C.c_int, _dp]),
    "mcgpu_change_molecule": (C.c_int, [_vp, C.c_int, C.POINTER(Move)]),
    "mcgpu_rollback": (C.c_int, [_vp, C.c_int]),
    "mcgpu_system_energy": (C.c_int, [_vp, _dp]),
    "mcgpu_move_energies": (C.c_int, [_vp, C.c_int, C.POINTER(Move), _dp, _dp]),
    "mcgpu_chain_run": (C.c_int, [_vp, C.c_uint64, C.c_uint32, C.c_int, C.c_int,
                                  C.POINTER(ChainStats), C.POINTER(Trace)]),
    "mcgpu_batch_create": (C.c_int, [_vp, C.c_int, C.POINTER(BoxDesc), C.POINTER(C.c_uint64),
                                     C.c_int, C.POINTER(_vp)]),
    "mcgpu_batch_destroy": (C.c_int, [_vp]),
    "mcgpu_batch_run": (C.c_int, [_vp, C.c_int, C.c_int]),
    "mcgpu_batch_autotune": (C.c_int, [_vp, C.c_int]),
    "mcgpu_batch_set_tile": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "mcgpu_batch_set_window": (C.c_int, [_vp, C.c_int]),
    "mcgpu_chain_set_window": (C.c_int, [_vp, C.c_int]),
    "mcgpu_batch_get_tile": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "mcgpu_batch_sync": (C.c_int, [_vp]),
    "mcgpu_batch_run_traced": (C.c_int, [_vp, C.c_int, C.POINTER(Trace), C.POINTER(VolTrace)]),
    "mcgpu_batch_set_npt": (C.c_int, [_vp, C.c_int, _dp, _dp, C.c_int]),
    "mcgpu_batch_set_verlet": (C.c_int, [_vp, C.c_double]),
    "mcgpu_box_set_verlet": (C.c_int, [_vp, C.c_double]),
    "mcgpu_batch_stats": (C.c_int, [_vp, C.POINTER(ChainStats)]),
    "mcgpu_batch_download": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp]),
    "mcgpu_batch_system_energy": (C.c_int, [_vp, _dp]),
    "mcgpu_batch_checkpoint": (C.c_int, [_vp, _vp, C.c_size_t, C.POINTER(C.c_size_t)]),
    "mcgpu_batch_restore": (C.c_int, [_vp, _vp, C.c_size_t]),
    "mcgpu_batch_set_lrc": (C.c_int, [_vp, _dp]),
    "mcgpu_batch_download_all": (C.c_int, [_vp, _dp, _dp, _dp]),
    "mcgpu_build_centres": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_uint64, _dp]),
    "mcgpu_server_create": (C.c_int, [_vp, C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "mcgpu_server_destroy": (C.c_int, [_vp]),
    "mcgpu_server_submit": (C.c_int, [_vp, C.POINTER(JobDesc), C.POINTER(C.c_int64)]),
    "mcgpu_server_step": (C.c_int, [_vp]),
    "mcgpu_server_drain": (C.c_int, [_vp]),
    "mcgpu_server_status": (C.c_int, [_vp, _ip, _ip, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_uint64)]),
    "mcgpu_server_results": (C.c_int, [_vp, C.POINTER(JobResult), C.c_int, _ip]),
    "mcgpu_server_clock": (C.c_double, [_vp]),
    "mcgpu_server_counters": (C.c_int, [_vp, C.POINTER(C.c_int64), _dp, C.POINTER(C.c_int64)]),
    "mcgpu_batch_set_precision": (C.c_int, [_vp, C.c_int]),
    "mcgpu_run_plain": (C.c_int, [_vp, C.c_uint, C.c_int, C.c_int, C.POINTER(PlainStats)]),
    "mcgpu_run_plain_device": (C.c_int, [_vp, C.c_uint, C.c_int, C.POINTER(PlainStats)]),
    "mcgpu_boxes_run_plain_device": (C.c_int, [C.POINTER(_vp), C.c_int, C.POINTER(C.c_uint),
                                               C.c_int, C.POINTER(PlainStats)]),
    "mcgpu_rand_stream": (C.c_int, [C.c_uint, C.c_int, C.POINTER(C.c_int32)]),
    "mcgpu_box_set_topology": (C.c_int, [_vp, C.POINTER(TopoDesc)]),
    "mcgpu_box_set_intra": (C.c_int, [_vp, C.c_int]),
    "mcgpu_intra_energy": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_double)]),
    "mcgpu_stretch_bond": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double]),
    "mcgpu_expand_angle": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double]),
    "mcgpu_save_intra": (C.c_int, [_vp, C.c_int]),
    "mcgpu_intramolecular_move": (C.c_int, [_vp, C.c_int]),
    "mcgpu_intra_set_step": (C.c_int, [_vp, C.c_int64]),
    "mcgpu_intra_get": (C.c_int, [_vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(IntraState)]),
    "mcgpu_system_energy_static": (C.c_int, [C.POINTER(BoxDesc), _vp, _vp]),
}

_lib = None


class MCGPUError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def lib() -> C.CDLL:
    """Loads the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python mcgpu_gb300/build.py` "
                "(there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_PROTOS)


def check(status: int, ctx=None) -> None:
    if status != MCGPU_OK:
        buf = C.create_string_buffer(512)
        lib().mcgpu_last_error(ctx, buf, 512)
        raise MCGPUError(status, buf.value.decode(errors="replace"))
