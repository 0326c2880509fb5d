"""ctypes binding of ``libmcgb.so`` (the C ABI declared in include/mcgb.h).

The library is the only compute path: if it cannot be loaded, importing a
model raises.  Every call passes torch's current CUDA stream, so library
kernels order with torch copies issued by :mod:`mcgb.device`.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import build as _build

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_F = ctypes.c_float
_D = ctypes.c_double

# name -> argument types (all return int status)
SIGNATURES = {
    "mcgb_rng_init": [_P, _I64, _U64, _U64, _P],
    "mcgb_rng_draw": [_P, _I64, _I, _I, _P, _P],
    "mcgb_expf": [_P, _P, _I64, _P],
    "mcgb_ising_update_color": [_P, _P, _P, _I, _I, _I, _F, _P],
    "mcgb_ising_sweep": [_P, _P, _P, _I, _I, _F, _I, _P],
    "mcgb_ising_energy": [_P, _I, _I, _F, _P, _P],
    "mcgb_ising_measure": [_P, _I, _I, _F, _P, _P, _P, _P],
    "mcgb_xy_update_color": [_P, _P, _P, _I, _I, _I, _F, _F, _P],
    "mcgb_xy_update_color_gauss": [_P, _P, _P, _P, _I, _I, _I, _F, _P],
    "mcgb_xy_sweep": [_P, _P, _P, _P, _I, _I, _F, _F, _I, _P],
    "mcgb_xy64_update_color": [_P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _P],
    "mcgb_xy64_energy": [_P, _I, _I, _I, _D, _P, _P],
    "mcgb_xy64_measure": [_P, _I, _I, _I, _D, _P, _P, _P],
    "mcgb_xy_energy": [_P, _I, _I, _F, _P, _P],
    "mcgb_xy_measure": [_P, _I, _I, _F, _P, _P, _P, _P],
    "mcgb_kawamura_update_color": [_P, _P, _P, _I, _I, _I, _F, _F, _P],
    "mcgb_kawamura_sweep": [_P, _P, _P, _I, _I, _F, _F, _I, _P],
    "mcgb_kawamura_energy": [_P, _I, _I, _F, _P, _P],
    "mcgb_kawamura_measure": [_P, _I, _I, _F, _P, _P, _P, _P],
    "mcgb_kawamura_local_energies": [_P, _I, _I, _P, _P, _I, _F, _P, _P],
    "mcgb_he3_update_color": [_P, _P, _P, _I, _I, _I, _P, _F, _F, _F, _P],
    "mcgb_he3_gaussian_update_color": [_P, _P, _P, _I, _I, _I, _P, _F, _F, _F, _F, _P, _P],
    "mcgb_he3_energy": [_P, _I, _I, _P, _F, _F, _P, _P],
    "mcgb_he3_measure": [_P, _I, _I, _P, _F, _F, _P, _P, _P, _P],
    "mcgb_he3_local_differences": [_P, _I, _I, _P, _P, _I, _P, _F, _F, _P, _P],
    "mcgb_pt_exchange": [_P, _P, _P, _P, _P, _P, _P, _I, _I, _I64, _P],
    "mcgb_pt_record_walkers": [_P, _P, _P, _I, _P],
    "mcgb_pt_exchange_clocked": [_P, _P, _P, _P, _P, _P, _P, _I, _P, _I, _P],
    "mcgb_pt_record_walkers_ring": [_P, _P, _P, _P, _I, _I64, _P],
    "mcgb_ring_push": [_P, _P, _P, _I64, _I64, _P],
    "mcgb_batch_channels": [_I],
    "mcgb_batch_smem_bytes": [_I, _I, _I],
    "mcgb_batch_max_clusters": [_I, _I, _I, _I64, _P],
    "mcgb_batch_window_run": [_I, _P, _P],
    "mcgb_batch_permute": [_P, _P, _I64, _P, _P, _I, _I, _I, _P],
    "mcgb_batch_refresh_aux": [_I, _P, _P],
    "mcgb_batch_recompute_energy": [_I, _P, _P, _P],
    "mcgb_batch_exchange": [_P, _P, _P],
    "mcgb_batch_window_exchange": [_I, _P, _P, _P, _P],
    "mcgb_batch_run_resident": [_I, _P, _P, _P, _I, _P],
    "mcgb_batch_set_wait_limit": [ctypes.c_int64],
    "mcgb_batch_clock_tick": [_P, _I, _I, _P],
    "mcgb_batch_tune_sigma": [_P, _P, _P, _P, _P, _I, _I, _F, _F, _F, _F, _P],
    "mcgb_batch_window_exchange_noalloc": [_I, _P, _P, _P],
    # handle API
    "mc_create": [_I, _P, _P, _I, _P, _U64, _P, _P],
    "mc_sweep": [_P, _I],
    "mc_update_color": [_P, _I],
    "mc_energy": [_P, _P],
    "mc_measure": [_P, _P, _P, _P],
    "mc_exchange": [_P, _I, _I64],
    "mc_rng_init": [_P, _U64, _U64],
    "mc_get_error": [_P],
    "mc_copy_in": [_P, _I, _P, _I64],
    "mc_copy_out": [_P, _I, _P, _I64],
    "mc_destroy": [_P],
}


class MCParams(ctypes.Structure):
    """ctypes mirror of ``mc_params`` (include/mcgb.h)."""

    _fields_ = [("J", ctypes.c_float), ("delta", ctypes.c_float), ("sigmas", ctypes.c_void_p),
                ("coefficients", ctypes.c_float * 5), ("K", ctypes.c_float), ("g_d", ctypes.c_float),
                ("rho", ctypes.c_float), ("mass", ctypes.c_float)]


# Buffers of mc_copy_in / mc_copy_out.
MC_STATE, MC_RNG, MC_BETAS, MC_ENERGIES, MC_W2T, MC_T2W, MC_SWAP_COUNTS, MC_TRIPS, MC_EXCHANGE_RNG = range(9)

# Entry points whose return value is not an int status.
RESTYPES = {
    "mcgb_last_error": ctypes.c_char_p,
    "mcgb_version": ctypes.c_char_p,
    "mcgb_batch_smem_bytes": ctypes.c_int64,
    "mcgb_batch_set_wait_limit": ctypes.c_int64,
}

EINVAL, ECUDA, ENOMEM, ETIMEOUT = -1, -2, -3, -4

_lib = None
_lock = threading.Lock()


class MCGBError(RuntimeError):
    """A CUDA-side failure reported by the mcgb library."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


class MCGBTimeout(MCGBError):
    """A bounded device-side wait gave up (the kernel returned instead of hanging)."""


def lib_path() -> Path:
    return _build.LIB_PATH


def load():
    """Load (building first if the library is missing or stale) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if _build.needs_build():
                _build.build()
            handle = ctypes.CDLL(str(_build.LIB_PATH))
            handle.mcgb_last_error.restype = ctypes.c_char_p
            handle.mcgb_last_error.argtypes = []
            handle.mcgb_version.restype = ctypes.c_char_p
            handle.mcgb_version.argtypes = []
            for name, args in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = RESTYPES.get(name, ctypes.c_int)
                fn.argtypes = args
            _lib = handle
    return _lib


def last_error() -> str:
    return load().mcgb_last_error().decode()


def check(status: int, name: str = "") -> None:
    if status == 0:
        return
    msg = last_error() or f"{name} failed with status {status}"
    if status == EINVAL:
        raise ValueError(msg)
    if status == ETIMEOUT:
        raise MCGBTimeout(status, msg)
    raise MCGBError(status, msg)


def call(name: str, *args) -> None:
    """Invoke ``name`` from the C ABI and raise on a nonzero status."""
    fn = getattr(load(), name)
    check(fn(*args), name)


def stream_handle():
    """torch's current CUDA stream as a cudaStream_t (void*)."""
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
