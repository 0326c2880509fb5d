"""Per-site xoroshiro128+ streams (numba.cuda.random restated on the device).

:func:`create_xoroshiro128p_states` replaces the reference's call of the same
name (core/runtime.py:51-53, core/parallel_tempering.py:177-179): stream k is
SplitMix64(seed) advanced by ``(subsequence_start + k) * 2**64`` steps, as
Numba computes by sequential host jumps; here ``libmcgb`` computes every
stream on the device by GF(2) jump-ahead.
"""

from __future__ import annotations

import numpy as np

from . import _lib
from .device import XOROSHIRO128P_DTYPE, DeviceArray


def create_xoroshiro128p_states(n, seed, subsequence_start=0, stream=0):
    states = DeviceArray((int(n),), XOROSHIRO128P_DTYPE)
    init_xoroshiro128p_states(states, seed, subsequence_start)
    return states


def init_xoroshiro128p_states(states, seed, subsequence_start=0, stream=0):
    n = states.shape[0]
    _lib.call("mcgb_rng_init", states.cptr, n, int(seed) & (2**64 - 1), int(subsequence_start),
              _lib.stream_handle())


def draw_uniforms(states, index, count, kind="float32"):
    """Draw ``count`` uniforms from stream ``index`` on the device (diagnostic)."""
    dtype = np.float32 if kind == "float32" else np.float64
    out = DeviceArray((count,), dtype)
    _lib.call("mcgb_rng_draw", states.cptr, int(index), int(count), 0 if kind == "float32" else 1,
              out.cptr, _lib.stream_handle())
    return out.copy_to_host()
