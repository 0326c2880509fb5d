"""Shared host-side helpers for the model plugins."""

import numpy as np

from .. import _lib
from ..device import DeviceArray, device_array, ptr


def geometry(state, dtype, trailing, who):
    """Validate a device state's dtype/shape and return (R, L)."""
    shape = tuple(state.shape)
    if len(shape) != 3 + len(trailing) or tuple(shape[3:]) != tuple(trailing) or shape[1] != shape[2]:
        raise ValueError(f"{who}: state must have shape (R, L, L{''.join(', %d' % t for t in trailing)})")
    if np.dtype(state.dtype) != np.dtype(dtype):
        raise ValueError(f"{who}: state must be {np.dtype(dtype)}, got {state.dtype}")
    R, L = int(shape[0]), int(shape[1])
    if L < 4 or L % 2:
        raise ValueError(f"{who}: L must be even and >= 4")
    return R, L


def check_rng(rng_states, R, L, who):
    if rng_states.shape[0] < R * L * L:
        raise ValueError(f"{who}: need {R * L * L} RNG streams, got {rng_states.shape[0]}")


def check_vector(a, n, dtype, who, name):
    if a.shape[0] < n or np.dtype(a.dtype) != np.dtype(dtype):
        raise ValueError(f"{who}: {name} must be a {np.dtype(dtype)} device array of length >= {n}")


class OutputBuffer:
    """Reusable (C, R) float64 device output for measurements."""

    def __init__(self):
        self._buf = None

    def get(self, channels, R):
        if self._buf is None or self._buf.shape != (channels, R):
            self._buf = device_array((channels, R), np.float64)
        return self._buf


def launch_measure(fn_name, out, channels, R, who, *args):
    """Enqueue a (channels, R) float64 measurement into the device array ``out``."""
    if tuple(out.shape) != (channels, R) or np.dtype(out.dtype) != np.float64:
        raise ValueError(f"{who}: output must be a float64 device array of shape ({channels}, {R})")
    _lib.call(fn_name, *args, ptr(out), _lib.stream_handle())


def read_channels(out, names):
    """Copy a (channels, R) measurement to the host as {name: (R,) array}."""
    values = out.copy_to_host()
    return {name: values[c].copy() for c, name in enumerate(names)}


def optional_indices(temperature_indices, R, who):
    if temperature_indices is None:
        return None
    check_vector(temperature_indices, R, np.int32, who, "temperature_indices")
    return ptr(temperature_indices)


def optional_cache(cached, R, who):
    if cached is None:
        return None
    check_vector(cached, R, np.float64, who, "cached energies")
    return ptr(cached)
