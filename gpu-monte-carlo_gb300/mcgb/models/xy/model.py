"""XY model plugin: float32 angles (R, L, L) in [-pi, pi), drop-in for the
reference's models/xy/model.py:15-74 (kernels models/xy/update.py:6-54 and
models/xy/measure.py:17-134, restated in csrc/lattice.cu).

``proposal="uniform"`` (default) is the reference's theta + delta*(2u-1);
``proposal="gaussian"`` draws theta + sigma*z with per-walker sigma held in
``sigmas`` (a device float32 array the caller owns, one entry per walker).
"""

import math

import numpy as np

from ... import _lib
from ...core.model import Model
from ...device import ptr
from .._common import (OutputBuffer, check_rng, check_vector, geometry, launch_measure, read_channels,
                       optional_cache, optional_indices)

MEASUREMENT_NAMES = ("energy", "mx", "my", "twist_cos_x", "twist_sin_x")
MEASURE_THREADS = 256


class XYModel(Model):
    def __init__(self, J=1.0, delta=1.5, proposal="uniform", sigmas=None):
        if J <= 0:
            raise ValueError("J must be positive")
        if not (0 < delta <= math.pi):
            raise ValueError("delta must be in (0, pi]")
        if proposal not in ("uniform", "gaussian"):
            raise ValueError("proposal must be 'uniform' or 'gaussian'")
        self.J = np.float32(J)
        self.delta = np.float32(delta)
        self.proposal = proposal
        self.sigmas = sigmas
        self._out = OutputBuffer()

    def initialize_state(self, L, replicas, seed):
        return np.zeros((replicas, L, L), dtype=np.float32)

    def update_color(self, state, rng_states, betas, color, blocks=None, threads=None):
        R, L = geometry(state, np.float32, (), "XYModel.update_color")
        check_rng(rng_states, R, L, "XYModel.update_color")
        check_vector(betas, R, np.float32, "XYModel.update_color", "betas")
        if self.proposal == "uniform":
            _lib.call("mcgb_xy_update_color", ptr(state), ptr(rng_states), ptr(betas), R, L,
                      int(color), float(self.J), float(self.delta), _lib.stream_handle())
        else:
            if self.sigmas is None:
                raise ValueError("Gaussian proposals need per-walker sigmas")
            check_vector(self.sigmas, R, np.float32, "XYModel.update_color", "sigmas")
            _lib.call("mcgb_xy_update_color_gauss", ptr(state), ptr(rng_states), ptr(betas),
                      ptr(self.sigmas), R, L, int(color), float(self.J), _lib.stream_handle())

    def enqueue_sweep(self, state, rng_states, betas):
        """One whole sweep in three launches (colours 0, {1, 2}, 3: colours 1
        and 2 share no bond), bit-identical to four update_color calls.
        Returns False, enqueueing nothing, when a subclass or the instance
        replaced update_color, so that its own colour updates run instead."""
        if type(self).update_color is not XYModel.update_color or "update_color" in vars(self):
            return False
        R, L = geometry(state, np.float32, (), "XYModel.enqueue_sweep")
        check_rng(rng_states, R, L, "XYModel.enqueue_sweep")
        check_vector(betas, R, np.float32, "XYModel.enqueue_sweep", "betas")
        sig = None
        if self.proposal == "gaussian":
            if self.sigmas is None:
                raise ValueError("Gaussian proposals need per-walker sigmas")
            check_vector(self.sigmas, R, np.float32, "XYModel.enqueue_sweep", "sigmas")
            sig = ptr(self.sigmas)
        _lib.call("mcgb_xy_sweep", ptr(state), ptr(rng_states), ptr(betas), sig, R, L, float(self.J),
                  float(self.delta), 1, _lib.stream_handle())
        return True

    measurement_names = MEASUREMENT_NAMES

    def measure_into(self, state, out, temperature_indices=None, cached_energies=None):
        """Enqueue the measurement into the (channels, R) float64 device array
        ``out`` without copying it to the host (the device sample ring of
        Simulation uses this)."""
        R, L = geometry(state, np.float32, (), "XYModel.measure")
        launch_measure("mcgb_xy_measure", out, len(MEASUREMENT_NAMES), R, "XYModel.measure", ptr(state), R, L,
                       float(self.J), optional_indices(temperature_indices, R, "XYModel.measure"),
                       optional_cache(cached_energies, R, "XYModel.measure"))

    def measure(self, state, temperature_indices=None, cached_energies=None):
        R = int(state.shape[0])
        out = self._out.get(len(MEASUREMENT_NAMES), R)
        self.measure_into(state, out, temperature_indices, cached_energies)
        return read_channels(out, MEASUREMENT_NAMES)

    def measure_with_energy(self, state, energies, temperature_indices=None):
        return self.measure(state, temperature_indices=temperature_indices, cached_energies=energies)

    def parameters(self):
        params = {"J": self.J, "delta": self.delta}
        if self.proposal != "uniform":
            params["proposal"] = self.proposal
        return params

    def measure_energy(self, state, output):
        R, L = geometry(state, np.float32, (), "XYModel.measure_energy")
        check_vector(output, R, np.float64, "XYModel.measure_energy", "output")
        _lib.call("mcgb_xy_energy", ptr(state), R, L, float(self.J), ptr(output), _lib.stream_handle())
