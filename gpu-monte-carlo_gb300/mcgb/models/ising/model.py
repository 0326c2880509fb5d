"""2D Ising model plugin: int8 spins (R, L, L), drop-in for the reference's
models/ising/model.py:12-64 (kernels models/ising/update.py:7-29 and
models/ising/measure.py:10-99, restated in csrc/lattice.cu)."""

import numpy as np

from ... import _lib
from ...core.model import Model
from ...device import ptr
from .._common import (OutputBuffer, check_rng, check_vector, geometry, launch_measure, read_channels,
                       optional_cache, optional_indices)

MEASUREMENT_NAMES = ("energy", "magnetization")
MEASURE_THREADS = 256


class IsingModel(Model):
    def __init__(self, J=1.0):
        self.J = np.float32(J)
        self._out = OutputBuffer()

    def initialize_state(self, L, replicas, seed):
        return np.ones((replicas, L, L), dtype=np.int8)

    def update_color(self, state, rng_states, betas, color, blocks=None, threads=None):
        R, L = geometry(state, np.int8, (), "IsingModel.update_color")
        check_rng(rng_states, R, L, "IsingModel.update_color")
        check_vector(betas, R, np.float32, "IsingModel.update_color", "betas")
        _lib.call("mcgb_ising_update_color", ptr(state), ptr(rng_states), ptr(betas), R, L,
                  int(color), float(self.J), _lib.stream_handle())

    def enqueue_sweep(self, state, rng_states, betas):
        """One whole sweep in three launches (colours 0, {1, 2}, 3: colours 1
        and 2 share no bond), bit-identical to four update_color calls.
        Returns False, enqueueing nothing, when a subclass or the instance
        replaced update_color, so that its own colour updates run instead."""
        if type(self).update_color is not IsingModel.update_color or "update_color" in vars(self):
            return False
        R, L = geometry(state, np.int8, (), "IsingModel.enqueue_sweep")
        check_rng(rng_states, R, L, "IsingModel.enqueue_sweep")
        check_vector(betas, R, np.float32, "IsingModel.enqueue_sweep", "betas")
        _lib.call("mcgb_ising_sweep", ptr(state), ptr(rng_states), ptr(betas), R, L, float(self.J), 1,
                  _lib.stream_handle())
        return True

    def sweep(self, state, rng_states, betas, n_sweeps=1):
        """n_sweeps full sweeps in three launches each (colours 0, {1, 2}, 3)."""
        R, L = geometry(state, np.int8, (), "IsingModel.sweep")
        check_rng(rng_states, R, L, "IsingModel.sweep")
        check_vector(betas, R, np.float32, "IsingModel.sweep", "betas")
        _lib.call("mcgb_ising_sweep", ptr(state), ptr(rng_states), ptr(betas), R, L,
                  float(self.J), int(n_sweeps), _lib.stream_handle())

    measurement_names = MEASUREMENT_NAMES

    def measure_into(self, state, out, temperature_indices=None, cached_energies=None):
        """Enqueue the measurement into the (channels, R) float64 device array
        ``out`` without copying it to the host (the device sample ring of
        Simulation uses this)."""
        R, L = geometry(state, np.int8, (), "IsingModel.measure")
        launch_measure("mcgb_ising_measure", out, len(MEASUREMENT_NAMES), R, "IsingModel.measure", ptr(state), R, L,
                       float(self.J), optional_indices(temperature_indices, R, "IsingModel.measure"),
                       optional_cache(cached_energies, R, "IsingModel.measure"))

    def measure(self, state, temperature_indices=None, cached_energies=None):
        R = int(state.shape[0])
        out = self._out.get(len(MEASUREMENT_NAMES), R)
        self.measure_into(state, out, temperature_indices, cached_energies)
        return read_channels(out, MEASUREMENT_NAMES)

    def measure_with_energy(self, state, energies, temperature_indices=None):
        return self.measure(state, temperature_indices=temperature_indices, cached_energies=energies)

    def measure_energy(self, state, output):
        R, L = geometry(state, np.int8, (), "IsingModel.measure_energy")
        check_vector(output, R, np.float64, "IsingModel.measure_energy", "output")
        _lib.call("mcgb_ising_energy", ptr(state), R, L, float(self.J), ptr(output), _lib.stream_handle())

    def parameters(self):
        return {"J": self.J}
