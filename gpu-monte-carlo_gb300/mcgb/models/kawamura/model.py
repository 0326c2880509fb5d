"""Kawamura model plugin (PRL 82, 964 (1999), Eq. 3):

    H = -J sum_<ij> (1 + tau_i tau_j) cos(theta_i - theta_j) (d_i . d_j)

float32 state (R, L, L, 5) = theta, tau, dx, dy, dz with |d| = 1.  Drop-in for
the reference's models/kawamura/model.py:19-61 (kernels
models/kawamura/update.py:7-65 and models/kawamura/measure.py:14-122,
restated in csrc/lattice.cu).
"""

import numpy as np

from ... import _lib
from ...core.model import Model
from ...device import ptr
from .._common import (OutputBuffer, check_rng, check_vector, geometry, launch_measure, read_channels,
                       optional_cache, optional_indices)

MEASUREMENT_NAMES = ("energy", "chirality", "px", "py", "spin2", "twist_cos_x", "twist_sin_x")
MEASURE_THREADS = 256


class KawamuraModel(Model):
    def __init__(self, J=1.0, delta=1.5):
        self.J = np.float32(J)
        self.delta = np.float32(delta)  # phase proposal half-width, <= pi
        self._out = OutputBuffer()

    def initialize_state(self, L, replicas, seed):
        state = np.zeros((replicas, L, L, 5), dtype=np.float32)
        state[..., 1] = 1  # ordered chirality, theta = 0, d = (0, 0, 1)
        state[..., 4] = 1
        return state

    def update_color(self, state, rng_states, betas, color, blocks=None, threads=None):
        R, L = geometry(state, np.float32, (5,), "KawamuraModel.update_color")
        check_rng(rng_states, R, L, "KawamuraModel.update_color")
        check_vector(betas, R, np.float32, "KawamuraModel.update_color", "betas")
        _lib.call("mcgb_kawamura_update_color", ptr(state), ptr(rng_states), ptr(betas), R, L,
                  int(color), float(self.J), float(self.delta), _lib.stream_handle())

    def enqueue_sweep(self, state, rng_states, betas):
        """One whole sweep in three launches (colours 0, {1, 2}, 3: colours 1
        and 2 share no bond), bit-identical to four update_color calls.
        Returns False, enqueueing nothing, when a subclass or the instance
        replaced update_color, so that its own colour updates run instead."""
        if type(self).update_color is not KawamuraModel.update_color or "update_color" in vars(self):
            return False
        R, L = geometry(state, np.float32, (5,), "KawamuraModel.enqueue_sweep")
        check_rng(rng_states, R, L, "KawamuraModel.enqueue_sweep")
        check_vector(betas, R, np.float32, "KawamuraModel.enqueue_sweep", "betas")
        _lib.call("mcgb_kawamura_sweep", ptr(state), ptr(rng_states), ptr(betas), R, L, float(self.J),
                  float(self.delta), 1, _lib.stream_handle())
        return True

    measurement_names = MEASUREMENT_NAMES

    def measure_into(self, state, out, temperature_indices=None, cached_energies=None):
        """Enqueue the measurement into the (channels, R) float64 device array
        ``out`` without copying it to the host (the device sample ring of
        Simulation uses this)."""
        R, L = geometry(state, np.float32, (5,), "KawamuraModel.measure")
        launch_measure("mcgb_kawamura_measure", out, len(MEASUREMENT_NAMES), R, "KawamuraModel.measure", ptr(state), R, L,
                       float(self.J), optional_indices(temperature_indices, R, "KawamuraModel.measure"),
                       optional_cache(cached_energies, R, "KawamuraModel.measure"))

    def measure(self, state, temperature_indices=None, cached_energies=None):
        R = int(state.shape[0])
        out = self._out.get(len(MEASUREMENT_NAMES), R)
        self.measure_into(state, out, temperature_indices, cached_energies)
        return read_channels(out, MEASUREMENT_NAMES)

    def measure_with_energy(self, state, energies, temperature_indices=None):
        return self.measure(state, temperature_indices=temperature_indices, cached_energies=energies)

    def measure_energy(self, state, output):
        R, L = geometry(state, np.float32, (5,), "KawamuraModel.measure_energy")
        check_vector(output, R, np.float64, "KawamuraModel.measure_energy", "output")
        _lib.call("mcgb_kawamura_energy", ptr(state), R, L, float(self.J), ptr(output), _lib.stream_handle())

    def local_energies(self, state, positions, proposed):
        """Local energies (stored site, proposal) for rows (r, i, j); float32 (2, n)."""
        from ...device import device_array, to_device

        R, L = geometry(state, np.float32, (5,), "KawamuraModel.local_energies")
        pos = to_device(np.asarray(positions, dtype=np.int32).reshape(-1, 3))
        prop = to_device(np.asarray(proposed, dtype=np.float32).reshape(-1, 5))
        n = pos.shape[0]
        out = device_array((2, n), np.float32)
        _lib.call("mcgb_kawamura_local_energies", ptr(state), R, L, ptr(pos), ptr(prop), n,
                  float(self.J), ptr(out), _lib.stream_handle())
        return out.copy_to_host()

    def parameters(self):
        return {"J": self.J, "delta": self.delta}
