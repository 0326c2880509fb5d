"""He3 thin-film Ginzburg-Landau model: complex64 order parameter (R, L, L, 3, 2).

Drop-in for the reference's models/he3/model.py:28-114 (kernels
models/he3/update.py:9-227 and models/he3/measure.py:22-143, restated in
csrc/he3.cu).  The GL coefficients ``betas`` (not the inverse temperatures)
optionally include the strong-coupling pressure correction.
"""

import ctypes

import numpy as np

from ... import _lib
from ...core.model import Model
from ...device import device_array, ptr, to_device
from .._common import (OutputBuffer, check_rng, check_vector, geometry, launch_measure, read_channels,
                       optional_cache, optional_indices)

MEASUREMENT_NAMES = (
    "energy", "density", "chirality", "phase_real", "phase_imag",
    "current_x", "curvature_x", "current_y", "curvature_y", "spin_alignment",
)
MEASURE_THREADS = 256

# Strong-coupling corrections delta_beta_i / |beta_1^wc| as a polynomial in
# p/34 (rows: powers 0..5; columns: beta_1..beta_5), published in Regan, Wiman
# & Sauls, PRB 101, 024517 (2020), Appendix Table I (arXiv:1908.04190),
# valid for 0 <= p <= 34 bar.  Published data, reproduced as given.
STRONG_COUPLING = np.array([
    [-0.009849, -0.04193, -0.01322, -0.004747, -0.08987],
    [-0.05043, -0.1177, -0.05428, -0.3788, -0.6925],
    [0.02205, -0.04322, 0.09559, -0.1774, 0.8761],
    [-0.02557, 0.08793, -0.06419, 0.1735, -0.5929],
    [0.05023, -0.08598, -0.009310, 0.1878, 0.02904],
    [-0.02769, 0.03639, 0.01862, -0.1522, 0.08870],
])


class He3Model(Model):
    def __init__(self, K=1.0, betas=(-0.5, 1, 1, 1, -1), delta=0.15,
                 pressure=None, reduced_temperature=1.0, g_d=0):
        """GL coefficients, optionally pressure-corrected at a fixed T/Tc.

        pressure=None keeps ``betas``; a pressure in bar (0..34) adds
        0.5 * reduced_temperature * correction(pressure / 34), the lattice
        coefficients being beta_i / (2 |beta_1^wc|).  reduced_temperature is
        independent of the Monte Carlo temperature ladder.
        """
        self.K = np.float32(K)
        self.pressure = None if pressure is None else float(pressure)
        self.reduced_temperature = float(reduced_temperature)
        coefficients = np.asarray(betas, dtype=np.float64)
        if self.pressure is not None:
            correction = np.polynomial.polynomial.polyval(self.pressure / 34, STRONG_COUPLING)
            coefficients = coefficients + 0.5 * self.reduced_temperature * correction
        self.betas = tuple(np.float32(b) for b in coefficients)
        self.delta = np.float32(delta)
        if not np.isfinite(g_d) or g_d < 0:
            raise ValueError("g_d must be finite and nonnegative")
        self.g_d = np.float32(g_d)
        self._out = OutputBuffer()

    def coefficients(self):
        """The five GL coefficients as a float32 host array."""
        return np.ascontiguousarray(np.asarray(self.betas, dtype=np.float32))

    def _cptr(self):
        # Host pointer to the coefficients; kept alive on self for the call.
        self._coeff_host = self.coefficients()
        return self._coeff_host.ctypes.data_as(ctypes.c_void_p)

    def initialize_state(self, L, replicas, seed):
        state = np.zeros((replicas, L, L, 3, 2), dtype=np.complex64)
        # Homogeneous positive-chirality minimum: d = (0, 0, 1), theta = 0.
        beta_chiral = self.betas[1] + self.betas[3] + self.betas[4]
        amplitude = np.float32(1 / np.sqrt(2 * beta_chiral))
        state[..., 2, 0] = amplitude
        state[..., 2, 1] = 1j * amplitude
        return state

    def update_color(self, state, rng_states, betas, color, blocks=None, threads=None):
        R, L = geometry(state, np.complex64, (3, 2), "He3Model.update_color")
        check_rng(rng_states, R, L, "He3Model.update_color")
        check_vector(betas, R, np.float32, "He3Model.update_color", "betas")
        _lib.call("mcgb_he3_update_color", ptr(state), ptr(rng_states), ptr(betas), R, L, int(color),
                  self._cptr(), float(self.K), float(self.delta), float(self.g_d), _lib.stream_handle())

    measurement_names = MEASUREMENT_NAMES

    def measure_into(self, state, out, temperature_indices=None, cached_energies=None):
        """Enqueue the measurement into the (channels, R) float64 device array
        ``out`` without copying it to the host (the device sample ring of
        Simulation uses this)."""
        R, L = geometry(state, np.complex64, (3, 2), "He3Model.measure")
        launch_measure("mcgb_he3_measure", out, len(MEASUREMENT_NAMES), R, "He3Model.measure", ptr(state), R, L,
                       self._cptr(), float(self.K), float(self.g_d),
                       optional_indices(temperature_indices, R, "He3Model.measure"),
                       optional_cache(cached_energies, R, "He3Model.measure"))

    def measure(self, state, temperature_indices=None, cached_energies=None):
        R = int(state.shape[0])
        out = self._out.get(len(MEASUREMENT_NAMES), R)
        self.measure_into(state, out, temperature_indices, cached_energies)
        return read_channels(out, MEASUREMENT_NAMES)

    def measure_with_energy(self, state, energies, temperature_indices=None):
        return self.measure(state, temperature_indices=temperature_indices, cached_energies=energies)

    def measure_energy(self, state, output):
        R, L = geometry(state, np.complex64, (3, 2), "He3Model.measure_energy")
        check_vector(output, R, np.float64, "He3Model.measure_energy", "output")
        _lib.call("mcgb_he3_energy", ptr(state), R, L, self._cptr(), float(self.K), float(self.g_d),
                  ptr(output), _lib.stream_handle())

    def local_differences(self, state, positions, proposed, g_d=None):
        """(gradient, potential, total) energy differences for rows (r, i, j); float64 (3, n)."""
        R, L = geometry(state, np.complex64, (3, 2), "He3Model.local_differences")
        pos = to_device(np.asarray(positions, dtype=np.int32).reshape(-1, 3))
        prop = to_device(np.asarray(proposed, dtype=np.complex64).reshape(-1, 3, 2))
        n = pos.shape[0]
        out = device_array((3, n), np.float64)
        _lib.call("mcgb_he3_local_differences", ptr(state), R, L, ptr(pos), ptr(prop), n, self._cptr(),
                  float(self.K), float(self.g_d if g_d is None else g_d), ptr(out), _lib.stream_handle())
        return out.copy_to_host()

    def parameters(self):
        return {"K": self.K, "betas": self.betas, "delta": self.delta,
                "pressure": self.pressure, "reduced_temperature": self.reduced_temperature,
                "g_d": float(self.g_d), "dipole_length_lattice": (
                    float(np.sqrt(2.0 * self.K / self.g_d)) if self.g_d > 0 else None)}
