"""Conditional-Gaussian proposals with full-Hamiltonian MH correction.

Drop-in for the reference's models/he3/gaussian_fast.py:122-156
(FastGaussianUpdater): step() replaces one sweep with four launches of the
conditional Gaussian AR kernel (csrc/he3.cu he3_gauss_color_kernel) and keeps
per-site int64 attempted/accepted/nonfinite counters on the device.
"""

import numpy as np

from ... import _lib
from ...device import ptr, to_device


class FastGaussianUpdater:
    """A float32 conditional Gaussian sampler; step() replaces one sweep."""

    def __init__(self, runtime, rho=0.0, mass=0.0):
        if len(runtime.state.shape) != 5 or tuple(runtime.state.shape[-2:]) != (3, 2):
            raise ValueError("FastGaussianUpdater requires full complex 3x2 He3 fields")
        rho, mass = np.float32(rho), np.float32(mass)
        eigenvalues = np.asarray([6, 10], dtype=np.float32) * runtime.model.K + mass
        if not np.isfinite(mass) or not np.all(np.isfinite(eigenvalues) & (eigenvalues > 0)):
            raise ValueError("Conditional quadratic Gaussian requires positive finite float32 "
                             "orbital eigenvalues")
        if not np.isfinite(rho) or not -1 < rho < 1:
            raise ValueError("Require -1 < float32(rho) < 1 for nondegenerate proposals")
        self.runtime, self.rho, self.mass = runtime, rho, mass
        self.counts = to_device(np.zeros((3, runtime.R, runtime.L, runtime.L), dtype=np.int64))
        self.sweeps = 0

    def step(self):
        self.runtime.invalidate_energy_cache()
        self.enqueue()
        self.sweeps += 1

    def enqueue(self):
        """The four colour launches of one sweep, nothing on the host."""
        rt = self.runtime
        model = rt.model
        for color in range(4):
            _lib.call("mcgb_he3_gaussian_update_color", ptr(rt.state), ptr(rt.rng_states), ptr(rt.betas),
                      rt.R, rt.L, color, model._cptr(), float(model.K), float(self.rho), float(self.mass),
                      float(model.g_d), ptr(self.counts), _lib.stream_handle())

    def diagnostics(self):
        counts = self.counts.copy_to_host().sum(axis=(2, 3))
        return {
            "algorithm": "float32_conditional_gaussian_full_hamiltonian_mh",
            "sweeps_including_compilation": self.sweeps,
            "rho": float(self.rho), "proposal_mass": float(self.mass),
            "attempts": counts[0].tolist(), "accepted": counts[1].tolist(),
            "nonfinite_rejections": counts[2].tolist(),
            "acceptance_rates": np.divide(counts[1], counts[0], out=np.zeros(self.runtime.R),
                                          where=counts[0] > 0).tolist(),
        }
