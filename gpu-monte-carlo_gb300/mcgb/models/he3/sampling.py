"""He3 runtime whose sweep is the conditional Gaussian MH update.

Drop-in for the reference's models/he3/sampling.py:8-33.
"""

from ...core.runtime import Runtime
from .gaussian_fast import FastGaussianUpdater
from .model import He3Model


class He3GaussianRuntime(Runtime):

    def __init__(self, model, L, temperatures, threads=16, seed=42, rho=-0.9, proposal_mass=0.0):
        if not isinstance(model, He3Model):
            raise TypeError("Requires He3Model")
        super().__init__(model, L, temperatures, threads=threads, seed=seed)
        self.gaussian = FastGaussianUpdater(self, rho=rho, mass=proposal_mass)

    def sweep(self):
        self.gaussian.step()

    def _enqueue_sweep(self):
        self.gaussian.enqueue()

    def _sweeps_done(self, n):
        self.gaussian.sweeps += n

    def sampling_diagnostics(self):
        return self.gaussian.diagnostics()
