"""Model plugin contract between Runtime and a physics model.

Same interface as the reference's core/model.py:6-62: a model supplies its
CPU initial state, launches one checkerboard colour on the device, and
reduces the device state to named float64 arrays with a leading replica axis.
"""

from abc import ABC, abstractmethod

import numpy as np


class Model(ABC):

    @abstractmethod
    def initialize_state(self, L, replicas, seed) -> np.ndarray:
        """Return initial CPU state with shape (replicas, L, L, ...)."""

    @abstractmethod
    def update_color(self, state, rng_states, betas, color, blocks, threads):
        """Launch the CUDA kernel for one checkerboard color.

        ``blocks``/``threads`` carry the reference's launch geometry for
        compatibility; mcgb kernels choose their own geometry.
        """

    @abstractmethod
    def measure(self, state, temperature_indices=None) -> dict:
        """Measure the GPU state; return named CPU arrays with a leading replica axis.

        ``temperature_indices`` (device int32, one entry per physical walker)
        scatters each walker's outputs into its temperature slot on the GPU.
        """

    def measure_energy(self, state, output):
        """Write total energies to a caller-owned float64 GPU array (R,).

        Walker order, the same Hamiltonian for every temperature; no host copy
        and no temporary device allocation.
        """
        raise NotImplementedError(
            "This model does not provide GPU total-energy measurements"
        )

    def measure_with_energy(self, state, energies, temperature_indices=None):
        """Measure observables reusing fresh walker-ordered GPU energies.

        ``energies`` is read-only.  The default ignores it.
        """
        return self.measure(state, temperature_indices=temperature_indices)

    def parameters(self) -> dict:
        """Physical parameters to include in run metadata."""
        return {}
