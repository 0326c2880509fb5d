"""The plain float64 form of an XY parallel-tempering ladder.

Every replica is updated by its own four colour launches (``mcgb_xy64_update_color``:
float64 angles, float64 proposals, float64 exponentials), the exchange
energies come from one float64 reduction per lattice (``mcgb_xy64_energy``) and
the swap itself is the reference's exchange kernel (``mcgb_pt_exchange``,
core/parallel_tempering.py:35-91).  The sweep/exchange schedule is
``ParallelTempering.sweep`` (core/parallel_tempering.py:245-269): one sweep,
then an exchange attempt every ``exchange_interval`` sweeps with alternating
pair parity.

This is the baseline the mixed-precision batched engine is compared with:
the same Markov chain family, computed the plain way.  Nothing in the batched
engine depends on it.  ``sweep`` replays each full exchange interval (its
per-lattice launches and the exchange) from a captured CUDA graph, with the
exchange's sweep and parity read from a device clock, so the form is timed
by its kernels -- one lattice per launch, float64 arithmetic -- and not by
host dispatch; ``graph=False`` launches everything directly.
"""

import numpy as np
import torch

from . import _lib
from .device import device_zeros, to_device
from .rng import create_xoroshiro128p_states

CHANNELS = ("energy", "mx", "my", "twist_cos_x", "twist_sin_x")


class PlainXYLadder:
    """One XY ladder of ``len(temperatures)`` replicas of an L x L lattice.

    ``sigmas`` (per temperature) selects Gaussian proposals theta + sigma*z;
    ``None`` selects the reference's uniform theta + delta*(2u - 1).
    """

    def __init__(self, L, temperatures, seed, sigmas=None, delta=1.5, J=1.0, exchange_interval=10,
                 exchange_seed=None, initial_state=None):
        T = np.asarray(temperatures, dtype=np.float64)
        if L < 2 or L % 2:
            raise ValueError("L must be even and at least 2")
        if T.ndim != 1 or len(T) < 2 or np.any(T <= 0) or np.any(np.diff(T) <= 0):
            raise ValueError("temperatures must be positive and increasing, at least two")
        if int(exchange_interval) != exchange_interval or exchange_interval < 1:
            raise ValueError("exchange_interval must be a positive integer")
        self.L, self.R, self.J, self.delta = int(L), len(T), float(J), float(delta)
        self.temperatures = T
        self.exchange_interval = int(exchange_interval)
        if initial_state is None:
            initial_state = np.zeros((self.R, L, L))
        initial_state = np.asarray(initial_state, dtype=np.float64)
        if initial_state.shape != (self.R, L, L):
            raise ValueError("initial_state must have shape (R, L, L)")
        self.theta = to_device(np.ascontiguousarray(initial_state))
        self.rng = create_xoroshiro128p_states(self.R * L * L, int(seed))
        self.betas64 = to_device(1.0 / T)                         # per temperature slot
        self.betas32 = to_device((1.0 / T).astype(np.float32))    # per walker, swapped by the exchange
        self.sigmas = None if sigmas is None else to_device(np.asarray(sigmas, np.float64))
        if self.sigmas is not None and self.sigmas.shape != (self.R,):
            raise ValueError("sigmas must hold one value per temperature")
        self.energies = device_zeros(self.R, np.float64)
        self.w2t = to_device(np.arange(self.R, dtype=np.int32))
        self.t2w = to_device(np.arange(self.R, dtype=np.int32))
        self.exchange_rng = create_xoroshiro128p_states(self.R - 1, int(seed) + 1 if exchange_seed is None
                                                        else int(exchange_seed))
        self.swap_counts = device_zeros((3, self.R - 1), np.int64)
        # Round-trip bookkeeping rows (origin end, visited the other end, start
        # sweep, trips, trip sweeps): only walkers starting at an end have an origin.
        trips = np.zeros((5, self.R), np.int64)
        trips[0] = -1
        trips[2] = -1
        trips[0, 0], trips[0, -1] = 0, self.R - 1
        trips[2, [0, -1]] = 0
        self.trips = to_device(trips)
        self.sweeps = 0
        self.exchange_rounds = 0
        self._parity = 0
        # Device clock {sweeps at the last exchange, rounds} read by the
        # clocked exchange kernel; sweeps since then, on the host.
        self.clock = device_zeros(2, np.int64)
        self._since_exchange = 0
        self._graphs = {}
        self._measured = device_zeros((len(CHANNELS), self.R), np.float64)

    def _energy(self, s):
        for r in range(self.R):
            _lib.call("mcgb_xy64_energy", self.theta.cptr, self.R, self.L, r, self.J, self.energies.cptr, s)

    def _enqueue(self, n_sweeps, exchange, advance):
        """Launches of n_sweeps sweeps and, if `exchange`, of the exchange
        round ``advance`` sweeps after the previous one (no host state)."""
        s = _lib.stream_handle()
        sig = None if self.sigmas is None else self.sigmas.cptr
        for _ in range(n_sweeps):
            for r in range(self.R):
                for c in range(4):
                    _lib.call("mcgb_xy64_update_color", self.theta.cptr, self.rng.cptr, self.betas64.cptr, sig,
                              self.w2t.cptr, self.R, self.L, r, c, self.J, self.delta, s)
        if exchange:
            self._energy(s)
            _lib.call("mcgb_pt_exchange_clocked", self.energies.cptr, self.betas32.cptr, self.w2t.cptr,
                      self.t2w.cptr, self.exchange_rng.cptr, self.swap_counts.cptr, self.trips.cptr,
                      self.R, self.clock.cptr, int(advance), s)

    def sweep(self, n=1, graph=True):
        """n sweeps with an exchange attempt every ``exchange_interval``
        sweeps (ParallelTempering.sweep's schedule, alternating parity)."""
        left = int(n)
        while left > 0:
            to_exchange = self.exchange_interval - self.sweeps % self.exchange_interval
            k = min(left, to_exchange)
            exchange = k == to_exchange
            advance = self._since_exchange + k
            if graph and exchange and k == self.exchange_interval:
                # A whole interval in this call (so advance == k): one graph.
                g = self._graphs.get(k)
                if g is None:
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g):
                        self._enqueue(k, True, k)
                    self._graphs[k] = g
                g.replay()
            else:
                self._enqueue(k, exchange, advance)
            self.sweeps += k
            left -= k
            if exchange:
                self._since_exchange = 0
                self.exchange_rounds += 1
                if self.R > 2:
                    self._parity = 1 - self._parity
            else:
                self._since_exchange = advance

    def measure_energy(self):
        """Float64 total energies in temperature order."""
        self._energy(_lib.stream_handle())
        return self.energies.copy_to_host()[self.t2w.copy_to_host()]

    def measure(self):
        """The reference's five XY channels (models/xy/measure.py:17-134),
        summed in float64, in temperature order: {name: (R,)}."""
        s = _lib.stream_handle()
        for r in range(self.R):
            _lib.call("mcgb_xy64_measure", self.theta.cptr, self.R, self.L, r, self.J, self.w2t.cptr,
                      self._measured.cptr, s)
        values = self._measured.copy_to_host()
        return {name: values[c].copy() for c, name in enumerate(CHANNELS)}

    def simulate(self, thermalization_sweeps=1000, measurement_sweeps=4000, sample_interval=10, channels="all"):
        """The Simulation.run schedule (core/simulation.py:28-96):
        ``{"samples": {channel: (n, R)}, "metadata": ...}`` with the five XY
        channels (``channels="energy"``: the energy alone)."""
        if thermalization_sweeps < 0:
            raise ValueError("Thermalization sweeps cannot be negative")
        if measurement_sweeps < 1:
            raise ValueError("Measurement sweeps must be positive")
        if sample_interval < 1 or sample_interval > measurement_sweeps:
            raise ValueError("Invalid sampling interval")
        self.sweep(thermalization_sweeps)
        rows = []
        for k in range(1, measurement_sweeps + 1):
            self.sweep(1)
            if k % sample_interval == 0:
                rows.append(self.measure() if channels == "all" else {"energy": self.measure_energy()})
        counts = self.swap_counts.copy_to_host()
        metadata = {"L": self.L, "temperatures": self.temperatures.copy(),
                    "model_parameters": {"J": self.J, "delta": self.delta},
                    "thermalization_sweeps": thermalization_sweeps, "measurement_sweeps": measurement_sweeps,
                    "sample_interval": sample_interval,
                    "acceptance_rates": np.divide(counts[1], counts[0], out=np.zeros(self.R - 1),
                                                  where=counts[0] > 0)}
        return {"samples": {k: np.stack([row[k] for row in rows]) for k in rows[0]}, "metadata": metadata}
