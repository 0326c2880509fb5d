"""Replica exchange on the device for a temperature-independent Hamiltonian.

Drop-in for the reference's core/parallel_tempering.py:94-317.  States and
site RNG stay in their walker slots; an accepted exchange swaps the two
walkers' betas and the walker<->temperature maps (``mcgb_pt_exchange``).
Matchings alternate between (0,1),(2,3),... and (1,2),(3,4),... for R > 2.
Round-trip counters and the optional walker-history capture run on the
device; diagnostics() is the only host copy.
"""

import operator

import numpy as np

from .. import _lib
from ..device import device_array, ptr, to_device
from ..rng import create_xoroshiro128p_states

# Rows of the (5, R) round-trip bookkeeping array, indexed by physical walker.
_ORIGIN, _VISITED_OTHER, _START_SWEEP, _ROUND_TRIPS, _ROUND_TRIP_SWEEPS = range(5)


def _positive_int(value, message):
    if isinstance(value, (bool, np.bool_)):
        raise ValueError(message)
    try:
        value = operator.index(value)
    except TypeError:
        raise ValueError(message) from None
    if value < 1:
        raise ValueError(message)
    return value


def _walker_ids(tracked_walkers, R):
    if tracked_walkers is None:
        return None
    message = "tracked_walkers must contain integer walker IDs"
    try:
        values = list(tracked_walkers)
        if any(isinstance(v, (bool, np.bool_)) for v in values):
            raise ValueError(message)
        ids = np.asarray([operator.index(v) for v in values], dtype=np.int64)
    except (TypeError, OverflowError):
        raise ValueError(message) from None
    if (ids.ndim != 1 or not len(ids) or np.any(ids < 0) or np.any(ids >= R)
            or len(np.unique(ids)) != len(ids)):
        raise ValueError("tracked_walkers must be distinct IDs in range(R)")
    return ids.astype(np.int32)


class ParallelTempering:
    """Wrap a Runtime and pass this object to Simulation in its place.

    Temperatures must be strictly increasing (distinct float32 betas).  A
    sweep runs all four colours before any exchange; every
    ``exchange_interval`` sweeps the fresh total energies are measured and one
    matching is attempted.  ``history_stride`` counts exchange rounds.
    Diagnostics are cumulative from construction.
    """

    def __init__(self, runtime, exchange_interval=10, seed=None,
                 tracked_walkers=None, history_stride=10):
        interval = _positive_int(exchange_interval, "exchange_interval must be a positive integer")
        if runtime.R < 2:
            raise ValueError("Parallel tempering requires at least two temperatures")
        history_stride = _positive_int(history_stride, "history_stride must be a positive integer")
        walker_ids = _walker_ids(tracked_walkers, runtime.R)

        beta = runtime.betas.copy_to_host()
        expected = (1.0 / runtime.temperatures).astype(np.float32)
        if not np.array_equal(beta, expected):
            raise ValueError("Runtime betas must initially match its temperature order")
        if not np.all(np.isfinite(beta) & (beta > 0)) or not np.all(np.diff(beta) < 0):
            raise ValueError("PT temperatures must have distinct, finite positive float32 betas")

        self.runtime = runtime
        self.model = runtime.model
        self.L = runtime.L
        self.R = runtime.R
        self.temperatures = runtime.temperatures
        self.seed = runtime.seed
        self.exchange_interval = interval
        self.exchange_seed = operator.index(runtime.seed + 1 if seed is None else seed)
        self.sweeps = 0
        self.exchange_rounds = 0
        self._parity = 0
        self._temperature_betas = beta.copy()

        self.energies = device_array(self.R, dtype=np.float64)
        # Fails here if the model has no device energy path.
        runtime.measure_energy(self.energies)
        identity = np.arange(self.R, dtype=np.int32)
        self.walker_to_temperature = to_device(identity)
        self.temperature_to_walker = to_device(identity)
        self._rng_states = create_xoroshiro128p_states(self.R - 1, seed=self.exchange_seed)
        # Per neighbouring edge: attempted, accepted, nonfinite-energy attempts.
        self._swap_counts = to_device(np.zeros((3, self.R - 1), dtype=np.int64))
        trips = np.zeros((5, self.R), dtype=np.int64)
        trips[_ORIGIN] = -1
        trips[_START_SWEEP] = -1
        trips[_ORIGIN, 0] = 0
        trips[_ORIGIN, -1] = self.R - 1
        trips[_START_SWEEP, [0, -1]] = 0
        self._trips = to_device(trips)

        self._tracked_walkers = walker_ids
        self._history_stride = history_stride
        self._history_chunk_rows = 1024
        self._history_chunks = []
        self._history_sweeps = []
        self._history_rounds = []
        self._tracked_walkers_gpu = None if walker_ids is None else to_device(walker_ids)
        if walker_ids is not None:
            self._record_walker_history()

    # ------------------------------------------------------------ history
    def _record_walker_history(self):
        row = len(self._history_sweeps) % self._history_chunk_rows
        if row == 0:
            self._history_chunks.append(device_array(
                (self._history_chunk_rows, len(self._tracked_walkers)), dtype=np.int32))
        _lib.call("mcgb_pt_record_walkers", ptr(self.walker_to_temperature),
                  ptr(self._tracked_walkers_gpu), ptr(self._history_chunks[-1][row]),
                  len(self._tracked_walkers), _lib.stream_handle())
        self._history_sweeps.append(self.sweeps)
        self._history_rounds.append(self.exchange_rounds)

    def _walker_history(self, final_walker_to_temperature):
        count = len(self._history_sweeps)
        rows = []
        for chunk in self._history_chunks:
            used = min(self._history_chunk_rows, count)
            rows.append(chunk[:used].copy_to_host())
            count -= used
        positions = np.concatenate(rows, axis=0)
        sweeps = np.asarray(self._history_sweeps, dtype=np.int64)
        rounds = np.asarray(self._history_rounds, dtype=np.int64)
        if rounds[-1] != self.exchange_rounds or sweeps[-1] != self.sweeps:
            # Append the current position without changing the recording state.
            positions = np.concatenate(
                (positions, final_walker_to_temperature[self._tracked_walkers][None, :]), axis=0)
            sweeps = np.append(sweeps, self.sweeps)
            rounds = np.append(rounds, self.exchange_rounds)
        return {
            "walker_ids": self._tracked_walkers.copy(),
            "sweeps": sweeps,
            "exchange_rounds": rounds,
            "temperature_indices": positions,
            "stride": self._history_stride,
            "stride_units": "exchange_rounds",
        }

    # ------------------------------------------------------------ schedule
    def sweep(self):
        self.runtime.sweep()
        self.sweeps += 1
        if self.sweeps % self.exchange_interval == 0:
            self.attempt_exchanges()

    def attempt_exchanges(self):
        """Measure the current TOTAL energies, then attempt the next matching."""
        self.runtime.measure_energy(self.energies)
        _lib.call("mcgb_pt_exchange", ptr(self.energies), ptr(self.runtime.betas),
                  ptr(self.walker_to_temperature), ptr(self.temperature_to_walker),
                  ptr(self._rng_states), ptr(self._swap_counts), ptr(self._trips),
                  self.R, self._parity, self.sweeps, _lib.stream_handle())
        self.exchange_rounds += 1
        if self.R > 2:
            self._parity = 1 - self._parity
        if (self._tracked_walkers is not None
                and self.exchange_rounds % self._history_stride == 0):
            self._record_walker_history()

    # ------------------------------------------------------------ replay hooks
    # Simulation replays whole schedules as captured CUDA graphs: these
    # enqueue the device work of one exchange round with the schedule read
    # from a device clock {sweeps, rounds}, and account on the host for the
    # rounds a replay ran.

    def _enqueue_exchange(self, clock, advance):
        """attempt_exchanges' launches: fresh energies, then the round after
        clock[0] + advance sweeps at parity clock[1] % 2 (no host state)."""
        rt = self.runtime
        rt.model.measure_energy(rt.state, self.energies)
        _lib.call("mcgb_pt_exchange_clocked", ptr(self.energies), ptr(rt.betas),
                  ptr(self.walker_to_temperature), ptr(self.temperature_to_walker),
                  ptr(self._rng_states), ptr(self._swap_counts), ptr(self._trips),
                  self.R, ptr(clock), int(advance), _lib.stream_handle())

    def _enqueue_history(self, ring, head):
        """A walker-history row into the device ring ``ring[head]``."""
        _lib.call("mcgb_pt_record_walkers_ring", ptr(self.walker_to_temperature),
                  ptr(self._tracked_walkers_gpu), ptr(ring), ptr(head), len(self._tracked_walkers),
                  int(ring.shape[0]), _lib.stream_handle())

    def _rounds_done(self, sweeps, rounds, history=None, coordinates=()):
        """Host bookkeeping after a replay that ran ``sweeps`` sweeps and
        ``rounds`` exchange rounds; ``history`` holds the walker-history rows
        it recorded at the (sweep, round) ``coordinates``."""
        self.sweeps += sweeps
        self.exchange_rounds += rounds
        if self.R > 2 and rounds % 2:
            self._parity = 1 - self._parity
        for k, (sweep, rnd) in enumerate(coordinates):
            row = len(self._history_sweeps) % self._history_chunk_rows
            if row == 0:
                self._history_chunks.append(device_array(
                    (self._history_chunk_rows, len(self._tracked_walkers)), dtype=np.int32))
            self._history_chunks[-1][row].raw().copy_(history[k].raw())
            self._history_sweeps.append(sweep)
            self._history_rounds.append(rnd)

    def measure(self):
        """CPU observables in the fixed temperature order."""
        return self.runtime.measure(temperature_indices=self.walker_to_temperature)

    def snapshot(self):
        """CPU snapshot in temperature order; the Runtime stays walker ordered."""
        state = self.runtime.snapshot()
        return state[self.temperature_to_walker.copy_to_host()]

    def diagnostics(self):
        """Copy the small diagnostic arrays to the host."""
        counts = self._swap_counts.copy_to_host()
        if np.any(counts[2]):
            raise FloatingPointError("Nonfinite energies encountered during replica exchange")
        trips = self._trips.copy_to_host()
        w_to_t = self.walker_to_temperature.copy_to_host()
        t_to_w = self.temperature_to_walker.copy_to_host()
        attempts, accepted = counts[:2]
        rates = np.divide(accepted, attempts, out=np.zeros(self.R - 1), where=attempts > 0)
        completed = int(trips[_ROUND_TRIPS].sum())
        mean_trip = float(trips[_ROUND_TRIP_SWEEPS].sum()) / completed if completed else None
        result = {
            "exchange_interval": self.exchange_interval,
            "exchange_seed": self.exchange_seed,
            "sweeps": self.sweeps,
            "exchange_rounds": self.exchange_rounds,
            "next_parity": self._parity,
            "diagnostics_scope": "since_wrapper_creation_including_thermalization",
            "temperature_betas": self._temperature_betas.copy(),
            "attempts": attempts.copy(),
            "accepted": accepted.copy(),
            "acceptance_rates": rates,
            "walker_to_temperature": w_to_t,
            "temperature_to_walker": t_to_w,
            "walker_round_trips": trips[_ROUND_TRIPS].copy(),
            "walker_round_trip_total_sweeps": trips[_ROUND_TRIP_SWEEPS].copy(),
            "mean_round_trip_sweeps": mean_trip,
        }
        if self._tracked_walkers is not None:
            result["walker_history"] = self._walker_history(w_to_t)
        return result
