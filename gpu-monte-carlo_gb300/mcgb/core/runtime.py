"""Device owner for one lattice size and one temperature ladder.

Drop-in for the reference's ``Runtime`` (core/runtime.py:8-135).  The
contract kept from it: the constructor ``Runtime(model, L, temperatures,
threads=16, seed=42)`` and its ValueError conditions and messages
(:14-30, :44-45); the attributes ``state`` (the model's initial state on the
device, reference layout), ``rng_states`` (one xoroshiro128+ stream per site,
index ``r*L*L + i*L + j``), ``betas`` (float32 ``1/T`` in walker order),
``threads_per_block``/``blocks_per_grid``, ``R``, ``L``, ``temperatures``,
``seed``; the methods ``sweep``, ``measure``, ``measure_energy``,
``invalidate_energy_cache`` and ``snapshot``; and the energy-cache rule
(:70-132): energies written by ``measure_energy`` into a caller-owned device
buffer serve ``measure`` until the configuration next changes.

This project's structure around it: every sweep is split into the device
work (``_enqueue_sweep``, launches only, so a CUDA graph can capture it) and
the host bookkeeping (``_sweeps_done`` and the energy cache), which lets
``Simulation`` replay a whole sweep/exchange/sample schedule as captured
graphs and account for it once; the energy cache is an ``EnergyCache`` object stamped with a
configuration generation.
"""

import numpy as np

from ..device import to_device
from ..rng import create_xoroshiro128p_states


class EnergyCache:
    """Total energies in a caller-owned device buffer, valid for one
    configuration generation.

    ``advance()`` starts a new generation (the state changed or may have
    changed) and drops the buffer; ``publish(buffer)`` stamps it with the
    current generation; ``current()`` returns it only while the generation
    is unchanged.  ``withdraw()`` drops it without a new generation (a
    producer failed part-way through writing it).
    """

    __slots__ = ("generation", "_buffer", "_stamp")

    def __init__(self):
        self.generation = 0
        self._buffer = None
        self._stamp = -1

    def advance(self):
        self.generation += 1
        self.withdraw()

    def withdraw(self):
        self._buffer, self._stamp = None, -1

    def publish(self, buffer):
        self._buffer, self._stamp = buffer, self.generation

    def current(self):
        if self._buffer is not None and self._stamp == self.generation:
            return self._buffer
        return None


def checked_temperatures(L, threads, temperatures):
    """The reference's argument checks, in its order and with its messages."""
    if L < 4 or L % 2 != 0:
        raise ValueError("L must be even and >= 4")
    if threads < 1 or threads ** 2 > 1024:
        raise ValueError("Invalid thread configuration")
    t = np.asarray(temperatures, dtype=np.float64)
    if t.ndim != 1 or t.size == 0:
        raise ValueError("Temperatures must be a nonempty 1D array")
    if not np.all(np.isfinite(t) & (t > 0)):
        raise ValueError("Temperatures must be positive and finite")
    return t.copy()


def launch_shape(L, R, threads):
    """The reference's colour-launch shape: (threads, threads) blocks over the
    (L/2, L/2) sites of one colour, one grid layer per replica."""
    tiles = -(-(L // 2) // threads)
    return (threads, threads, 1), (tiles, tiles, R)


class Runtime:
    """State, per-site RNG streams and betas of R replicas of an L x L lattice."""

    def __init__(self, model, L, temperatures, threads=16, seed=42):
        self.temperatures = checked_temperatures(L, threads, temperatures)
        self.model = model
        self.L = L
        self.R = int(self.temperatures.size)
        self.seed = seed

        first = np.asarray(model.initialize_state(L, self.R, seed))
        if first.shape[:3] != (self.R, L, L):
            raise ValueError("Invalid model state shape")
        self.state = to_device(np.ascontiguousarray(first))
        self.rng_states = create_xoroshiro128p_states(self.R * L * L, seed=seed)
        self.betas = to_device((1.0 / self.temperatures).astype(np.float32))
        self.threads_per_block, self.blocks_per_grid = launch_shape(L, self.R, threads)
        self._energy = EnergyCache()
        self._window = None  # the window launch of _enqueue_sweeps, built on first use

    # ------------------------------------------------------------ energies
    def invalidate_energy_cache(self):
        """Forget cached energies: call before changing the state, fields or
        Hamiltonian parameters from outside.  sweep() does it by itself;
        temperature exchanges leave the physical energy unchanged."""
        self._energy.advance()

    def measure_energy(self, output):
        """Total energies in walker order into the caller's device buffer,
        which then serves measure() until the configuration changes."""
        # Withdraw first: a producer that fails part-way must not leave a
        # half-written buffer looking valid.
        self._energy.withdraw()
        result = self.model.measure_energy(self.state, output)
        self._energy.publish(output)
        return result

    # ------------------------------------------------------------ sweeps
    def sweep(self):
        """One sweep: colours 0, 1, 2, 3 of every replica."""
        # The cache goes before any launch is queued, so a sweep that fails
        # to launch never leaves stale energies published.
        self._energy.advance()
        self._enqueue_sweep()
        self._sweeps_done(1)

    def _enqueue_sweep(self):
        """The device work of one sweep: kernel launches on the current
        stream and nothing else (no host state changes), so a captured CUDA
        graph repeats it exactly."""
        fused = getattr(self.model, "enqueue_sweep", None)
        if fused is not None and fused(self.state, self.rng_states, self.betas):
            return
        for colour in range(4):
            self.model.update_color(self.state, self.rng_states, self.betas, colour,
                                    self.blocks_per_grid, self.threads_per_block)

    def _enqueue_sweeps(self, n):
        """The device work of n consecutive sweeps with nothing between them:
        for the built-in Ising plugin and the XY plugin with the reference's
        uniform proposal one window launch with the lattice on chip
        (window_sweeps.py), bit-identical to n sweeps of colour launches;
        otherwise n times _enqueue_sweep."""
        self._prepare_sweeps()
        if self._window:
            self._window.enqueue(n)
            return
        for _ in range(n):
            self._enqueue_sweep()

    def _prepare_sweeps(self):
        """Build the window launch of _enqueue_sweeps (its device tables are
        copied in synchronously, so this must run before any stream capture)."""
        if self._window is None:
            from .window_sweeps import WindowSweeps
            self._window = WindowSweeps.for_runtime(self) or False

    def _sweeps_done(self, n):
        """Host bookkeeping, other than the energy cache, after n sweeps whose
        launches were enqueued (none here; sampler subclasses count sweeps)."""

    # ------------------------------------------------------------ observables
    def measure(self, temperature_indices=None):
        """Host observables, in temperature order when indices are given."""
        cached = self._energy.current()
        if cached is not None:
            return self.model.measure_with_energy(self.state, cached, temperature_indices=temperature_indices)
        return self.model.measure(self.state, temperature_indices=temperature_indices)

    def snapshot(self):
        return self.state.copy_to_host()
