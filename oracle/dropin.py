"""CPU replay of the reference's host control flow on the oracle's kernels --
test infrastructure only (the checker; nothing in the product imports it).

Restates, with the oracle's C kernels standing in for the Numba launches:

* ``core/runtime.py:87-99`` -- a sweep is colours 0, 1, 2, 3 of every
  replica; ``:70-132`` -- the energy cache: ``measure_energy`` makes it valid,
  the next sweep invalidates it, and ``measure`` takes the cached energies
  while it is valid;
* ``core/parallel_tempering.py:245-269`` -- a sweep, then every
  ``exchange_interval`` sweeps a total-energy reduction and one exchange
  round (``:35-91``, ``orc_pt_exchange``) at the current parity, which
  alternates when R > 2; exchange streams seeded with ``seed + 1`` (``:165``,
  ``:177-179``); walker history every ``history_stride`` rounds (``:206-243``);
* ``core/simulation.py:28-96`` -- thermalisation sweeps, then a measurement
  in temperature order every ``sample_interval`` sweeps.

Model kinds: ``ising`` (acceptance exponentials from a table of CUDA's
``expf`` values, keyed by the float32 argument bits), ``xy``, ``kawamura``,
``he3`` and ``he3g`` (the conditional-Gaussian sampler).
"""

from __future__ import annotations

import numpy as np

from . import (he3_energy, he3_gaussian_update_color, he3_measure, he3_update_color, ising_energy,
               ising_exponent_arguments, ising_measure, ising_sweeps_tab, kawamura_energy, kawamura_measure,
               kawamura_update_color, pt_exchange, pt_initial_trips, rng_states, xy_energy, xy_measure,
               xy_update_color)

CHANNELS = {
    "ising": ("energy", "magnetization"),
    "xy": ("energy", "mx", "my", "twist_cos_x", "twist_sin_x"),
    "kawamura": ("energy", "chirality", "px", "py", "spin2", "twist_cos_x", "twist_sin_x"),
    "he3": ("energy", "density", "chirality", "phase_real", "phase_imag", "current_x", "curvature_x",
            "current_y", "curvature_y", "spin_alignment"),
}


class ModelOps:
    """One model's sweep / energy / measure on the oracle."""

    def __init__(self, kind, params, expf_table=None):
        self.kind, self.p = kind, dict(params)
        self.expf = expf_table or {}
        self.counts = None

    @property
    def channels(self):
        return CHANNELS["he3" if self.kind == "he3g" else self.kind]

    def _ising_table(self, betas):
        args = ising_exponent_arguments(betas, self.p["J"]).view(np.uint32)
        rows = np.empty(args.shape, np.uint32)
        for idx, bits in np.ndenumerate(args):
            if int(bits) not in self.expf:
                raise KeyError(f"no CUDA expf value recorded for argument {int(bits):08x}")
            rows[idx] = self.expf[int(bits)]
        return rows.view(np.float32)

    def sweep(self, state, rng, betas):
        p, k = self.p, self.kind
        if k == "ising":
            ising_sweeps_tab(state, rng, betas, self._ising_table(betas), p["J"], 1)
            return
        for color in range(4):
            if k == "xy":
                xy_update_color(state, rng, betas, color, p["J"], p["delta"])
            elif k == "kawamura":
                kawamura_update_color(state, rng, betas, color, p["J"], p["delta"])
            elif k == "he3":
                he3_update_color(state, rng, betas, color, p["coefficients"], p["K"], p["delta"], p["g_d"])
            elif k == "he3g":
                if self.counts is None:
                    R, L = state.shape[0], state.shape[1]
                    self.counts = np.zeros((3, R, L, L), np.int64)
                he3_gaussian_update_color(state, rng, betas, color, p["coefficients"], p["K"], p["rho"],
                                          p["mass"], p["g_d"], self.counts)
            else:
                raise ValueError(k)

    def energy(self, state):
        p, k = self.p, self.kind
        if k == "ising":
            return ising_energy(state, p["J"])
        if k == "xy":
            return xy_energy(state, p["J"])
        if k == "kawamura":
            return kawamura_energy(state, p["J"])
        return he3_energy(state, p["coefficients"], p["K"], p["g_d"])

    def measure(self, state, temperature_indices=None, cached=None):
        p, k = self.p, self.kind
        if k == "ising":
            out = ising_measure(state, p["J"], temperature_indices, cached)
        elif k == "xy":
            out = xy_measure(state, p["J"], temperature_indices, cached)
        elif k == "kawamura":
            out = kawamura_measure(state, p["J"], temperature_indices, cached)
        else:
            out = he3_measure(state, p["coefficients"], p["K"], p["g_d"], temperature_indices, cached)
        return dict(zip(self.channels, out))


class Runtime:
    """State, per-site streams, float32 betas and the energy cache of one ladder."""

    def __init__(self, ops, state, temperatures, seed):
        self.ops = ops
        self.state = np.ascontiguousarray(state).copy()
        self.R, self.L = self.state.shape[0], self.state.shape[1]
        self.temperatures = np.asarray(temperatures, np.float64)
        self.seed = seed
        self.rng = rng_states(self.R * self.L * self.L, seed)
        self.betas = (1.0 / self.temperatures).astype(np.float32)
        self.cached = None

    def sweep(self):
        self.cached = None
        self.ops.sweep(self.state, self.rng, self.betas)

    def measure_energy(self):
        self.cached = self.ops.energy(self.state)
        return self.cached

    def measure(self, temperature_indices=None):
        return self.ops.measure(self.state, temperature_indices, self.cached)


class ParallelTempering:
    """Replica exchange over a Runtime with the reference's schedule."""

    def __init__(self, runtime, exchange_interval=10, seed=None, tracked_walkers=None, history_stride=10):
        rt = self.runtime = runtime
        self.R, self.interval = rt.R, exchange_interval
        self.exchange_seed = rt.seed + 1 if seed is None else seed
        self.sweeps = self.exchange_rounds = self.parity = 0
        self.energies = rt.measure_energy()
        self.w2t = np.arange(self.R, dtype=np.int32)
        self.t2w = np.arange(self.R, dtype=np.int32)
        self.rng = rng_states(self.R - 1, self.exchange_seed)
        self.swap_counts = np.zeros((3, self.R - 1), np.int64)
        self.trips = pt_initial_trips(self.R)
        self.tracked = None if tracked_walkers is None else np.asarray(tracked_walkers, np.int32)
        self.stride = history_stride
        self.history, self.history_sweeps, self.history_rounds = [], [], []
        if self.tracked is not None:
            self._record()

    def _record(self):
        self.history.append(self.w2t[self.tracked].copy())
        self.history_sweeps.append(self.sweeps)
        self.history_rounds.append(self.exchange_rounds)

    def sweep(self):
        self.runtime.sweep()
        self.sweeps += 1
        if self.sweeps % self.interval == 0:
            self.attempt_exchanges()

    def attempt_exchanges(self):
        self.energies = self.runtime.measure_energy()
        pt_exchange(self.energies, self.runtime.betas, self.w2t, self.t2w, self.rng, self.swap_counts,
                    self.trips, self.parity, self.sweeps)
        self.exchange_rounds += 1
        if self.R > 2:
            self.parity = 1 - self.parity
        if self.tracked is not None and self.exchange_rounds % self.stride == 0:
            self._record()

    def measure(self):
        return self.runtime.measure(self.w2t)

    def walker_history(self):
        rows = list(self.history)
        sweeps, rounds = list(self.history_sweeps), list(self.history_rounds)
        if rounds[-1] != self.exchange_rounds or sweeps[-1] != self.sweeps:
            rows.append(self.w2t[self.tracked].copy())
            sweeps.append(self.sweeps)
            rounds.append(self.exchange_rounds)
        return {"walker_ids": self.tracked.copy(), "sweeps": np.asarray(sweeps, np.int64),
                "exchange_rounds": np.asarray(rounds, np.int64), "temperature_indices": np.stack(rows)}


def simulate(pt, thermalization_sweeps, measurement_sweeps, sample_interval):
    """core/simulation.py:28-96: samples per channel (n_samples, R) and the sample sweeps."""
    for _ in range(thermalization_sweeps):
        pt.sweep()
    samples, sweeps = {}, []
    for step in range(1, measurement_sweeps + 1):
        pt.sweep()
        if step % sample_interval:
            continue
        for name, v in pt.measure().items():
            samples.setdefault(name, []).append(np.asarray(v).copy())
        sweeps.append(thermalization_sweeps + step)
    return {k: np.stack(v) for k, v in samples.items()}, np.asarray(sweeps)
