"""Thermalise, then sample every ``sample_interval`` sweeps.

Drop-in for the reference's ``Simulation`` (core/simulation.py:5-96).  The
contract kept from it: the constructor and its ValueError conditions and
messages (:14-21); the schedule (``thermalization_sweeps`` sweeps, then a
measurement after every ``sample_interval``-th of ``measurement_sweeps``
sweeps, through the runtime's ``sweep``/``measure``); and the result
``{"samples": {channel: (n_samples, R)}, "metadata": {...}}`` with the run
settings, ``sample_sweeps`` and, for a ParallelTempering runtime, its
diagnostics.  The model's channel checks (:48-66) hold for runtimes run step
by step.

How it runs is this project's: for the built-in models (and the library's
own Runtime / ParallelTempering / He3GaussianRuntime) the whole schedule is
planned up front and replayed as captured CUDA graphs with a device-side
sample ring (``schedule.GraphReplay``): the same kernels in the same order,
so the samples are bit-identical to a step-by-step run, with one host copy
of all samples at the end instead of a synchronising copy and a Python
append per sample.  Any other runtime or model runs step by step.  Setting
``replay = False`` on an instance forces the step-by-step loop.
"""

import numpy as np

from .parallel_tempering import ParallelTempering
from .schedule import GraphReplay, plan


def _checked_schedule(thermalization_sweeps, measurement_sweeps, sample_interval):
    if thermalization_sweeps < 0:
        raise ValueError("Thermalization sweeps cannot be negative")
    if measurement_sweeps < 1:
        raise ValueError("Measurement sweeps must be positive")
    if sample_interval < 1 or sample_interval > measurement_sweeps:
        raise ValueError("Invalid sampling interval")


class _SampleTable:
    """Per-channel sample lists with the reference's consistency checks."""

    def __init__(self, R):
        self.R = R
        self.columns = None

    def add(self, measurement):
        if not measurement:
            raise ValueError("Model returned no measurements")
        if self.columns is None:
            self.columns = {name: [] for name in measurement}
        if measurement.keys() != self.columns.keys():
            raise ValueError("Measurement channels changed")
        for name, value in measurement.items():
            value = np.asarray(value)
            if value.ndim < 1 or value.shape[0] != self.R:
                raise ValueError(f"Invalid replica dimension for {name}")
            self.columns[name].append(value.copy())

    def stacked(self):
        return {name: np.stack(rows, axis=0) for name, rows in (self.columns or {}).items()}


class Simulation:

    def __init__(self, runtime, thermalization_sweeps=1000, measurement_sweeps=4000, sample_interval=10):
        _checked_schedule(thermalization_sweeps, measurement_sweeps, sample_interval)
        self.runtime = runtime
        self.thermalization_sweeps = thermalization_sweeps
        self.measurement_sweeps = measurement_sweeps
        self.sample_interval = sample_interval
        self.replay = True

    def _plan(self):
        rt = self.runtime
        if isinstance(rt, ParallelTempering):
            stride = rt._history_stride if rt._tracked_walkers is not None else None
            return plan(self.thermalization_sweeps, self.measurement_sweeps, self.sample_interval,
                        rt.exchange_interval, rt.sweeps, rt.exchange_rounds, stride)
        return plan(self.thermalization_sweeps, self.measurement_sweeps, self.sample_interval)

    def _step_by_step(self, sample_sweeps):
        rt = self.runtime
        table = _SampleTable(rt.R)
        for _ in range(self.thermalization_sweeps):
            rt.sweep()
        due = iter(sample_sweeps)
        next_due = next(due, None)
        for k in range(1, self.measurement_sweeps + 1):
            rt.sweep()
            if self.thermalization_sweeps + k == next_due:
                table.add(rt.measure())
                next_due = next(due, None)
        return table.stacked()

    def run(self):
        rt = self.runtime
        schedule = self._plan()
        if self.replay and GraphReplay.supports(rt):
            samples = GraphReplay(rt).run(schedule)
        else:
            samples = self._step_by_step(schedule.sample_sweeps)
        metadata = {
            "L": rt.L,
            "temperatures": rt.temperatures.copy(),
            "seed": rt.seed,
            "model_parameters": rt.model.parameters(),
            "thermalization_sweeps": self.thermalization_sweeps,
            "measurement_sweeps": self.measurement_sweeps,
            "sample_interval": self.sample_interval,
            "sample_sweeps": np.asarray(schedule.sample_sweeps),
        }
        if isinstance(rt, ParallelTempering):
            metadata["parallel_tempering"] = rt.diagnostics()
        return {"samples": samples, "metadata": metadata}
