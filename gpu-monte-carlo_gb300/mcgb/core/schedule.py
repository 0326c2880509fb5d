"""The sweep / exchange / sample schedule of a Simulation run, and its replay
as captured CUDA graphs.

A run of the reference's host loop (core/simulation.py:39-78 over
core/parallel_tempering.py:245-269) is, sweep by sweep, a fixed sequence of
device work: the colour launches of one sweep; every ``exchange_interval``
sweeps (counted from the ParallelTempering's creation) a total-energy
reduction and one exchange round, and every ``history_stride`` rounds a
walker-history row; every ``sample_interval`` measured sweeps a measurement
in temperature order (from the round's energies when the sweep ended with an
exchange).  ``plan`` cuts that sequence into segments ending at each event,
run-length encoded; ``GraphReplay`` captures each distinct segment (several
copies of it per graph) once and replays it, with the two things that vary
between copies kept on the device: the exchange schedule (a clock {sweeps,
rounds} that mcgb_pt_exchange_clocked reads and advances) and the sample and
history slots (rings whose head counters mcgb_ring_push and
mcgb_pt_record_walkers_ring advance).  The kernels are the ones the
step-by-step loop launches, in the same order, so the chain, the counters and
every sample are bit-identical to it; what goes away is a Python call and a
synchronising host copy per sample and the per-launch host overhead.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from .. import _lib
from ..device import device_array, device_zeros, ptr, to_device

# Copies of one segment per captured graph: 1, 2, 4, ... up to this.
MAX_COPIES = 64
# A chunk used once is captured only if it holds about this many launches.
MIN_GRAPH_WORK = 64


@dataclass(frozen=True)
class Segment:
    sweeps: int            # sweeps in the segment, >= 1
    exchange: bool = False  # an exchange round after its last sweep
    advance: int = 0       # sweeps since the previous round (when exchange)
    record: bool = False   # a walker-history row after that round
    sample: bool = False   # a sample after its last sweep (and round)


@dataclass
class Plan:
    runs: list = field(default_factory=list)           # [(Segment, count)]
    n_sweeps: int = 0
    n_rounds: int = 0
    sample_sweeps: list = field(default_factory=list)  # cumulative sweep of each sample
    history: list = field(default_factory=list)        # (sweep, round) of each history row
    ends_with_exchange: bool = False


def plan(thermalization, measurement, sample_interval, interval=None, start_sweeps=0, start_rounds=0,
         history_stride=None):
    """The schedule of ``thermalization + measurement`` sweeps.

    ``interval`` None: no exchanges (a bare Runtime).  Exchange rounds happen
    after sweeps whose count since the ParallelTempering's creation
    (``start_sweeps`` + k) is a multiple of ``interval``; history rows after
    rounds whose count is a multiple of ``history_stride`` (None: none).
    """
    p = Plan()
    total = thermalization + measurement
    rounds, last_exchange, length = start_rounds, start_sweeps, 0
    for k in range(1, total + 1):
        g = start_sweeps + k
        length += 1
        exchange = interval is not None and g % interval == 0
        record = False
        if exchange:
            rounds += 1
            record = history_stride is not None and rounds % history_stride == 0
            if record:
                p.history.append((g, rounds))
        sample = k > thermalization and (k - thermalization) % sample_interval == 0
        if sample:
            p.sample_sweeps.append(k)
        if exchange or sample or k == total:
            seg = Segment(length, exchange, g - last_exchange if exchange else 0, record, sample)
            if p.runs and p.runs[-1][0] == seg:
                p.runs[-1] = (seg, p.runs[-1][1] + 1)
            else:
                p.runs.append((seg, 1))
            length = 0
            if exchange:
                last_exchange = g
        p.ends_with_exchange = exchange
    p.n_sweeps = total
    p.n_rounds = rounds - start_rounds
    return p


def chunks(count):
    """Split ``count`` copies into graph sizes 64, 32, ..., 1."""
    out = []
    while count:
        c = 1 << min(MAX_COPIES.bit_length() - 1, count.bit_length() - 1)
        out.append(c)
        count -= c
    return out


def _defined_in(cls, name):
    for klass in cls.__mro__:
        if name in vars(klass):
            return klass
    return None


class GraphReplay:
    """Runs a Plan for a Runtime or a ParallelTempering over one."""

    def __init__(self, runtime):
        from .parallel_tempering import ParallelTempering
        self.pt = runtime if isinstance(runtime, ParallelTempering) else None
        self.rt = self.pt.runtime if self.pt is not None else runtime

    @staticmethod
    def supports(runtime):
        """Whether every launch of the schedule is known to be pure device
        work: a built-in model plugin (exactly its class), a Runtime whose
        sweep has a matching launch-only form, and the library's own
        ParallelTempering.  Anything else -- user subclasses included --
        runs step by step through its own Python methods."""
        from ..models.he3.model import He3Model
        from ..models.ising.model import IsingModel
        from ..models.kawamura.model import KawamuraModel
        from ..models.xy.model import XYModel
        from .parallel_tempering import ParallelTempering
        from .runtime import Runtime
        pt = runtime if isinstance(runtime, ParallelTempering) else None
        if pt is not None and type(pt) is not ParallelTempering:
            return False
        rt = pt.runtime if pt is not None else runtime
        if not isinstance(rt, Runtime):
            return False
        if type(rt.model) not in (IsingModel, XYModel, KawamuraModel, He3Model):
            return False
        cls = type(rt)
        if not issubclass(_defined_in(cls, "_enqueue_sweep"), _defined_in(cls, "sweep")):
            return False
        if not all(_defined_in(cls, m) is Runtime for m in ("measure", "measure_energy", "invalidate_energy_cache")):
            return False
        # Methods replaced on an instance (a wrapper, a test double) are the
        # caller's code too.
        replaced = {"sweep", "measure", "measure_energy", "invalidate_energy_cache", "_enqueue_sweep",
                    "attempt_exchanges", "update_color", "measure_into", "measure_with_energy", "enqueue_sweep"}
        return not any(replaced & set(vars(obj)) for obj in (pt, rt, rt.model) if obj is not None)

    # ------------------------------------------------------------ device work
    def _enqueue(self, seg, ctx):
        rt, pt = self.rt, self.pt
        rt._enqueue_sweeps(seg.sweeps)
        if seg.exchange:
            pt._enqueue_exchange(ctx["clock"], seg.advance)
            if seg.record:
                pt._enqueue_history(ctx["history"], ctx["history_head"])
        if seg.sample:
            order = pt.walker_to_temperature if pt is not None else None
            cached = pt.energies if (pt is not None and seg.exchange) else None
            rt.model.measure_into(rt.state, ctx["staging"], order, cached)
            ring = ctx["ring"]
            _lib.call("mcgb_ring_push", ptr(ctx["staging"]), ptr(ring), ptr(ctx["head"]),
                      int(ctx["staging"].size), int(ring.shape[0]), _lib.stream_handle())

    def run(self, p):
        """Enqueue the whole plan, account for it on the host, and return the
        samples {channel: (n_samples, R) float64} in temperature order."""
        rt, pt = self.rt, self.pt
        rt._prepare_sweeps()  # device tables of the sweep launch, before any capture
        names = tuple(rt.model.measurement_names)
        C, R = len(names), rt.R
        n_samples = len(p.sample_sweeps)
        ctx = {"staging": device_array((C, R), np.float64),
               "ring": device_array((max(n_samples, 1), C, R), np.float64),
               "head": device_zeros(1, np.int64)}
        if pt is not None:
            ctx["clock"] = to_device(np.array([pt.sweeps, pt.exchange_rounds], np.int64))
            if p.history:
                ctx["history"] = device_array((len(p.history), len(pt._tracked_walkers)), np.int32)
                ctx["history_head"] = device_zeros(1, np.int64)

        # A chunk of segments is captured once and replayed when its shape
        # repeats or when it alone holds enough launches to repay a capture
        # (a device synchronisation); small one-off chunks launch directly.
        uses = {}
        for seg, count in p.runs:
            for c in chunks(count):
                uses[(seg, c)] = uses.get((seg, c), 0) + 1
        graphs = {}
        for seg, count in p.runs:
            for c in chunks(count):
                key = (seg, c)
                if uses[key] < 2 and c * (seg.sweeps + 2) < MIN_GRAPH_WORK:
                    for _ in range(c):
                        self._enqueue(seg, ctx)
                    continue
                g = graphs.get(key)
                if g is None:
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g):
                        for _ in range(c):
                            self._enqueue(seg, ctx)
                    graphs[key] = g
                g.replay()

        # Host bookkeeping of everything the device ran.
        rt._energy.advance()
        rt._sweeps_done(p.n_sweeps)
        if pt is not None:
            rows = [ctx["history"][k] for k in range(len(p.history))] if p.history else None
            pt._rounds_done(p.n_sweeps, p.n_rounds, rows, p.history)
            if p.ends_with_exchange:
                rt._energy.publish(pt.energies)
        data = ctx["ring"].copy_to_host()[:n_samples]
        return {name: data[:, c, :].copy() for c, name in enumerate(names)}
