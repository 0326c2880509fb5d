"""Runs of sweeps of the drop-in Runtime as one window launch.

The reference's Runtime sweeps with four colour launches
(core/runtime.py:87-99 over models/ising/update.py:7-29 and
models/xy/update.py:6-54).  For the built-in Ising plugin and the XY plugin
with the reference's uniform proposal, ``n`` sweeps with nothing between them
(the sweeps between two exchanges or samples of a Simulation) run here as one
launch of the batched engine's window kernel on the Runtime's own arrays, in
the reference layout (MCGB_MODEL_ISING_REF / MCGB_MODEL_XY_REF): a
thread-block cluster per replica keeps its strip of the lattice and its RNG
streams on chip for all ``n`` sweeps, and the result is bit-identical to the
``4 n`` colour launches.
"""

from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..batch import REPLICA_DTYPE, BatchWindow, LadderBatch
from ..device import device_zeros, to_device

MODEL_ISING_REF, MODEL_XY_REF = 6, 7
# The reference-layout windows hold at most this many plaquettes of a colour
# per CTA: one per thread of a 1024-thread CTA (the shared-memory stream
# variant).
MAX_PLAQUETTES = 1024
# Sweeps of one window launch (the library takes up to 2^24); longer runs
# take several launches, which continue the chain bit for bit.
MAX_LAUNCH_SWEEPS = 1 << 20


def _shape(L):
    """(cluster_size, threads) for a replica of size L: the fewest CTAs whose
    strips hold at most MAX_PLAQUETTES plaquettes of a colour, one plaquette
    per thread; None when no cluster of up to 16 CTAs does."""
    for C in (1, 2, 4, 8, 16):
        Ce = LadderBatch.effective_cluster(L, C)
        npl = (L // 2) * (L // 2) // Ce
        if npl <= MAX_PLAQUETTES:
            return C, max(64, -(-npl // 32) * 32)
    return None


class WindowSweeps:
    """The window launch of a Runtime: its replica table, cluster work lists
    and the per-replica scratch the window kernel writes (running energies,
    acceptance counts), allocated once."""

    def __init__(self, runtime, model_id, C, T, n_clusters):
        R, L = runtime.R, runtime.L
        self.runtime, self.model_id = runtime, model_id
        self.cluster_size, self.threads, self.n_clusters = C, T, n_clusters
        rows = [(L, r, r, 1, r * L * L) for r in range(R)]
        self.table_host = np.array(rows, dtype=REPLICA_DTYPE)
        self.table = to_device(self.table_host)
        # Replicas are alike: cluster k runs replicas k, k + n_clusters, ...
        lists = [list(range(k, R, n_clusters)) for k in range(n_clusters)]
        ptrs = np.zeros(n_clusters + 1, np.int32)
        ptrs[1:] = np.cumsum([len(x) for x in lists])
        self.work_ptr = to_device(ptrs)
        self.work_idx = to_device(np.array([r for x in lists for r in x], np.int32))
        self.w2t = device_zeros(R, np.int32)
        self.e_run = device_zeros(2 * R, np.float32)
        self.energies = device_zeros(R, np.float64)
        self.accepted = device_zeros(R, np.int64)
        self.clock = device_zeros(2, np.int64)

    @classmethod
    def for_runtime(cls, runtime):
        """The window launch for this Runtime, or None when its sweeps are not
        the reference's Ising or uniform-proposal XY update of the built-in
        plugin class (a subclass, a replaced method, Gaussian proposals) or
        its lattice needs more than 16 CTAs a replica."""
        from ..models.ising.model import IsingModel
        from ..models.xy.model import XYModel
        from .runtime import Runtime
        model = runtime.model
        if type(model) is IsingModel:
            model_id = MODEL_ISING_REF
        elif type(model) is XYModel and model.proposal == "uniform":
            model_id = MODEL_XY_REF
        else:
            return None
        if "update_color" in vars(model) or "enqueue_sweep" in vars(model):
            return None
        if type(runtime)._enqueue_sweep is not Runtime._enqueue_sweep or "_enqueue_sweep" in vars(runtime):
            return None
        shape = _shape(runtime.L)
        if shape is None:
            return None
        C, T = shape
        lib = _lib.load()
        smem = int(lib.mcgb_batch_smem_bytes(model_id, int(runtime.L), C))
        if smem < 0:
            return None
        n = ctypes.c_int(0)
        if lib.mcgb_batch_max_clusters(model_id, C, T, smem, ctypes.byref(n)) != 0 or n.value < 1:
            return None
        return cls(runtime, model_id, C, T, min(runtime.R, n.value))

    def enqueue(self, n_sweeps):
        """n_sweeps sweeps of every replica on the current stream: one launch,
        or one per MAX_LAUNCH_SWEEPS sweeps of a longer run."""
        n_sweeps = int(n_sweeps)
        while n_sweeps > 0:
            n = min(n_sweeps, MAX_LAUNCH_SWEEPS)
            self._launch(n)
            n_sweeps -= n

    def _launch(self, n_sweeps):
        rt = self.runtime
        w = BatchWindow()
        w.table, w.host_table, w.n_replicas = self.table.ptr, self.table_host.ctypes.data, rt.R
        w.work_ptr, w.work_idx = self.work_ptr.ptr, self.work_idx.ptr
        w.n_clusters, w.cluster_size, w.threads = self.n_clusters, self.cluster_size, self.threads
        w.state, w.rng, w.betas, w.w2t = rt.state.ptr, rt.rng_states.ptr, rt.betas.ptr, self.w2t.ptr
        w.e_run, w.energies, w.accepted = self.e_run.ptr, self.energies.ptr, self.accepted.ptr
        w.clock = self.clock.ptr
        w.n_sweeps = int(n_sweeps)
        w.J = float(rt.model.J)
        w.delta = float(getattr(rt.model, "delta", 0.0))
        _lib.call("mcgb_batch_window_run", self.model_id, ctypes.byref(w), _lib.stream_handle())
