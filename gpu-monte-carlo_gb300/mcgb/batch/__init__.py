"""Batched ladder engine: every replica of every ladder in one launch per window.

The reference runs one ``Runtime`` per (L, temperature ladder), four kernel
launches per sweep, an energy reduction and an exchange kernel every
``exchange_interval`` sweeps and a measurement kernel plus a host copy per
sample (core/runtime.py:87-99, core/parallel_tempering.py:245-273,
core/simulation.py:28-96).  :class:`LadderBatch` runs the same schedule for a
table of replicas of any mix of L: one launch per window of
``exchange_interval`` sweeps (a thread-block cluster per replica, state in
shared memory, RNG in registers) that also decides the replica exchange pair
by pair and ticks the clock -- or one resident launch of many such windows
-- captured as a CUDA graph and replayed; samples accumulate in a device
buffer that is copied once.  A batch of several sizes may run one launch per
size group, each with its own cluster shape (:meth:`LadderBatch.split_by_size`,
chosen by :meth:`LadderBatch.autotune` when faster).

Replica (L, ladder k, slot t) keeps the RNG stream that a ``Runtime`` of that
ladder with seed ``seeds[k]`` gives the same site, so an Ising batch is
bit-identical to the per-colour path; the exchange streams of ladder k equal
``ParallelTempering``'s with ``exchange_seeds[k]``.
"""

from __future__ import annotations

import ctypes
import heapq

import numpy as np
import torch

from .. import _lib
from ..device import XOROSHIRO128P_DTYPE, DeviceArray, device_zeros, ptr, to_device
from ..rng import create_xoroshiro128p_states

REPLICA_DTYPE = np.dtype([("L", "<i4"), ("ladder", "<i4"), ("ladder_start", "<i4"),
                          ("n_temps", "<i4"), ("state_offset", "<i8")])

MODEL_ISING, MODEL_XY, MODEL_KAWAMURA, MODEL_HE3, MODEL_HE3_GAUSS, MODEL_KAWAMURA_GAUSS = range(6)

CHANNELS = {
    MODEL_ISING: ("energy", "magnetization"),
    MODEL_XY: ("energy", "mx", "my", "twist_cos_x", "twist_sin_x"),
    MODEL_KAWAMURA: ("energy", "chirality", "px", "py", "spin2", "twist_cos_x", "twist_sin_x"),
    MODEL_HE3: ("energy", "density", "chirality", "phase_real", "phase_imag",
                "current_x", "curvature_x", "current_y", "curvature_y", "spin_alignment"),
}
CHANNELS[MODEL_HE3_GAUSS] = CHANNELS[MODEL_HE3]
CHANNELS[MODEL_KAWAMURA_GAUSS] = CHANNELS[MODEL_KAWAMURA]
# Sweeps per window of a batch without replica exchange: nothing happens
# between its windows but the clock tick, so long windows spare the strip
# reload, write-back and launch of each short one.
NO_EXCHANGE_WINDOW = 100

# Models whose proposals have per-temperature widths sigma_t.
GAUSSIAN_WIDTHS = (MODEL_XY, MODEL_KAWAMURA_GAUSS)


class BatchWindow(ctypes.Structure):
    """ctypes mirror of ``mcgb_batch_window`` (include/mcgb.h)."""

    _fields_ = [
        ("table", ctypes.c_void_p), ("host_table", ctypes.c_void_p), ("n_replicas", ctypes.c_int32),
        ("work_ptr", ctypes.c_void_p), ("work_idx", ctypes.c_void_p),
        ("n_clusters", ctypes.c_int32), ("cluster_size", ctypes.c_int32), ("threads", ctypes.c_int32),
        ("state", ctypes.c_void_p), ("rng", ctypes.c_void_p), ("aux", ctypes.c_void_p),
        ("betas", ctypes.c_void_p),
        ("w2t", ctypes.c_void_p), ("e_run", ctypes.c_void_p), ("energies", ctypes.c_void_p),
        ("accepted", ctypes.c_void_p), ("counters", ctypes.c_void_p), ("samples", ctypes.c_void_p),
        ("staging", ctypes.c_void_p),
        ("n_temps_total", ctypes.c_int32), ("n_slots", ctypes.c_int32),
        ("clock", ctypes.c_void_p), ("first_sample_sweep", ctypes.c_int64),
        ("sample_interval", ctypes.c_int32), ("n_sweeps", ctypes.c_int32),
        ("J", ctypes.c_float), ("delta", ctypes.c_float), ("sigma_t", ctypes.c_void_p),
        ("coefficients", ctypes.c_float * 5), ("K", ctypes.c_float), ("g_d", ctypes.c_float),
        ("rho", ctypes.c_float), ("mass", ctypes.c_float),
        ("host_work_idx", ctypes.c_void_p), ("n_work", ctypes.c_int32), ("hold_clock", ctypes.c_int32),
    ]


class BatchPT(ctypes.Structure):
    """ctypes mirror of ``mcgb_batch_pt``."""

    _fields_ = [
        ("t2w", ctypes.c_void_p), ("rng", ctypes.c_void_p), ("swap_counts", ctypes.c_void_p),
        ("trips", ctypes.c_void_p), ("ladder_starts", ctypes.c_void_p), ("ladder_sizes", ctypes.c_void_p),
        ("n_ladders", ctypes.c_int32), ("channels", ctypes.c_int32),
    ]


def _model_info(model, gaussian, proposal="uniform"):
    from ..models.he3.model import He3Model
    from ..models.ising.model import IsingModel
    from ..models.kawamura.model import KawamuraModel
    from ..models.xy.model import XYModel

    if isinstance(model, IsingModel):
        return MODEL_ISING, np.dtype(np.int8), ()
    if isinstance(model, XYModel):
        return MODEL_XY, np.dtype(np.float32), ()
    if isinstance(model, KawamuraModel):
        return (MODEL_KAWAMURA_GAUSS if proposal == "gaussian" else MODEL_KAWAMURA), np.dtype(np.float32), (5,)
    if isinstance(model, He3Model):
        return (MODEL_HE3_GAUSS if gaussian else MODEL_HE3), np.dtype(np.complex64), (3, 2)
    raise TypeError(f"unsupported model {type(model).__name__}")


def lpt_work_lists(costs, n_clusters):
    """Longest-processing-time assignment of replicas to clusters (CSR lists)."""
    order = np.argsort(-np.asarray(costs, dtype=np.float64), kind="stable")
    heap = [(0.0, k) for k in range(n_clusters)]
    lists = [[] for _ in range(n_clusters)]
    for r in order:
        load, k = heapq.heappop(heap)
        lists[k].append(int(r))
        heapq.heappush(heap, (load + float(costs[r]), k))
    ptrs = np.zeros(n_clusters + 1, dtype=np.int32)
    ptrs[1:] = np.cumsum([len(x) for x in lists])
    idx = np.asarray([r for x in lists for r in x], dtype=np.int32)
    loads = np.zeros(n_clusters)
    for k, x in enumerate(lists):
        loads[k] = sum(costs[r] for r in x)
    return ptrs, idx, loads


def side_by_side_pick(rows):
    """Which option of each group to run when the groups of a window run side
    by side.  rows[k] lists group k's options as (ms, occupancy, ...): its
    time alone and the GPU time it takes (ms times the fraction of the GPU it
    holds).  The window takes at least its longest group and at least the
    summed occupancy; coordinate descent over the groups minimises the larger
    of the two, starting from each group's first (fastest) option.  Returns
    the chosen index per group."""
    pick = [0] * len(rows)

    def cost(sel):
        return max(max(rows[k][i][0] for k, i in enumerate(sel)), sum(rows[k][i][1] for k, i in enumerate(sel)))

    for _ in range(8):
        changed = False
        for k in range(len(rows)):
            best = min(range(len(rows[k])), key=lambda i: cost(pick[:k] + [i] + pick[k + 1:]))
            if cost(pick[:k] + [best] + pick[k + 1:]) < cost(pick) - 1e-9:
                pick[k], changed = best, True
        if not changed:
            break
    return pick


def visit_costs(Ls, C, T):
    """Relative time a cluster of C CTAs x T threads spends on each replica of
    sizes Ls, for its work lists: the visits a thread makes per colour phase
    (the strip's plaquettes over the threads, rounded up -- a strip smaller
    than the block leaves threads idle, so a small lattice costs more than
    its share of sites) plus a fixed share for the strip load, write-back
    and exchange."""
    npl = np.array([int(L) ** 2 // (4 * LadderBatch.effective_cluster(L, C)) for L in Ls], dtype=np.float64)
    return np.ceil(npl / int(T)) + 0.5


class _Group:
    """Replicas that share one cluster shape: one launch per window (or one
    resident launch of many windows) runs them.  A ladder has one lattice
    size, so grouping by size never splits a ladder."""

    def __init__(self, idx):
        self.idx = np.asarray(idx, dtype=np.int64)
        self.cluster_size = self.threads = self.n_clusters = 0
        self.work_ptr = self.work_idx = self.work_host = None
        self.resident = False
        # Concurrent groups: the group's stream, its copy of the clock and
        # its own exchange bookkeeping (mailboxes, decision words, launch
        # counter, error flag).
        self.stream = self.clock = self.sync = None


def _validate_ladder(L, temperatures, pt):
    if L < 4 or L % 2:
        raise ValueError("L must be even and >= 4")
    t = np.asarray(temperatures, dtype=np.float64)
    if t.ndim != 1 or len(t) == 0:
        raise ValueError("Temperatures must be a nonempty 1D array")
    if not np.all(np.isfinite(t) & (t > 0)):
        raise ValueError("Temperatures must be positive and finite")
    if pt:
        if len(t) < 2:
            raise ValueError("Parallel tempering requires at least two temperatures")
        b = (1.0 / t).astype(np.float32)
        if not np.all(np.diff(b) < 0):
            raise ValueError("PT temperatures must have distinct, finite positive float32 betas")
    return t


class LadderBatch:
    """Replicas of one model over ladders ``[(L, temperatures), ...]``.

    Parameters mirror the drop-in classes: per-ladder ``seeds`` (site RNG,
    default ``42 + L``, made distinct per ladder) and ``exchange_seeds``
    (default ``seed + 1``); ``exchange_interval=None`` disables replica
    exchange.  ``proposal`` selects the XY move ("uniform" or "gaussian" with
    per-temperature widths starting at ``sigma0``); ``gaussian`` selects the
    He3 conditional Gaussian sampler.
    """

    def __init__(self, model, ladders, seeds=None, exchange_interval=10, exchange_seeds=None,
                 proposal="uniform", sigma0=1.0, gaussian=False, rho=-0.9, proposal_mass=0.0,
                 cluster_size=None, threads=None, initial_states=None, resident=True):
        self.model = model
        self._resident_wanted = bool(resident)
        self._resident_checked = False
        # Size groups launched side by side on streams of their own (set by
        # split_by_size or autotune); otherwise one after another.
        self.concurrent = False
        self.model_id, self.dtype, self.site_shape = _model_info(model, gaussian, proposal)
        self.channels = CHANNELS[self.model_id]
        self.pt = exchange_interval is not None
        if self.pt and (isinstance(exchange_interval, bool) or int(exchange_interval) != exchange_interval
                        or exchange_interval < 1):
            raise ValueError("exchange_interval must be a positive integer")
        self.exchange_interval = int(exchange_interval) if self.pt else None
        self.ladders = [(int(L), _validate_ladder(int(L), T, self.pt)) for L, T in ladders]
        if not self.ladders:
            raise ValueError("need at least one ladder")
        n_l = len(self.ladders)
        if seeds is None:
            seen = {}
            seeds = []
            for L, _ in self.ladders:
                k = seen.get(L, 0)
                seen[L] = k + 1
                seeds.append(42 + L + 100003 * k)
        self.seeds = [int(s) for s in seeds]
        if len(self.seeds) != n_l:
            raise ValueError("one seed per ladder")
        self.exchange_seeds = ([s + 1 for s in self.seeds] if exchange_seeds is None
                               else [int(s) for s in exchange_seeds])
        self.proposal = proposal
        if proposal not in ("uniform", "gaussian"):
            raise ValueError("proposal must be 'uniform' or 'gaussian'")
        if proposal == "gaussian" and self.model_id not in GAUSSIAN_WIDTHS:
            raise ValueError("Gaussian widths apply to the XY and Kawamura models "
                             "(He3 selects its sampler with gaussian=True)")

        # ---------------------------------------------------------- replica table
        rows, starts, sizes, offset = [], [], [], 0
        self.ref_offsets = []
        for k, (L, T) in enumerate(self.ladders):
            start = len(rows)
            starts.append(start)
            sizes.append(len(T))
            for _ in range(len(T)):
                rows.append((L, k, start, len(T), offset))
                self.ref_offsets.append(offset)
                offset += L * L
        self.n_sites = offset
        self.R = len(rows)
        self.table_host = np.array(rows, dtype=REPLICA_DTYPE)
        self.table = to_device(self.table_host)
        self.ladder_starts_host = np.asarray(starts, np.int32)
        self.ladder_sizes_host = np.asarray(sizes, np.int32)
        self.ladder_starts = to_device(self.ladder_starts_host)
        self.ladder_sizes = to_device(self.ladder_sizes_host)
        self.ref_offsets_dev = to_device(np.asarray(self.ref_offsets, np.int64))
        self.max_L = int(self.table_host["L"].max())
        self.temperatures = np.concatenate([T for _, T in self.ladders])

        # ---------------------------------------------------------- device buffers
        site = int(np.prod(self.site_shape, dtype=np.int64))
        self.elem_bytes = self.dtype.itemsize * site
        # The chain state -- spins/angles, RNG streams, running energies and,
        # for XY and Kawamura, the (cos, sin) cache -- lives in one device
        # allocation (256-byte aligned pieces, the cache last).  The cache is
        # a function of the angles (refresh_aux reproduces it bit for bit),
        # so a host round trip moves the prefix before it, one copy each way.
        has_aux = self.model_id in (MODEL_XY, MODEL_KAWAMURA, MODEL_KAWAMURA_GAUSS)
        pieces = [("state", (self.n_sites,) + self.site_shape, self.dtype),
                  ("rng", (self.n_sites,), XOROSHIRO128P_DTYPE),
                  ("e_run", (2 * self.R,), np.dtype(np.float32))]
        if has_aux:
            pieces.append(("aux", (self.n_sites, 2), np.dtype(np.float32)))
        offsets, total = [], 0
        for _, shape, dt in pieces:
            offsets.append(total)
            total += -(-int(np.prod(shape, dtype=np.int64)) * np.dtype(dt).itemsize // 256) * 256
        import torch as _t
        self._chain = _t.zeros(max(total, 1), dtype=_t.uint8, device=_t.device("cuda", _t.cuda.current_device()))
        for (name, shape, dt), off in zip(pieces, offsets):
            nb = int(np.prod(shape, dtype=np.int64)) * np.dtype(dt).itemsize
            setattr(self, name, DeviceArray(shape, dt, _storage=self._chain[off:off + max(nb, 1)]))
        self._chain_host = self._chain[:offsets[3]] if has_aux else self._chain
        if not has_aux:
            self.aux = None
        ref_state = DeviceArray((self.n_sites,) + self.site_shape, self.dtype)
        ref_rng = DeviceArray((self.n_sites,), XOROSHIRO128P_DTYPE)
        for k, (L, T) in enumerate(self.ladders):
            o = self.ref_offsets[starts[k]]
            n = len(T) * L * L
            init = (np.asarray(model.initialize_state(L, len(T), self.seeds[k]))
                    if initial_states is None else np.asarray(initial_states[k]))
            if init.shape != (len(T), L, L) + self.site_shape:
                raise ValueError(f"initial state of ladder {k} has shape {init.shape}")
            ref_state[o:o + n].copy_to_device(init.reshape((n,) + self.site_shape))
            sub = create_xoroshiro128p_states(n, self.seeds[k])
            ref_rng[o:o + n].raw().copy_(sub.raw())
        self._permute(ref_state, self.state, self.elem_bytes, 0)
        self._permute(ref_rng, self.rng, 16, 0)
        del ref_state, ref_rng

        self.betas = to_device((1.0 / self.temperatures).astype(np.float32))
        self._initial_betas = (1.0 / self.temperatures).astype(np.float32)
        local = np.concatenate([np.arange(n, dtype=np.int32) for n in sizes])
        self.w2t = to_device(local)
        self.t2w = to_device(local)
        self.energies = device_zeros(self.R, np.float64)
        self.accepted = device_zeros(self.R, np.int64)
        self.accepted_prev = device_zeros(self.R, np.int64)
        self.counters = device_zeros((3, self.R), np.int64)
        self.clock = device_zeros(2, np.int64)
        self.drift = device_zeros(self.R, np.float64)
        self.sigma_t = to_device(np.full(self.R, sigma0, np.float32))
        self.staging = device_zeros((len(self.channels), self.R), np.float64)
        self.sweeps = 0
        self.exchange_rounds = 0

        if self.pt:
            n_pairs = self.R - n_l
            pair_rng = DeviceArray((n_pairs,), XOROSHIRO128P_DTYPE)
            for k, n in enumerate(sizes):
                sub = create_xoroshiro128p_states(n - 1, self.exchange_seeds[k])
                po = starts[k] - k
                pair_rng[po:po + n - 1].raw().copy_(sub.raw())
            self.pair_rng = pair_rng
            self.swap_counts = device_zeros((3, n_pairs), np.int64)
            # Bookkeeping of the fused window + exchange launch: per-pair
            # mailboxes (4 words each) and decision words, the launch
            # counter, then the error flag.
            self.sync = device_zeros(5 * self.R + 2, np.int32)
            trips = np.zeros((5, self.R), np.int64)
            trips[0] = -1
            trips[2] = -1
            for k, n in enumerate(sizes):
                s0 = starts[k]
                trips[0, s0] = 0
                trips[0, s0 + n - 1] = n - 1
                trips[2, s0] = 0
                trips[2, s0 + n - 1] = 0
            self.trips = to_device(trips)

        # He3 parameters
        self.coefficients = np.zeros(5, np.float32)
        self.K = self.g_d = 0.0
        if self.model_id in (MODEL_HE3, MODEL_HE3_GAUSS):
            self.coefficients[:] = np.asarray(model.betas, np.float32)
            self.K, self.g_d = float(model.K), float(model.g_d)
        self.rho, self.mass = float(np.float32(rho)), float(np.float32(proposal_mass))

        self.samples = None
        self.n_slots = 0
        self.first_sample_sweep = 0
        self.sample_interval = 0
        self._graphs = {}
        self.groups = [_Group(np.arange(self.R))]
        self.configure(cluster_size, threads)
        self.refresh_aux()
        self.recompute_energy()

    # ------------------------------------------------------------ layout
    def _permute(self, src, dst, elem_bytes, direction):
        _lib.call("mcgb_batch_permute", ptr(src), ptr(dst), int(elem_bytes), ptr(self.table),
                  ptr(self.ref_offsets_dev), self.R, self.max_L, direction, _lib.stream_handle())

    def ladder_state(self, k):
        """Reference-layout state (n_temps, L, L, ...) of ladder k, walker order."""
        L, T = self.ladders[k]
        ref = DeviceArray((self.n_sites,) + self.site_shape, self.dtype)
        self._permute(self.state, ref, self.elem_bytes, 1)
        o = self.ref_offsets[self.ladder_starts_host[k]]
        n = len(T) * L * L
        return ref[o:o + n].copy_to_host().reshape((len(T), L, L) + self.site_shape)

    def set_ladder_state(self, k, values):
        """Overwrite ladder k's state from a reference-layout array; refreshes energies."""
        L, T = self.ladders[k]
        values = np.ascontiguousarray(values, dtype=self.dtype)
        if values.shape != (len(T), L, L) + self.site_shape:
            raise ValueError("state shape does not match the ladder")
        ref = DeviceArray((self.n_sites,) + self.site_shape, self.dtype)
        self._permute(self.state, ref, self.elem_bytes, 1)
        o = self.ref_offsets[self.ladder_starts_host[k]]
        n = len(T) * L * L
        ref[o:o + n].copy_to_device(values.reshape((n,) + self.site_shape))
        self._permute(ref, self.state, self.elem_bytes, 0)
        self.refresh_aux()
        self.recompute_energy()

    def ladder_rng(self, k):
        """Reference-layout RNG streams of ladder k as an (n, 2) uint64 array."""
        L, T = self.ladders[k]
        ref = DeviceArray((self.n_sites,), XOROSHIRO128P_DTYPE)
        self._permute(self.rng, ref, 16, 1)
        o = self.ref_offsets[self.ladder_starts_host[k]]
        n = len(T) * L * L
        h = ref[o:o + n].copy_to_host()
        return np.stack([h["s0"], h["s1"]], axis=1)

    # ------------------------------------------------------------ launch shape
    def _sizes(self, idx=None):
        return np.unique(self.table_host["L"] if idx is None else self.table_host["L"][idx])

    def _smem(self, C, idx=None):
        best = 0
        for L in self._sizes(idx):
            v = int(_lib.load().mcgb_batch_smem_bytes(self.model_id, int(L), int(C)))
            if v < 0:
                _lib.check(v, "mcgb_batch_smem_bytes")
            best = max(best, v)
        return best

    @staticmethod
    def effective_cluster(L, C):
        """CTAs of a C-CTA cluster that hold a replica of size L."""
        rows = int(L) // 2
        for c in range(int(C), 1, -1):
            if rows % c == 0:
                return c
        return 1

    def candidate_shapes(self, idx=None):
        """(cluster_size, threads) pairs valid for every replica of the batch
        (or of the replicas `idx`)."""
        out = []
        Ls = self._sizes(idx)
        for C in (1, 2, 4, 8, 16):
            smem = self._smem(C, idx)
            if smem > 232448:
                continue
            npl_max = max(int(L) ** 2 // (4 * self.effective_cluster(L, C)) for L in Ls)
            t_max = {MODEL_HE3: 512, MODEL_HE3_GAUSS: 512, MODEL_KAWAMURA: 512,
                     MODEL_KAWAMURA_GAUSS: 512}.get(self.model_id, 1024)
            # Powers of two, and multiples of 96 for sizes whose plaquette
            # counts carry a factor of 3 (L = 48, 96, ...): a thread count
            # that divides a colour's plaquettes keeps every thread's share
            # equal, so no warp idles at the colour barriers.
            for T in (96, 128, 192, 256, 288, 384, 512, 576, 768, 1024):
                if T > t_max or (T > 32 * ((npl_max + 31) // 32) and T > 128):
                    continue
                out.append((C, T))
        return out

    def _costs(self, C, idx=None):
        """Relative time a cluster spends on each replica (sites per active CTA)."""
        Ls = (self.table_host["L"] if idx is None else self.table_host["L"][idx]).astype(np.int64)
        return np.array([L * L / self.effective_cluster(L, C) for L in Ls], dtype=np.float64)

    def _work_costs(self, C, T, idx=None):
        return visit_costs(self.table_host["L"] if idx is None else self.table_host["L"][idx], C, T)

    def max_clusters(self, C, T, idx=None):
        n = ctypes.c_int(0)
        _lib.call("mcgb_batch_max_clusters", self.model_id, C, T, self._smem(C, idx), ctypes.byref(n))
        return n.value

    def configure(self, cluster_size=None, threads=None):
        """Choose each group's cluster shape (heuristic unless given) and build
        its work lists."""
        for g in self.groups:
            self._configure_group(g, cluster_size, threads)
        self._resident_checked = False
        self._graphs.clear()

    def _configure_group(self, g, cluster_size=None, threads=None):
        idx = g.idx
        if cluster_size is None or threads is None:
            best = None
            Ls = self._sizes(idx)
            for C, T in self.candidate_shapes(idx):
                if cluster_size is not None and C != cluster_size:
                    continue
                if threads is not None and T != threads:
                    continue
                m = self.max_clusters(C, T, idx)
                if m < 1:
                    continue
                ncl = min(m, len(idx))
                # Estimated window time ~ (largest cluster load) / threads.
                _, _, loads = lpt_work_lists(self._costs(C, idx), ncl)
                npl = max(int(L) ** 2 // (4 * self.effective_cluster(L, C)) for L in Ls)
                occupancy = min(1.0, npl / T)
                score = loads.max() / (T * occupancy) + 0.02 * C
                if best is None or score < best[0]:
                    best = (score, C, T)
            if best is None:
                raise ValueError("no cluster shape fits this batch")
            _, cluster_size, threads = best
        if int(cluster_size) not in range(1, 17):
            raise ValueError("cluster_size must be 1..16")
        if self._smem(int(cluster_size), idx) > 232448:
            raise ValueError("a strip does not fit in shared memory; use a larger cluster_size")
        C, T = int(cluster_size), int(threads)
        m = self.max_clusters(C, T, idx)
        if m < 1:
            raise ValueError(f"cluster shape ({C}, {T}) cannot be resident")
        g.cluster_size, g.threads, g.n_clusters = C, T, min(m, len(idx))
        wp, wi, _ = lpt_work_lists(self._work_costs(C, T, idx), g.n_clusters)
        g.work_host = np.ascontiguousarray(idx[wi].astype(np.int32))
        g.work_ptr, g.work_idx = to_device(wp), to_device(g.work_host)
        # Resident launches (many windows per launch, strips kept on chip)
        # need one replica per cluster and every cluster resident at once.
        # Concurrent groups share the GPU, so no group runs cooperative
        # (resident) launches then.
        g.resident = (self._resident_wanted and self.pt and g.n_clusters == len(idx)
                      and bool(np.all(np.diff(wp) == 1)) and not self._side_by_side())

    def split_by_size(self, split=True, concurrent=False):
        """One group -- one launch per window, its own cluster shape -- per
        lattice size (split=True), or one group for the whole batch.  With
        `concurrent` the groups' launches of a window run side by side on
        streams of their own, each from its own copy of the device clock and
        with its own exchange bookkeeping (a ladder never spans groups), and
        the step continues once all have finished; otherwise one after
        another on the current stream."""
        Ls = self.table_host["L"]
        if split:
            self.groups = [_Group(np.flatnonzero(Ls == L)) for L in np.unique(Ls)]
        else:
            self.groups = [_Group(np.arange(self.R))]
        self.concurrent = bool(concurrent) and split
        self._graphs.clear()
        self.configure()

    def _side_by_side(self):
        return self.concurrent and len(self.groups) > 1

    def _group_resources(self):
        for g in self.groups:
            if g.stream is None:
                g.stream = torch.cuda.Stream()
                g.clock = device_zeros(2, np.int64)
                if self.pt:
                    g.sync = device_zeros(len(self.sync), np.int32)

    def _syncs(self):
        """Every exchange-bookkeeping array in use."""
        if not self.pt:
            return []
        return [self.sync] + [g.sync for g in self.groups if g.sync is not None]

    def _side_by_side_launch(self, launch, take_group_clock):
        """launch(g, stream handle) for every group on the group's stream,
        forked from and joined back into the current stream (so a CUDA graph
        captures the fork and the join).  Each group starts from a copy of
        the clock; with take_group_clock the groups advanced their copies
        (all by the same windows) and the batch clock takes group 0's."""
        self._group_resources()
        main = torch.cuda.current_stream()
        fork = torch.cuda.Event()
        fork.record(main)
        joins = []
        for g in self.groups:
            g.stream.wait_event(fork)
            with torch.cuda.stream(g.stream):
                g.clock.raw().copy_(self.clock.raw())
                launch(g, _lib.stream_handle())
                done = torch.cuda.Event()
                done.record(g.stream)
                joins.append(done)
        for done in joins:
            main.wait_event(done)
        if take_group_clock:
            self.clock.raw().copy_(self.groups[0].clock.raw())

    # The first group's shape (the only group unless the batch is split).
    @property
    def cluster_size(self):
        return self.groups[0].cluster_size

    @property
    def threads(self):
        return self.groups[0].threads

    @property
    def n_clusters(self):
        return self.groups[0].n_clusters

    @property
    def work_ptr(self):
        return self.groups[0].work_ptr

    @property
    def work_idx(self):
        return self.groups[0].work_idx

    @property
    def resident(self):
        """Whether exchange windows run as resident launches (any group)."""
        return any(g.resident for g in self.groups)

    def launches_per_step(self, n_windows):
        """Kernel launches of a step of n_windows full windows: per group one
        resident launch or one fused launch per window with exchange; without
        exchange, per window one launch per group and the clock tick."""
        if self.pt:
            return sum(1 if (g.resident and n_windows > 1) else n_windows for g in self.groups)
        return n_windows * (len(self.groups) + 1)

    def shapes(self):
        """[(lattice sizes, cluster_size, threads, resident)] per group."""
        return [([int(L) for L in self._sizes(g.idx)], g.cluster_size, g.threads, g.resident) for g in self.groups]

    # ------------------------------------------------------------ argument blocks
    def _window(self, n_sweeps, staging=False, group=None, clock=None):
        g = self.groups[0] if group is None else group
        w = BatchWindow()
        w.table = self.table.ptr
        w.host_table = self.table_host.ctypes.data
        w.n_replicas = self.R
        w.work_ptr, w.work_idx = g.work_ptr.ptr, g.work_idx.ptr
        w.n_clusters, w.cluster_size, w.threads = g.n_clusters, g.cluster_size, g.threads
        if len(self.groups) > 1:
            w.host_work_idx = g.work_host.ctypes.data
            w.n_work = len(g.idx)
        w.state, w.rng, w.betas, w.w2t = self.state.ptr, self.rng.ptr, self.betas.ptr, self.w2t.ptr
        w.aux = None if self.aux is None else self.aux.ptr
        w.e_run, w.energies, w.accepted = self.e_run.ptr, self.energies.ptr, self.accepted.ptr
        w.counters = self.counters.ptr if self.model_id == MODEL_HE3_GAUSS else None
        if self.samples is not None:
            w.samples = self.samples.ptr
            w.staging = self.staging.ptr if (staging and self.pt) else None
            w.n_temps_total = self.R
            w.n_slots = self.n_slots
            w.first_sample_sweep = self.first_sample_sweep
            w.sample_interval = self.sample_interval
        w.clock = self.clock.ptr if clock is None else clock.ptr
        w.n_sweeps = int(n_sweeps)
        w.J = float(getattr(self.model, "J", 1.0))
        w.delta = float(getattr(self.model, "delta", 0.0))
        w.sigma_t = self.sigma_t.ptr if self._gaussian_widths() else None
        for q in range(5):
            w.coefficients[q] = float(self.coefficients[q])
        w.K, w.g_d, w.rho, w.mass = self.K, self.g_d, self.rho, self.mass
        return w

    def _gaussian_widths(self):
        return self.model_id in GAUSSIAN_WIDTHS and self.proposal == "gaussian"

    def _pt(self):
        p = BatchPT()
        p.t2w, p.rng = self.t2w.ptr, self.pair_rng.ptr
        p.swap_counts, p.trips = self.swap_counts.ptr, self.trips.ptr
        p.ladder_starts, p.ladder_sizes = self.ladder_starts.ptr, self.ladder_sizes.ptr
        p.n_ladders = len(self.ladders)
        p.channels = len(self.channels)
        return p

    # ------------------------------------------------------------ stepping
    def _enqueue_window(self, n_sweeps, exchange, tune=False):
        s = _lib.stream_handle()
        if self._side_by_side() and not tune:
            p = self._pt() if exchange else None
            self._keep_pt, keep = p, []

            def launch(g, gs):
                w = self._window(n_sweeps, staging=exchange, group=g, clock=g.clock)
                keep.append(w)
                if exchange:
                    # Window, exchange and the group clock's tick in one launch.
                    _lib.call("mcgb_batch_window_exchange", self.model_id, ctypes.byref(w), ctypes.byref(p),
                              g.sync.cptr, gs)
                else:
                    _lib.call("mcgb_batch_window_run", self.model_id, ctypes.byref(w), gs)

            self._side_by_side_launch(launch, take_group_clock=exchange)
            self._keep = keep
            if not exchange:
                _lib.call("mcgb_batch_clock_tick", self.clock.cptr, int(n_sweeps), 0, s)
            return
        if exchange and not tune:
            # Window, exchange and clock tick in one launch per group (the
            # last group's launch advances the clock).
            p = self._pt()
            self._keep_pt = p
            for i, g in enumerate(self.groups):
                w = self._window(n_sweeps, staging=True, group=g)
                w.hold_clock = int(i + 1 < len(self.groups))
                self._keep = w
                _lib.call("mcgb_batch_window_exchange", self.model_id, ctypes.byref(w), ctypes.byref(p),
                          self.sync.cptr, s)
            return
        for g in self.groups:
            w = self._window(n_sweeps, staging=exchange, group=g)
            self._keep = w
            _lib.call("mcgb_batch_window_run", self.model_id, ctypes.byref(w), s)
        if tune:
            # The window's acceptance belongs to the temperatures it ran at:
            # tune before the exchange moves replicas.
            _lib.call("mcgb_batch_tune_sigma", self.sigma_t.cptr, self.accepted.cptr, self.accepted_prev.cptr,
                      self.w2t.cptr, self.table.cptr, self.R, int(n_sweeps), 0.5, 2.0, 0.02, 2 * np.pi, s)
        if exchange:
            p = self._pt()
            _lib.call("mcgb_batch_exchange", ctypes.byref(w), ctypes.byref(p), s)
        _lib.call("mcgb_batch_clock_tick", self.clock.cptr, int(n_sweeps), int(bool(exchange)), s)

    def enqueue_plain_windows(self, n_sweeps):
        """One window of n_sweeps sweeps of every group, without exchange or
        clock tick, side by side when the groups run so: the window kernels
        alone, as a benchmark times them (the chain advances)."""
        if self._side_by_side():
            keep = []

            def launch(g, gs):
                w = self._window(n_sweeps, group=g, clock=g.clock)
                keep.append(w)
                _lib.call("mcgb_batch_window_run", self.model_id, ctypes.byref(w), gs)

            self._side_by_side_launch(launch, take_group_clock=False)
            self._keep = keep
            return
        s = _lib.stream_handle()
        for g in self.groups:
            w = self._window(n_sweeps, group=g)
            self._keep = w
            _lib.call("mcgb_batch_window_run", self.model_id, ctypes.byref(w), s)

    def _schedule(self, n_sweeps):
        """Split n_sweeps into (length, exchange_after) windows aligned to the PT schedule."""
        out = []
        s, left = self.sweeps, n_sweeps
        while left > 0:
            if self.pt:
                to_ex = self.exchange_interval - (s % self.exchange_interval)
                n = min(left, to_ex)
                out.append((n, n == to_ex))
            else:
                n = min(left, NO_EXCHANGE_WINDOW)
                out.append((n, False))
            s += n
            left -= n
        return out

    def run(self, n_sweeps, tune=False, graph=True):
        """Advance every replica by n_sweeps sweeps (with exchanges on schedule).

        Runs of full windows replay captured CUDA graphs of up to 64 windows;
        partial windows at the ends launch directly.
        """
        plan = self._schedule(int(n_sweeps))
        full = (self.exchange_interval, True) if self.pt else (NO_EXCHANGE_WINDOW, False)
        i = 0
        while i < len(plan):
            if graph and plan[i] == full:
                j = i
                while j < len(plan) and plan[j] == full:
                    j += 1
                remaining = j - i
                while remaining:
                    if self.resident and full[1] and not tune:
                        chunk = min(64, remaining)  # one resident launch
                    else:
                        chunk = 1 << min(6, remaining.bit_length() - 1)
                    self._replay(chunk, full, tune)
                    remaining -= chunk
                i = j
                continue
            n, ex = plan[i]
            self._enqueue_window(n, ex, tune)
            self._advance(n, ex)
            i += 1

    def _advance(self, n, exchanged, times=1):
        self.sweeps += n * times
        if exchanged:
            self.exchange_rounds += times

    def _enqueue_resident(self, n_sweeps, count, fallback=False):
        """`count` exchange windows: one resident launch per resident group,
        then, window by window, one launch per other group.  Every launch
        reads the clock as the step found it but the one that advances it:
        the last launch of a window (or the last resident launch when every
        group is resident).  With `fallback`, a group whose cooperative launch
        is refused (nothing of it runs) moves to the window-by-window launches."""
        s = _lib.stream_handle()
        p = self._pt()
        self._keep_pt = p
        if self._side_by_side():
            keep = []

            def launch(g, gs):
                for _ in range(count):
                    w = self._window(n_sweeps, staging=True, group=g, clock=g.clock)
                    keep.append(w)
                    _lib.call("mcgb_batch_window_exchange", self.model_id, ctypes.byref(w), ctypes.byref(p),
                              g.sync.cptr, gs)

            self._side_by_side_launch(launch, take_group_clock=True)
            self._keep = keep
            return
        res = [g for g in self.groups if g.resident]
        non = [g for g in self.groups if not g.resident]
        for i, g in enumerate(res):
            w = self._window(n_sweeps, staging=True, group=g)
            w.hold_clock = int(bool(non) or i + 1 < len(res))
            self._keep = w
            try:
                _lib.call("mcgb_batch_run_resident", self.model_id, ctypes.byref(w), ctypes.byref(p),
                          self.sync.cptr, int(count), s)
            except _lib.MCGBError:
                if not fallback:
                    raise
                g.resident = False
                non.append(g)
        for _ in range(count if non else 0):
            for i, g in enumerate(non):
                w = self._window(n_sweeps, staging=True, group=g)
                w.hold_clock = int(i + 1 < len(non))
                self._keep = w
                _lib.call("mcgb_batch_window_exchange", self.model_id, ctypes.byref(w), ctypes.byref(p),
                          self.sync.cptr, s)

    def _replay(self, count, step, tune):
        resident = self.resident and step[1] and not tune and count > 1
        if resident and not self._resident_checked:
            # The first resident step runs directly: a group whose clusters
            # cannot all be resident on this device has its cooperative launch
            # refused before anything of it runs, and falls back to one
            # launch per window.
            self._enqueue_resident(step[0], count, fallback=True)
            self._resident_checked = True
            self._graphs.clear()
            self._advance(step[0], step[1], count)
            return
        key = (count, step, tune, self.samples is not None and self.samples.ptr, resident, self._side_by_side())
        g = self._graphs.get(key)
        if g is None:
            # Capture reads only argument blocks; the device clock advances at replay.
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                if resident:
                    self._enqueue_resident(step[0], count)
                else:
                    for _ in range(count):
                        self._enqueue_window(step[0], step[1], tune)
            self._graphs[key] = g
        g.replay()
        self._advance(step[0], step[1], count)

    def set_wait_limit(self, polls):
        """Polls a resident launch's wait between windows makes before giving
        up (None: the default, about a second); returns the previous value.
        Captured graphs hold the old limit, so they are dropped."""
        self._graphs.clear()
        self._resident_checked = False
        return int(_lib.load().mcgb_batch_set_wait_limit(-1 if polls is None else int(polls)))

    def check_errors(self):
        """Raise MCGBTimeout if a fused launch gave up a bounded wait: a
        resident launch waiting between windows for a pair's decision (flag
        1) or a window waiting for its strip's bulk copies (flag 2).  Its
        samples and exchange statistics are then unreliable and its slot maps
        may disagree; before raising, the maps are rebuilt from w2t (identity
        for a ladder whose w2t is no permutation), the betas set to match and
        the sync array zeroed, so later runs are sound."""
        if not self.pt:
            return
        flag = max(int(sy.copy_to_host()[-1]) for sy in self._syncs())
        if flag:
            self._repair_maps()
            for sy in self._syncs():
                sy.copy_to_device(np.zeros(len(sy), np.int32))
            what = ("a window timed out waiting for its strip's bulk copies" if flag == 2
                    else "a resident launch timed out waiting between windows")
            raise _lib.MCGBTimeout(-4, what)

    def _repair_maps(self):
        w2t = self.w2t.copy_to_host()
        t2w = np.empty_like(w2t)
        for s0, n in zip(self.ladder_starts_host, self.ladder_sizes_host):
            local = w2t[s0:s0 + n]
            if not np.array_equal(np.sort(local), np.arange(n)):
                local[:] = np.arange(n)
            t2w[s0:s0 + n] = np.argsort(local)
        self.w2t.copy_to_device(w2t)
        self.t2w.copy_to_device(t2w.astype(np.int32))
        starts = np.repeat(self.ladder_starts_host, self.ladder_sizes_host)
        self.betas.copy_to_device(self._initial_betas[starts + w2t])

    def exchange_now(self):
        """Attempt one matching now (fresh energies from the running cache)."""
        if not self.pt:
            raise ValueError("this batch has no replica exchange")
        s = _lib.stream_handle()
        w = self._window(0)
        _lib.call("mcgb_batch_exchange", ctypes.byref(w), ctypes.byref(self._pt()), s)
        _lib.call("mcgb_batch_clock_tick", self.clock.cptr, 0, 1, s)
        self.exchange_rounds += 1

    # ------------------------------------------------------------ host I/O
    def pinned_state_buffers(self):
        """A pinned host buffer for the chain state (spins/angles, RNG
        streams, running energies), engine layout."""
        import torch as _t
        return {"chain": _t.empty(self._chain_host.numel(), dtype=_t.uint8, pin_memory=True)}

    def upload_state(self, host, recompute=False):
        """Asynchronous host-to-device copy from pinned buffers.  A buffer from
        pinned_state_buffers/download_state resumes the chain exactly (one
        copy, then the (cos, sin) cache rebuilt from the angles on the
        device); a dict of ``state`` and ``rng`` bytes alone (engine layout)
        uploads those, then also recomputes the exact energies on the
        device, as does ``recompute``."""
        if "chain" in host:
            self._chain_host.copy_(host["chain"], non_blocking=True)
        else:
            self.state.raw().copy_(host["state"], non_blocking=True)
            self.rng.raw().copy_(host["rng"], non_blocking=True)
        self.refresh_aux()
        if recompute or "chain" not in host:
            self.recompute_energy()

    def download_state(self, host):
        """Asynchronous device-to-host copy of the chain state (one copy)."""
        host["chain"].copy_(self._chain_host, non_blocking=True)

    def _chain_arrays(self):
        """Names of the device arrays that hold the chain and its bookkeeping."""
        names = ["state", "rng", "betas", "w2t", "t2w", "e_run", "energies", "accepted", "accepted_prev",
                 "clock", "sigma_t", "counters"]
        if self.aux is not None:
            names.append("aux")
        if self.pt:
            names += ["pair_rng", "swap_counts", "trips"]
        return names

    def checkpoint(self):
        """Everything needed to resume the chain bit-exactly, as host arrays."""
        ck = {n: getattr(self, n).copy_to_host().copy() for n in self._chain_arrays()}
        ck["sweeps"], ck["exchange_rounds"] = self.sweeps, self.exchange_rounds
        return ck

    def restore(self, ck):
        """Resume from checkpoint(); the batch must have the same ladders."""
        for name, value in ck.items():
            if name in ("sweeps", "exchange_rounds"):
                continue
            arr = getattr(self, name)
            if arr.nbytes != np.asarray(value).nbytes:
                raise ValueError(f"checkpoint field {name} does not match this batch")
            arr.copy_to_device(value)
        self.sweeps, self.exchange_rounds = int(ck["sweeps"]), int(ck["exchange_rounds"])

    def refresh_aux(self):
        """Recompute the (cos, sin) cache from the state."""
        if self.aux is not None:
            w = self._window(0)
            _lib.call("mcgb_batch_refresh_aux", self.model_id, ctypes.byref(w), _lib.stream_handle())

    def recompute_energy(self):
        """FP64 total energies; returns drift = running - exact per replica."""
        w = self._window(0)
        _lib.call("mcgb_batch_recompute_energy", self.model_id, ctypes.byref(w), self.drift.cptr,
                  _lib.stream_handle())
        return self.drift

    # ------------------------------------------------------------ sampling
    def allocate_samples(self, first_sample_sweep, sample_interval, n_slots):
        self.samples = device_zeros((n_slots, len(self.channels), self.R), np.float64)
        self.n_slots, self.first_sample_sweep = int(n_slots), int(first_sample_sweep)
        self.sample_interval = int(sample_interval)
        self._graphs.clear()

    def simulate(self, thermalization_sweeps=1000, measurement_sweeps=4000, sample_interval=10,
                 tune_sigma=None, graph=True):
        """Simulation.run for every ladder: returns one ``{"samples", "metadata"}``
        per ladder (core/simulation.py:28-96 schema; samples in temperature order)."""
        if thermalization_sweeps < 0:
            raise ValueError("Thermalization sweeps cannot be negative")
        if measurement_sweeps < 1:
            raise ValueError("Measurement sweeps must be positive")
        if sample_interval < 1 or sample_interval > measurement_sweeps:
            raise ValueError("Invalid sampling interval")
        if tune_sigma is None:
            tune_sigma = self._gaussian_widths()
        start = self.sweeps
        self.samples = None
        self.run(thermalization_sweeps, tune=tune_sigma, graph=graph)
        n_slots = measurement_sweeps // sample_interval
        self.allocate_samples(start + thermalization_sweeps + sample_interval, sample_interval, n_slots)
        self.run(measurement_sweeps, tune=False, graph=graph)
        data = self.samples.copy_to_host()
        self.check_errors()
        sample_sweeps = thermalization_sweeps + sample_interval * np.arange(1, n_slots + 1)
        runs = []
        for k, (L, T) in enumerate(self.ladders):
            s0, n = int(self.ladder_starts_host[k]), len(T)
            samples = {name: data[:, c, s0:s0 + n].copy() for c, name in enumerate(self.channels)}
            metadata = {
                "L": L, "temperatures": T.copy(), "seed": self.seeds[k],
                "model_parameters": self.model.parameters(),
                "thermalization_sweeps": thermalization_sweeps,
                "measurement_sweeps": measurement_sweeps,
                "sample_interval": sample_interval,
                "sample_sweeps": sample_sweeps.copy(),
            }
            if self.pt:
                metadata["parallel_tempering"] = self.diagnostics(k)
            runs.append({"samples": samples, "metadata": metadata})
        self.samples = None
        return runs

    # ------------------------------------------------------------ diagnostics
    def diagnostics(self, k):
        """core/parallel_tempering.py:280-317 diagnostics of ladder k."""
        counts = self.swap_counts.copy_to_host()
        s0, n = int(self.ladder_starts_host[k]), int(self.ladder_sizes_host[k])
        po = s0 - k
        c = counts[:, po:po + n - 1]
        if np.any(c[2]):
            raise FloatingPointError("Nonfinite energies encountered during replica exchange")
        trips = self.trips.copy_to_host()[:, s0:s0 + n]
        w2t = self.w2t.copy_to_host()[s0:s0 + n]
        t2w = self.t2w.copy_to_host()[s0:s0 + n]
        attempts, accepted = c[0], c[1]
        rates = np.divide(accepted, attempts, out=np.zeros(n - 1), where=attempts > 0)
        completed = int(trips[3].sum())
        return {
            "exchange_interval": self.exchange_interval,
            "exchange_seed": self.exchange_seeds[k],
            "sweeps": self.sweeps,
            "exchange_rounds": self.exchange_rounds,
            "next_parity": (self.exchange_rounds & 1) if n > 2 else 0,
            "diagnostics_scope": "since_wrapper_creation_including_thermalization",
            "temperature_betas": self._initial_betas[s0:s0 + n].copy(),
            "attempts": attempts.copy(), "accepted": accepted.copy(), "acceptance_rates": rates,
            "walker_to_temperature": w2t, "temperature_to_walker": t2w,
            "walker_round_trips": trips[3].copy(),
            "walker_round_trip_total_sweeps": trips[4].copy(),
            "mean_round_trip_sweeps": float(trips[4].sum()) / completed if completed else None,
        }

    def acceptance(self):
        """Accepted moves per replica so far (device counters)."""
        return self.accepted.copy_to_host()

    def sampling_diagnostics(self):
        """He3 Gaussian sampler counters per replica (walker order), in the
        keys of models/he3/gaussian_fast.py:147-156."""
        L2 = self.table_host["L"].astype(np.int64) ** 2
        attempts = L2 * self.sweeps
        accepted = self.accepted.copy_to_host()
        nonfinite = self.counters.copy_to_host()[2]
        return {
            "algorithm": "float32_conditional_gaussian_full_hamiltonian_mh",
            "sweeps_including_compilation": self.sweeps,
            "rho": self.rho, "proposal_mass": self.mass,
            "attempts": attempts.tolist(), "accepted": accepted.tolist(),
            "nonfinite_rejections": nonfinite.tolist(),
            "acceptance_rates": np.divide(accepted, attempts, out=np.zeros(self.R),
                                          where=attempts > 0).tolist(),
        }

    # ------------------------------------------------------------ autotuning
    def autotune(self, sweeps_per_trial=None, shapes=None, verbose=False, split=None, sample_interval=None):
        """Time each valid (cluster_size, threads) on a copy-free trial window
        and keep the fastest, per group.  For a batch of several lattice sizes
        (`split` None) it also tunes one group per size and keeps that when a
        few real steps of it beat the single launch's by 2 %; `split`
        True/False forces either.  With `sample_interval` the trial windows
        also take samples at that cadence (into a scratch ring): a sample's
        reduction across a cluster's CTAs costs more on larger clusters, so
        frequent sampling can favour another shape.  State and RNG are saved
        and restored, so tuning does not change the Markov chain.  Returns
        the trial times [(ms, cluster_size, threads)] of the kept grouping's
        groups."""
        n = sweeps_per_trial or (self.exchange_interval or 10)
        saved_state = self.state.raw().clone()
        saved_aux = None if self.aux is None else self.aux.raw().clone()
        saved_rng = self.rng.raw().clone()
        saved_e = self.e_run.raw().clone()
        saved_acc = self.accepted.raw().clone()
        saved_clock = self.clock.raw().clone()
        saved_samples, self.samples = self.samples, None
        saved_ring = (self.n_slots, self.first_sample_sweep, self.sample_interval)
        if sample_interval:
            si = int(sample_interval)
            if si < 1:
                raise ValueError("sample_interval must be positive")
            self.allocate_samples(self.sweeps + si, si, n // si + 1)

        per_group = []

        def tune_groups():
            total, trials = 0.0, []
            per_group.clear()
            for g in self.groups:
                res = self._tune_group(g, n, shapes, verbose)
                total += res[0][0]
                trials += res
                per_group.append(res)
            return total, trials

        ragged = len(self._sizes()) > 1
        if split is None and ragged:
            self.split_by_size(False)
            one, one_trials = tune_groups()
            one_shape = (self.cluster_size, self.threads)
            self.split_by_size(True)
            many, many_trials = tune_groups()
            many_shapes = [(g.cluster_size, g.threads) for g in self.groups]
            packed_shapes = self._side_by_side_shapes(per_group)
            # Trial windows launch every group once per window; a production
            # step replays graphs of resident launches, which hide most of
            # that cost.  So the grouping is chosen on a few real steps.
            many_run = self._time_steps(n)
            # The same groups launched side by side on streams of their own.
            self.split_by_size(True, concurrent=True)
            for g, (C, T) in zip(self.groups, many_shapes):
                self._configure_group(g, C, T)
            side_run = self._time_steps(n)
            side_shapes = many_shapes
            if packed_shapes != many_shapes:
                # Shapes chosen for sharing the GPU (below) rather than each
                # group's fastest alone.
                for g, (C, T) in zip(self.groups, packed_shapes):
                    self._configure_group(g, C, T)
                packed_run = self._time_steps(n)
                if verbose:
                    print(f"autotune: side by side {side_run:.3f} ms with each group's fastest shape, "
                          f"{packed_run:.3f} ms with shapes {packed_shapes}")
                if packed_run < side_run:
                    side_run, side_shapes = packed_run, packed_shapes
            side_shapes, side_run = self._refine_side_by_side(per_group, side_shapes, side_run, n, verbose)
            self.split_by_size(False)
            self.configure(*one_shape)
            one_run = self._time_steps(n)
            if verbose:
                print(f"autotune: one launch {one:.3f} ms, one per size {many:.3f} ms per {n}-sweep window "
                      f"(trials); {one_run:.3f} ms against {many_run:.3f} ms one after another and "
                      f"{side_run:.3f} ms side by side (steps)")
            best = min(many_run, side_run)
            if best < 0.98 * one_run:
                side = side_run < many_run
                self.split_by_size(True, concurrent=side)
                for g, (C, T) in zip(self.groups, side_shapes if side else many_shapes):
                    self._configure_group(g, C, T)
                self._graphs.clear()
                self._resident_checked = False
                results = many_trials
            else:
                results = one_trials
        else:
            if split is not None and ragged and split != (len(self.groups) > 1):
                self.split_by_size(split, concurrent=self.concurrent)
            _, results = tune_groups()
        self.state.raw().copy_(saved_state)
        if saved_aux is not None:
            self.aux.raw().copy_(saved_aux)
        self.rng.raw().copy_(saved_rng)
        self.e_run.raw().copy_(saved_e)
        self.accepted.raw().copy_(saved_acc)
        self.clock.raw().copy_(saved_clock)
        self.samples = saved_samples
        self.n_slots, self.first_sample_sweep, self.sample_interval = saved_ring
        self._graphs.clear()
        self._resident_checked = False
        self.recompute_energy()
        return results

    def _refine_side_by_side(self, per_group, shapes, best_ms, n, verbose=False, tolerance=0.3, budget=10,
                             margin=0.03):
        """Side-by-side groups on real steps: a group's shapes whose time
        alone is within `tolerance` of its fastest can share the GPU with the
        other groups' launches better or worse than those times say (a
        group of many small CTAs beside one of few large ones), so each such
        runner-up is timed in place of the group's current shape, the slowest
        groups first, at most `budget` timings.  A runner-up replaces the
        current shape only when it is faster by `margin` twice: in its own
        timing and again when both are timed once more (the minimum over
        several noisy timings would otherwise favour noise); the time of the
        shapes it came with stands otherwise.  The kept shapes are
        configured.  Returns (shapes, ms per window)."""
        shapes = list(shapes)
        order = sorted(range(len(per_group)), key=lambda k: -per_group[k][0][0])
        tried = 0

        def timed(sh):
            nonlocal tried
            for g, (c, t) in zip(self.groups, sh):
                self._configure_group(g, c, t)
            tried += 1
            return self._time_steps(n)

        for k in order:
            fastest = per_group[k][0][0]
            for ms, C, T in per_group[k]:
                if tried >= budget:
                    break
                if (C, T) == shapes[k] or ms > (1.0 + tolerance) * fastest:
                    continue
                trial = shapes[:k] + [(C, T)] + shapes[k + 1:]
                run = timed(trial)
                if verbose:
                    print(f"autotune: side by side with {trial}: {run:.3f} ms against {best_ms:.3f} ms")
                if run < (1.0 - margin) * best_ms:
                    current, again = timed(shapes), timed(trial)
                    if verbose:
                        print(f"autotune: again {again:.3f} ms against {current:.3f} ms")
                    if again < (1.0 - margin) * current:
                        best_ms, shapes = again, trial
        for g, (c, t) in zip(self.groups, shapes):
            self._configure_group(g, c, t)
        return shapes, best_ms

    def _side_by_side_shapes(self, per_group):
        """Shapes for the groups of a split batch running side by side, from
        each group's trial times [(ms, C, T)] (side_by_side_pick); a group's
        occupancy is its trial time scaled by the fraction of the GPU's
        co-resident clusters its launch holds."""
        rows = []
        for g, res in zip(self.groups, per_group):
            row = []
            for ms, C, T in res:
                m = self.max_clusters(C, T, g.idx)
                if m >= 1:
                    row.append((ms, min(1.0, min(m, len(g.idx)) / m) * ms, C, T))
            if not row:
                return [(C, T) for _, C, T in (r[0] for r in per_group)]
            rows.append(row)
        return [(row[i][2], row[i][3]) for row, i in zip(rows, side_by_side_pick(rows))]

    def _time_steps(self, n, windows=8):
        """ms per n-sweep window of `windows` windows run as production runs
        them (graph replay, resident launches, exchanges), after a warm-up of
        the same plan, which captures the graphs the timed run replays.
        Everything the run changes is put back."""
        kept = {name: getattr(self, name).raw().clone() for name in self._chain_arrays()}
        sweeps, rounds = self.sweeps, self.exchange_rounds
        self._graphs.clear()
        self._resident_checked = False
        self.run(windows * n)
        self.run(windows * n)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        self.run(windows * n)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / windows
        self.check_errors()
        for name, raw in kept.items():
            getattr(self, name).raw().copy_(raw)
        self.sweeps, self.exchange_rounds = sweeps, rounds
        if self.pt:
            # decision words of the rounds just run would match the same
            # rounds run again
            for sy in self._syncs():
                sy.copy_to_device(np.zeros(len(sy), np.int32))
        self._graphs.clear()
        self._resident_checked = False
        return ms

    def _tune_group(self, g, n, shapes=None, verbose=False):
        """Time group g's window over its candidate shapes; keep the fastest."""
        results = []
        for C, T in (shapes or self.candidate_shapes(g.idx)):
            try:
                self._configure_group(g, C, T)
            except ValueError:
                continue
            s = _lib.stream_handle()
            w = self._window(n, group=g)
            _lib.call("mcgb_batch_window_run", self.model_id, ctypes.byref(w), s)
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 3
            ev0.record()
            for _ in range(reps):
                _lib.call("mcgb_batch_window_run", self.model_id, ctypes.byref(w), s)
            ev1.record()
            torch.cuda.synchronize()
            ms = ev0.elapsed_time(ev1) / reps
            results.append((ms, C, T))
            if verbose:
                print(f"autotune sizes {list(self._sizes(g.idx))} C={C} T={T}: {ms:.3f} ms per {n}-sweep window")
        if not results:
            raise ValueError("no cluster shape fits this group")
        results.sort()
        _, C, T = results[0]
        self._configure_group(g, C, T)
        return results


def smoke_run():
    """A short batched XY run with exchanges, compared with an FP64 recompute."""
    from ..models.xy.model import XYModel

    b = LadderBatch(XYModel(), [(16, np.geomspace(0.7, 1.2, 4)), (32, np.geomspace(0.7, 1.2, 4))],
                    exchange_interval=5, proposal="gaussian")
    b.run(20)
    e = b.energies.copy_to_host()
    drift = b.recompute_energy().copy_to_host()
    if not np.all(np.isfinite(e)) or np.max(np.abs(drift)) > 1e-3 * np.max(np.abs(e)):
        raise AssertionError("batched XY energy drift too large")
    b.diagnostics(0)
