// Kernel-side argument block of the batched engine and the host helpers that
// validate a mcgb_batch_window and launch a window kernel with its cluster
// shape.
#pragma once

#include "batch_window.cuh"

namespace mcgb {

struct BatchArgs {
    WindowCommon c;
    void *state;
    float2 *aux;
    float J, delta;
    const float *sigma_t;
    float coeff[5];
    float K, g_d, rho, mass;
    long long *counters;
    int n_replicas;
    FusedExchange fx;  // enabled = 0: the window only
};

inline BatchArgs make_args(const mcgb_batch_window &w)
{
    BatchArgs a;
    a.c.table = w.table;
    a.c.work_ptr = w.work_ptr;
    a.c.work_idx = w.work_idx;
    a.c.rng = w.rng;
    a.c.betas = w.betas;
    a.c.w2t = w.w2t;
    a.c.e_run = w.e_run;
    a.c.energies = w.energies;
    a.c.accepted = w.accepted;
    a.c.samples = w.samples;
    a.c.staging = w.staging;
    a.c.n_temps_total = w.n_temps_total;
    a.c.n_slots = w.n_slots;
    a.c.clock = reinterpret_cast<const long long *>(w.clock);
    a.c.first_sample_sweep = w.first_sample_sweep;
    a.c.sample_interval = w.sample_interval;
    a.c.n_sweeps = w.n_sweeps;
    a.c.cluster_size = w.cluster_size;
    a.c.n_clusters = w.n_clusters;
    a.state = w.state;
    a.aux = static_cast<float2 *>(w.aux);
    a.J = w.J;
    a.delta = w.delta;
    a.sigma_t = w.sigma_t;
    for (int q = 0; q < 5; ++q) a.coeff[q] = w.coefficients[q];
    a.K = w.K;
    a.g_d = w.g_d;
    a.rho = w.rho;
    a.mass = w.mass;
    a.counters = w.counters;
    a.n_replicas = w.n_replicas;
    a.fx = FusedExchange{};
    a.fx.enabled = 0;
    return a;
}

// Host-side checks shared by the exchange entry points.
inline int check_exchange(const mcgb_batch_window &w, const mcgb_batch_pt &pt)
{
    MCGB_REQUIRE(w.energies && w.betas && w.w2t && w.clock && pt.t2w && pt.rng && pt.swap_counts && pt.trips &&
                     pt.ladder_starts && pt.ladder_sizes,
                 "batch_exchange: null pointer");
    MCGB_REQUIRE(pt.n_ladders >= 1 && w.n_replicas >= 2 * pt.n_ladders,
                 "batch_exchange: every ladder needs >= 2 replicas");
    MCGB_REQUIRE(w.n_sweeps >= 0, "batch_exchange: n_sweeps must be >= 0");
    MCGB_REQUIRE(w.staging == nullptr || (w.samples && pt.channels >= 1 && w.n_temps_total >= w.n_replicas),
                 "batch_exchange: bad staging buffer");
    return MCGB_OK;
}

inline ExchangeArgs make_exchange_args(const mcgb_batch_window &w, const mcgb_batch_pt &pt)
{
    ExchangeArgs x;
    x.energies = w.energies;
    x.betas = const_cast<float *>(w.betas);
    x.w2t = const_cast<int32_t *>(w.w2t);
    x.t2w = pt.t2w;
    x.rng = static_cast<ulonglong2 *>(pt.rng);
    x.counts = reinterpret_cast<long long *>(pt.swap_counts);
    x.trips = reinterpret_cast<long long *>(pt.trips);
    x.starts = pt.ladder_starts;
    x.sizes = pt.ladder_sizes;
    x.n_pairs_total = w.n_replicas - pt.n_ladders;
    x.n_replicas = w.n_replicas;
    x.clock = reinterpret_cast<const long long *>(w.clock);
    x.window_sweeps = w.n_sweeps;
    x.samples = w.samples;
    x.staging = w.staging;
    x.channels = pt.channels;
    x.n_temps_total = w.n_temps_total;
    x.n_slots = w.n_slots;
    x.sample_interval = w.sample_interval;
    x.first_sample_sweep = w.first_sample_sweep;
    return x;
}

// Validate the table against the cluster shape.  Returns a negative status
// on error, else 0; strips are sized per replica by effective_cluster.
inline int validate_window(const mcgb_batch_window &w)
{
    MCGB_REQUIRE(w.table && w.host_table && w.work_ptr && w.work_idx, "batch window: null table/work list");
    MCGB_REQUIRE(w.state && w.rng && w.betas && w.w2t && w.e_run && w.energies && w.accepted && w.clock,
                 "batch window: null state pointer");
    MCGB_REQUIRE(w.n_replicas >= 1 && w.n_clusters >= 1, "batch window: empty batch");
    MCGB_REQUIRE(w.cluster_size >= 1 && w.cluster_size <= 16, "batch window: cluster_size must be 1..16");
    MCGB_REQUIRE(w.threads >= 32 && w.threads <= 1024 && w.threads % 32 == 0,
                 "batch window: threads must be a multiple of 32 in [32, 1024]");
    MCGB_REQUIRE(w.n_sweeps >= 0 && w.n_sweeps <= kMaxWindowSweeps, "batch window: n_sweeps must be in [0, %d]",
                 kMaxWindowSweeps);
    MCGB_REQUIRE(w.samples == nullptr || (w.n_slots >= 1 && w.n_temps_total >= 1 && w.sample_interval >= 1 &&
                                          w.sample_interval <= kMaxWindowSweeps),
                 "batch window: bad sample buffer");
    for (int r = 0; r < w.n_replicas; ++r) {
        const mcgb_replica &rep = w.host_table[r];
        MCGB_REQUIRE(rep.L >= 4 && rep.L % 2 == 0 && rep.L <= 32768, "batch window: replica %d has bad L=%d", r,
                     rep.L);
        MCGB_REQUIRE(rep.ladder_start >= 0 && rep.ladder_start + rep.n_temps <= w.n_replicas &&
                         rep.ladder_start <= r && r < rep.ladder_start + rep.n_temps,
                     "batch window: replica %d has an inconsistent ladder range", r);
        MCGB_REQUIRE(rep.state_offset >= 0, "batch window: negative state offset");
    }
    MCGB_REQUIRE(w.samples == nullptr || w.n_temps_total >= w.n_replicas,
                 "batch window: n_temps_total must cover every replica");
    if (w.host_work_idx != nullptr) {
        MCGB_REQUIRE(w.n_work >= 1 && w.n_work <= w.n_replicas, "batch window: bad n_work %d", w.n_work);
        for (int k = 0; k < w.n_work; ++k)
            MCGB_REQUIRE(w.host_work_idx[k] >= 0 && w.host_work_idx[k] < w.n_replicas,
                         "batch window: work entry %d names replica %d of %d", k, w.host_work_idx[k], w.n_replicas);
    }
    return MCGB_OK;
}

// The replicas a launch runs: host_work_idx when given, else the table.
inline int work_count(const mcgb_batch_window &w) { return w.host_work_idx ? w.n_work : w.n_replicas; }
inline int work_replica(const mcgb_batch_window &w, int k) { return w.host_work_idx ? w.host_work_idx[k] : k; }

// Shared memory for the largest strip among the replicas a launch runs.
template <class M>
inline size_t batch_smem(const mcgb_batch_window &w, int C, bool streams = false)
{
    size_t best = 0;
    for (int k = 0; k < work_count(w); ++k) {
        const int L = w.host_table[work_replica(w, k)].L, Ce = effective_cluster(L, C);
        const size_t b = window_smem_bytes<M>((long long)L * L / (4 * Ce), (long long)L / 2, streams);
        if (b > best) best = b;
    }
    return best;
}

template <class M>
inline size_t single_smem(int L, int C)
{
    const int Ce = effective_cluster(L, C);
    return window_smem_bytes<M>((long long)L * L / (4 * Ce), (long long)L / 2);
}

template <class M, int NPMAX>
int launch_window(const BatchArgs &a, const mcgb_batch_window &w, cudaStream_t stream, const char *name)
{
    auto kern = window_kernel<M, NPMAX>;
    const size_t smem = batch_smem<M>(w, w.cluster_size, smem_stream_variant<M, NPMAX>());
    MCGB_REQUIRE(smem <= 232448, "%s: a strip needs %zu bytes of shared memory (> 227 KB); use a larger "
                                 "cluster_size", name, smem);
    int st = cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "cudaFuncSetAttribute(max dynamic smem)");
    if (st) return st;
    if (w.cluster_size > 8) {
        st = cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                         "cudaFuncSetAttribute(non-portable cluster)");
        if (st) return st;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(w.n_clusters * w.cluster_size));
    cfg.blockDim = dim3((unsigned)w.threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)w.cluster_size;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (a.fx.enabled && a.fx.n_windows > 1) {
        // A resident launch's clusters wait for one another between windows:
        // a cooperative launch guarantees they are all resident at once (or
        // fails to launch).
        attr[1].id = cudaLaunchAttributeCooperative;
        attr[1].val.cooperative = 1;
        cfg.numAttrs = 2;
    }
    const cudaError_t err = cudaLaunchKernelEx(&cfg, kern, a);
    // A launch refused for its configuration (e.g. a cooperative grid too
    // large to be resident) is not sticky: clear it so later checks do not
    // report it again.
    if (err != cudaSuccess) (void)cudaGetLastError();
    return cuda_status(err, name);
}

// Whether the shared-memory stream variant fits next to a strip of `smem`
// bytes with `threads` threads: its streams take at most 64 bytes a thread
// (one plaquette of four colours), the bound both the variant choice and the
// occupancy query use.
inline bool smem_streams_fit(size_t smem, int threads)
{
    return smem + (size_t)64 * threads + 16 <= 232448;
}

// The variant a batch runs: the streams in registers when every strip fits,
// preferring the two-plaquette variant (compiled for fewer threads, so with
// the larger register budget) whenever the thread count allows it; else the
// global-memory streams, two visits in flight when the policy allows it and
// the CTA has at most kPairThreads threads (kGlobalPairVariant), one
// otherwise (NPMAX = 0).  A policy with kPairThreads = 0 has no
// two-plaquette variant.
template <class M>
int pick_npmax(const mcgb_batch_window &w)
{
    long long npl = 0;
    for (int k = 0; k < work_count(w); ++k) {
        const int L = w.host_table[work_replica(w, k)].L;
        const long long n = (long long)L * L / (4 * effective_cluster(L, w.cluster_size));
        if (n > npl) npl = n;
    }
    if (npl <= 2LL * w.threads && w.threads <= window_max_threads<M, 2>()) return 2;
    if (npl <= w.threads && w.threads <= window_max_threads<M, 1>() &&
        (!smem_stream_variant<M, 1>() || smem_streams_fit(batch_smem<M>(w, w.cluster_size), w.threads)))
        return 1;
    if (M::kGlobalInFlight == 2 && w.threads <= window_max_threads<M, kGlobalPairVariant>())
        return kGlobalPairVariant;
    return 0;
}

template <class M>
int launch_any(const BatchArgs &a, const mcgb_batch_window &w, cudaStream_t s, const char *name)
{
    MCGB_REQUIRE(w.threads <= M::kMaxThreads, "%s: at most %d threads per CTA", name, M::kMaxThreads);
    const int npmax = pick_npmax<M>(w);
    if constexpr (M::kRefLayout) {
        // The reference layout is indexed for the register and shared-memory
        // stream variants only.
        MCGB_REQUIRE(npmax == 1 || npmax == 2,
                     "%s: strips of at most two plaquettes per thread (more CTAs or threads per replica)", name);
    }
    switch (npmax) {
    case 1: return launch_window<M, 1>(a, w, s, name);
    case 2:
        if constexpr (M::kPairThreads > 0) return launch_window<M, 2>(a, w, s, name);
        return launch_window<M, 0>(a, w, s, name);
    case kGlobalPairVariant:
        if constexpr (M::kGlobalInFlight == 2) return launch_window<M, kGlobalPairVariant>(a, w, s, name);
        return launch_window<M, 0>(a, w, s, name);
    default: return launch_window<M, 0>(a, w, s, name);
    }
}

template <class M, int NPMAX>
int max_clusters_for(int C, int threads, size_t smem, int *out)
{
    auto kern = window_kernel<M, NPMAX>;
    // The shared-memory stream variant runs at most one plaquette a thread:
    // its streams take at most 64 bytes a thread more.
    if (smem_stream_variant<M, NPMAX>()) smem += (size_t)64 * threads + 16;
    int st = cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "cudaFuncSetAttribute(max dynamic smem)");
    if (st) return st;
    if (C > 8) {
        st = cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                         "cudaFuncSetAttribute(non-portable cluster)");
        if (st) return st;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(C * 256));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cuda_status(cudaOccupancyMaxActiveClusters(out, kern, &cfg), "cudaOccupancyMaxActiveClusters");
}

// Clusters resident at once for this shape, whichever variant the batch ends
// up running (the smallest count over the variants the thread count allows).
template <class M>
int max_clusters_any(int C, int threads, size_t smem, int *out)
{
    MCGB_REQUIRE(threads <= M::kMaxThreads, "at most %d threads per CTA for this model", M::kMaxThreads);
    int best = 0, n = 0;
    if constexpr (M::kRefLayout) {
        best = 1 << 30;  // the variants below only
    } else {
        if (int st = max_clusters_for<M, 0>(C, threads, smem, &best)) return st;
    }
    if (threads <= window_max_threads<M, 1>() && (!smem_stream_variant<M, 1>() || smem_streams_fit(smem, threads))) {
        if (int st = max_clusters_for<M, 1>(C, threads, smem, &n)) return st;
        if (n < best) best = n;
    }
    if constexpr (M::kPairThreads > 0) {
        if (threads <= window_max_threads<M, 2>()) {
            if (int st = max_clusters_for<M, 2>(C, threads, smem, &n)) return st;
            if (n < best) best = n;
        }
    }
    if constexpr (M::kGlobalInFlight == 2) {
        if (threads <= window_max_threads<M, kGlobalPairVariant>()) {
            if (int st = max_clusters_for<M, kGlobalPairVariant>(C, threads, smem, &n)) return st;
            if (n < best) best = n;
        }
    }
    *out = best == (1 << 30) ? 0 : best;
    return MCGB_OK;
}

// Colour-major plane index of site (i, j) of a replica of size L.
__host__ __device__ __forceinline__ int64_t cm_index(int i, int j, int L)
{
    const int LP = L >> 1;
    const int c = ((i & 1) << 1) | (j & 1);
    return (int64_t)c * LP * LP + (int64_t)(i >> 1) * LP + (j >> 1);
}

}  // namespace mcgb
