// Batched engine: layout permutation, per-ladder replica exchange, Gaussian
// width tuning and the C-ABI dispatch of the window kernels.
#include "batch_args.cuh"

namespace mcgb {

int lattice_window(int model, const mcgb_batch_window &w, cudaStream_t s, const FusedExchange *fx = nullptr);
int64_t lattice_smem(int model, int max_L, int C);
int lattice_max_clusters(int model, int C, int threads, size_t smem, int *out);
int lattice_energy64(int model, const mcgb_batch_window &w, double *drift, cudaStream_t s);
int refresh_aux(const mcgb_batch_window &w, int stride, cudaStream_t s);
int continuum_window(int model, const mcgb_batch_window &w, cudaStream_t s, const FusedExchange *fx = nullptr);
int64_t continuum_smem(int model, int max_L, int C);
int continuum_max_clusters(int model, int C, int threads, size_t smem, int *out);
int continuum_energy64(int model, const mcgb_batch_window &w, double *drift, cudaStream_t s);

// One thread per site; grid.y = replica.  W is the copy word type.
template <typename W>
__global__ void permute_kernel(const W *__restrict__ src, W *__restrict__ dst, int words,
                               const mcgb_replica *__restrict__ table, const int64_t *__restrict__ ref_off,
                               int direction)
{
    const int r = blockIdx.y;
    const mcgb_replica rep = table[r];
    const int L = rep.L;
    const int64_t n = (int64_t)L * L;
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = (int)(k / L), j = (int)(k - (int64_t)i * L);
    const int64_t ref = ref_off[r] + k;
    const int64_t cm = rep.state_offset + cm_index(i, j, L);
    const int64_t from = direction == 0 ? ref : cm, to = direction == 0 ? cm : ref;
    for (int q = 0; q < words; ++q) dst[to * words + q] = src[from * words + q];
}

// One block per ladder.
__global__ void batch_exchange_kernel(const ExchangeArgs x) { exchange_ladder(x, blockIdx.x); }

__global__ void clock_tick_kernel(long long *clock, int n_sweeps, int exchanged)
{
    clock[0] += n_sweeps;
    clock[1] += exchanged;
}

__global__ void tune_sigma_kernel(float *sigma_t, const long long *accepted, long long *prev, const int32_t *w2t,
                                  const mcgb_replica *table, int n, int n_sweeps, float target, float gain,
                                  float lo, float hi)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const mcgb_replica rep = table[r];
    const long long d = accepted[r] - prev[r];
    prev[r] = accepted[r];
    const double rate = (double)d / ((double)rep.L * rep.L * (double)n_sweeps);
    const int slot = rep.ladder_start + w2t[r];
    float sg = sigma_t[slot] * expf(gain * (float)(rate - target));
    sigma_t[slot] = fminf(fmaxf(sg, lo), hi);
}

}  // namespace mcgb

using namespace mcgb;

static bool is_lattice(int model)
{
    return model == MCGB_MODEL_ISING || model == MCGB_MODEL_XY || model == MCGB_MODEL_ISING_REF ||
           model == MCGB_MODEL_XY_REF;
}
static bool known_model(int model) { return model >= MCGB_MODEL_ISING && model <= MCGB_MODEL_XY_REF; }
// Models of the batch arrays; the reference-layout ones take windows only.
static bool batch_model(int model) { return model >= MCGB_MODEL_ISING && model <= MCGB_MODEL_KAWAMURA_GAUSS; }

extern "C" int mcgb_batch_channels(int model)
{
    switch (model) {
    case MCGB_MODEL_ISING: return 2;
    case MCGB_MODEL_XY: return 5;
    case MCGB_MODEL_KAWAMURA:
    case MCGB_MODEL_KAWAMURA_GAUSS: return 7;
    case MCGB_MODEL_HE3:
    case MCGB_MODEL_HE3_GAUSS: return 10;
    default: set_error("unknown model %d", model); return MCGB_EINVAL;
    }
}

extern "C" int64_t mcgb_batch_smem_bytes(int model, int L, int cluster_size)
{
    MCGB_REQUIRE(known_model(model), "unknown model %d", model);
    MCGB_REQUIRE(cluster_size >= 1 && cluster_size <= 16, "cluster_size must be 1..16");
    MCGB_REQUIRE(L >= 4 && L % 2 == 0, "L must be even and >= 4");
    return is_lattice(model) ? lattice_smem(model, L, cluster_size) : continuum_smem(model, L, cluster_size);
}

extern "C" int mcgb_batch_max_clusters(int model, int cluster_size, int threads, int64_t smem_bytes, int *out)
{
    MCGB_REQUIRE(known_model(model), "unknown model %d", model);
    MCGB_REQUIRE(out != nullptr, "max_clusters: null output");
    MCGB_REQUIRE(cluster_size >= 1 && cluster_size <= 16, "cluster_size must be 1..16");
    MCGB_REQUIRE(threads >= 32 && threads <= 1024 && threads % 32 == 0, "bad thread count");
    MCGB_REQUIRE(smem_bytes > 0 && smem_bytes <= 232448, "bad shared memory size");
    return is_lattice(model) ? lattice_max_clusters(model, cluster_size, threads, (size_t)smem_bytes, out)
                             : continuum_max_clusters(model, cluster_size, threads, (size_t)smem_bytes, out);
}

extern "C" int mcgb_batch_window_run(int model, const mcgb_batch_window *w, void *stream)
{
    MCGB_REQUIRE(known_model(model), "unknown model %d", model);
    MCGB_REQUIRE(w != nullptr, "batch window: null argument block");
    if (model == MCGB_MODEL_XY) MCGB_REQUIRE(w->J > 0, "XY: J must be positive");
    if (model == MCGB_MODEL_HE3_GAUSS) MCGB_REQUIRE(w->counters != nullptr, "He3 Gaussian: null counters");
    if (model == MCGB_MODEL_KAWAMURA_GAUSS) MCGB_REQUIRE(w->sigma_t != nullptr, "Kawamura Gaussian: null widths");
    return is_lattice(model) ? lattice_window(model, *w, as_stream(stream))
                             : continuum_window(model, *w, as_stream(stream));
}

extern "C" int mcgb_batch_recompute_energy(int model, const mcgb_batch_window *w, double *drift, void *stream)
{
    MCGB_REQUIRE(batch_model(model), "unknown batch model %d", model);
    MCGB_REQUIRE(w && w->table && w->state && w->e_run && w->energies && w->n_replicas >= 1,
                 "recompute_energy: null pointer");
    return is_lattice(model) ? lattice_energy64(model, *w, drift, as_stream(stream))
                             : continuum_energy64(model, *w, drift, as_stream(stream));
}

extern "C" int mcgb_batch_refresh_aux(int model, const mcgb_batch_window *w, void *stream)
{
    MCGB_REQUIRE(w != nullptr, "refresh_aux: null argument block");
    if (model == MCGB_MODEL_XY) return refresh_aux(*w, 1, as_stream(stream));
    if (model == MCGB_MODEL_KAWAMURA || model == MCGB_MODEL_KAWAMURA_GAUSS) return refresh_aux(*w, 5, as_stream(stream));
    return MCGB_OK;
}

extern "C" int mcgb_batch_permute(const void *src, void *dst, int64_t elem_bytes, const mcgb_replica *table,
                                  const int64_t *ref_offsets, int n_replicas, int max_L, int direction, void *stream)
{
    MCGB_REQUIRE(src && dst && table && ref_offsets, "permute: null pointer");
    MCGB_REQUIRE(n_replicas >= 1 && n_replicas <= 65535, "permute: n_replicas must be 1..65535");
    MCGB_REQUIRE(max_L >= 4 && max_L % 2 == 0, "permute: bad max_L");
    MCGB_REQUIRE(direction == 0 || direction == 1, "permute: direction must be 0 or 1");
    MCGB_REQUIRE(elem_bytes >= 1, "permute: bad element size");
    const int64_t n = (int64_t)max_L * max_L;
    dim3 grid((unsigned)((n + 255) / 256), (unsigned)n_replicas);
    cudaStream_t s = as_stream(stream);
    if (elem_bytes % 16 == 0)
        permute_kernel<uint4><<<grid, 256, 0, s>>>(static_cast<const uint4 *>(src), static_cast<uint4 *>(dst),
                                                   (int)(elem_bytes / 16), table, ref_offsets, direction);
    else if (elem_bytes % 4 == 0)
        permute_kernel<uint32_t><<<grid, 256, 0, s>>>(static_cast<const uint32_t *>(src), static_cast<uint32_t *>(dst),
                                                      (int)(elem_bytes / 4), table, ref_offsets, direction);
    else
        permute_kernel<uint8_t><<<grid, 256, 0, s>>>(static_cast<const uint8_t *>(src), static_cast<uint8_t *>(dst),
                                                     (int)elem_bytes, table, ref_offsets, direction);
    return check_launch("permute_kernel");
}

extern "C" int mcgb_batch_exchange(const mcgb_batch_window *w, const mcgb_batch_pt *pt, void *stream)
{
    MCGB_REQUIRE(w && pt, "batch_exchange: null argument block");
    if (int st = check_exchange(*w, *pt)) return st;
    batch_exchange_kernel<<<pt->n_ladders, 128, 0, as_stream(stream)>>>(make_exchange_args(*w, *pt));
    return check_launch("batch_exchange_kernel");
}

extern "C" int mcgb_batch_window_exchange(int model, const mcgb_batch_window *w, const mcgb_batch_pt *pt,
                                          int32_t *sync, void *stream)
{
    MCGB_REQUIRE(batch_model(model), "unknown batch model %d", model);
    MCGB_REQUIRE(w && pt, "window_exchange: null argument block");
    MCGB_REQUIRE(sync != nullptr, "window_exchange: null sync counters");
    if (int st = check_exchange(*w, *pt)) return st;
    if (model == MCGB_MODEL_XY) MCGB_REQUIRE(w->J > 0, "XY: J must be positive");
    if (model == MCGB_MODEL_HE3_GAUSS) MCGB_REQUIRE(w->counters != nullptr, "He3 Gaussian: null counters");
    if (model == MCGB_MODEL_KAWAMURA_GAUSS) MCGB_REQUIRE(w->sigma_t != nullptr, "Kawamura Gaussian: null widths");
    MCGB_REQUIRE((reinterpret_cast<uintptr_t>(sync) & 15) == 0, "window_exchange: sync must be 16-byte aligned");
    MCGB_REQUIRE(pt->channels <= 32, "window_exchange: at most 32 sample channels");
    const FusedExchange fx = make_fused(make_exchange_args(*w, *pt), sync, 1, w->hold_clock, kWaitSpinLimit);
    return is_lattice(model) ? lattice_window(model, *w, as_stream(stream), &fx)
                             : continuum_window(model, *w, as_stream(stream), &fx);
}

static long long g_wait_limit = kWaitSpinLimit;

extern "C" int64_t mcgb_batch_set_wait_limit(int64_t polls)
{
    const long long old = g_wait_limit;
    g_wait_limit = polls < 0 ? kWaitSpinLimit : polls;
    return old;
}

extern "C" int mcgb_batch_run_resident(int model, const mcgb_batch_window *w, const mcgb_batch_pt *pt,
                                       int32_t *sync, int n_windows, void *stream)
{
    MCGB_REQUIRE(batch_model(model), "unknown batch model %d", model);
    MCGB_REQUIRE(w && pt, "run_resident: null argument block");
    MCGB_REQUIRE(sync != nullptr, "run_resident: null sync counters");
    MCGB_REQUIRE(n_windows >= 1, "run_resident: n_windows must be >= 1");
    MCGB_REQUIRE((long long)n_windows * w->n_sweeps <= kMaxLaunchSweeps,
                 "run_resident: at most %lld sweeps a launch", kMaxLaunchSweeps);
    MCGB_REQUIRE(n_windows == 1 || w->n_clusters == work_count(*w),
                 "run_resident: a resident launch needs one cluster per replica it runs");
    if (int st = check_exchange(*w, *pt)) return st;
    if (model == MCGB_MODEL_XY) MCGB_REQUIRE(w->J > 0, "XY: J must be positive");
    if (model == MCGB_MODEL_HE3_GAUSS) MCGB_REQUIRE(w->counters != nullptr, "He3 Gaussian: null counters");
    if (model == MCGB_MODEL_KAWAMURA_GAUSS) MCGB_REQUIRE(w->sigma_t != nullptr, "Kawamura Gaussian: null widths");
    MCGB_REQUIRE((reinterpret_cast<uintptr_t>(sync) & 15) == 0, "run_resident: sync must be 16-byte aligned");
    MCGB_REQUIRE(pt->channels <= 32, "run_resident: at most 32 sample channels");
    const FusedExchange fx = make_fused(make_exchange_args(*w, *pt), sync, n_windows, w->hold_clock, g_wait_limit);
    return is_lattice(model) ? lattice_window(model, *w, as_stream(stream), &fx)
                             : continuum_window(model, *w, as_stream(stream), &fx);
}

extern "C" int mcgb_batch_clock_tick(int64_t *clock, int n_sweeps, int exchanged, void *stream)
{
    MCGB_REQUIRE(clock != nullptr, "clock_tick: null clock");
    MCGB_REQUIRE(n_sweeps >= 0 && (exchanged == 0 || exchanged == 1), "clock_tick: bad arguments");
    clock_tick_kernel<<<1, 1, 0, as_stream(stream)>>>(reinterpret_cast<long long *>(clock), n_sweeps, exchanged);
    return check_launch("clock_tick_kernel");
}

extern "C" int mcgb_batch_tune_sigma(float *sigma_t, const long long *accepted, long long *accepted_prev,
                                     const int32_t *w2t, const mcgb_replica *table, int n_replicas, int n_sweeps,
                                     float target, float gain, float lo, float hi, void *stream)
{
    MCGB_REQUIRE(sigma_t && accepted && accepted_prev && w2t && table, "tune_sigma: null pointer");
    MCGB_REQUIRE(n_replicas >= 1 && n_sweeps >= 1, "tune_sigma: bad sizes");
    MCGB_REQUIRE(lo > 0 && hi >= lo, "tune_sigma: bad clamp range");
    tune_sigma_kernel<<<(n_replicas + 127) / 128, 128, 0, as_stream(stream)>>>(
        sigma_t, accepted, accepted_prev, w2t, table, n_replicas, n_sweeps, target, gain, lo, hi);
    return check_launch("tune_sigma_kernel");
}
