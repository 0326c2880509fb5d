// Batched engine: layout permutation, per-ladder replica exchange, Gaussian
// width tuning and the C-ABI dispatch of the window kernels.
#include "batch_args.cuh"

namespace mcgb {

int lattice_window(int model, const mcgb_batch_window &w, cudaStream_t s);
int64_t lattice_smem(int model, int max_L, int C);
int lattice_max_clusters(int model, int C, int threads, size_t smem, int *out);
int lattice_energy64(int model, const mcgb_batch_window &w, double *drift, cudaStream_t s);
int refresh_aux(const mcgb_batch_window &w, int stride, cudaStream_t s);
int continuum_window(int model, const mcgb_batch_window &w, cudaStream_t s);
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

// One block per ladder: core/parallel_tempering.py:35-91 on ladder-local
// indices.  Replicas of ladder l are [start, start + n); its exchange streams
// and swap counters are at pair offset start - l.
struct ExchangeArgs {
    const double *energies;
    float *betas;
    int32_t *w2t, *t2w;
    ulonglong2 *rng;
    long long *counts, *trips;
    const int32_t *starts, *sizes;
    int n_pairs_total, n_replicas;
    const long long *clock;
    int window_sweeps;
    // deferred window-end sample
    double *samples;
    const double *staging;
    int channels, n_temps_total, n_slots, sample_interval;
    long long first_sample_sweep;
};

__global__ void batch_exchange_kernel(const ExchangeArgs x)
{
    const int l = blockIdx.x;
    const int start = x.starts[l], R = x.sizes[l];
    const long long sweep = x.clock[0] + x.window_sweeps;
    const int parity = R > 2 ? (int)(x.clock[1] & 1) : 0;
    const int poff = start - l;
    const double *E = x.energies + start;
    float *B = x.betas + start;
    int32_t *W2T = x.w2t + start, *T2W = x.t2w + start;
    long long *attempts = x.counts + poff, *accepted = x.counts + x.n_pairs_total + poff,
              *nonfinite = x.counts + 2 * x.n_pairs_total + poff;
    for (int left = parity + 2 * (int)threadIdx.x; left < R - 1; left += 2 * blockDim.x) {
        const int right = left + 1;
        const int a = T2W[left], b = T2W[right];
        const double ea = E[a], eb = E[b];
        attempts[left] += 1;
        if (!isfinite(ea) || !isfinite(eb)) {
            nonfinite[left] += 1;
            continue;
        }
        const double log_ratio = ((double)B[a] - (double)B[b]) * (ea - eb);
        ulonglong2 st = x.rng[poff + left];
        const double u = xoro_uniform_f64(st);
        x.rng[poff + left] = st;
        if (log_ratio >= 0.0 || u == 0.0 || log(u) < log_ratio) {
            T2W[left] = b;
            T2W[right] = a;
            W2T[a] = right;
            W2T[b] = left;
            const float ba = B[a];
            B[a] = B[b];
            B[b] = ba;
            accepted[left] += 1;
        }
    }
    __syncthreads();
    const int n = x.n_replicas;
    long long *origin = x.trips + start, *visited = x.trips + n + start, *sweep0 = x.trips + 2 * n + start,
              *ntrips = x.trips + 3 * n + start, *tsweeps = x.trips + 4 * n + start;
    for (int wk = threadIdx.x; wk < R; wk += blockDim.x) {
        const int t = W2T[wk];
        if (t != 0 && t != R - 1) continue;
        const long long o = origin[wk];
        if (o < 0) {
            origin[wk] = t;
            sweep0[wk] = sweep;
        } else if (t != o) {
            visited[wk] = 1;
        } else if (visited[wk]) {
            ntrips[wk] += 1;
            tsweeps[wk] += sweep - sweep0[wk];
            sweep0[wk] = sweep;
            visited[wk] = 0;
        }
    }
    if (x.staging != nullptr && x.samples != nullptr) {
        const int slot = sample_slot(sweep, x.first_sample_sweep, x.sample_interval, x.n_slots);
        if (slot >= 0) {
            for (int wk = threadIdx.x; wk < R; wk += blockDim.x) {
                const int dst = start + W2T[wk];
                for (int q = 0; q < x.channels; ++q)
                    x.samples[((size_t)slot * x.channels + q) * x.n_temps_total + dst] =
                        x.staging[(size_t)q * n + start + wk];
            }
        }
    }
}

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

static bool is_lattice(int model) { return model == MCGB_MODEL_ISING || model == MCGB_MODEL_XY; }
static bool known_model(int model) { return model >= MCGB_MODEL_ISING && model <= MCGB_MODEL_HE3_GAUSS; }

extern "C" int mcgb_batch_channels(int model)
{
    switch (model) {
    case MCGB_MODEL_ISING: return 2;
    case MCGB_MODEL_XY: return 5;
    case MCGB_MODEL_KAWAMURA: return 7;
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
    return is_lattice(model) ? lattice_window(model, *w, as_stream(stream))
                             : continuum_window(model, *w, as_stream(stream));
}

extern "C" int mcgb_batch_recompute_energy(int model, const mcgb_batch_window *w, double *drift, void *stream)
{
    MCGB_REQUIRE(known_model(model), "unknown model %d", model);
    MCGB_REQUIRE(w && w->table && w->state && w->e_run && w->energies && w->n_replicas >= 1,
                 "recompute_energy: null pointer");
    return is_lattice(model) ? lattice_energy64(model, *w, drift, as_stream(stream))
                             : continuum_energy64(model, *w, drift, as_stream(stream));
}

extern "C" int mcgb_batch_refresh_aux(int model, const mcgb_batch_window *w, void *stream)
{
    MCGB_REQUIRE(w != nullptr, "refresh_aux: null argument block");
    if (model == MCGB_MODEL_XY) return refresh_aux(*w, 1, as_stream(stream));
    if (model == MCGB_MODEL_KAWAMURA) return refresh_aux(*w, 5, as_stream(stream));
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
    MCGB_REQUIRE(w->energies && w->betas && w->w2t && w->clock && pt->t2w && pt->rng && pt->swap_counts &&
                     pt->trips && pt->ladder_starts && pt->ladder_sizes,
                 "batch_exchange: null pointer");
    MCGB_REQUIRE(pt->n_ladders >= 1 && w->n_replicas >= 2 * pt->n_ladders,
                 "batch_exchange: every ladder needs >= 2 replicas");
    MCGB_REQUIRE(w->n_sweeps >= 0, "batch_exchange: n_sweeps must be >= 0");
    MCGB_REQUIRE(w->staging == nullptr || (w->samples && pt->channels >= 1 && w->n_temps_total >= w->n_replicas),
                 "batch_exchange: bad staging buffer");
    ExchangeArgs x;
    x.energies = w->energies;
    x.betas = const_cast<float *>(w->betas);
    x.w2t = const_cast<int32_t *>(w->w2t);
    x.t2w = pt->t2w;
    x.rng = static_cast<ulonglong2 *>(pt->rng);
    x.counts = reinterpret_cast<long long *>(pt->swap_counts);
    x.trips = reinterpret_cast<long long *>(pt->trips);
    x.starts = pt->ladder_starts;
    x.sizes = pt->ladder_sizes;
    x.n_pairs_total = w->n_replicas - pt->n_ladders;
    x.n_replicas = w->n_replicas;
    x.clock = reinterpret_cast<const long long *>(w->clock);
    x.window_sweeps = w->n_sweeps;
    x.samples = w->samples;
    x.staging = w->staging;
    x.channels = pt->channels;
    x.n_temps_total = w->n_temps_total;
    x.n_slots = w->n_slots;
    x.sample_interval = w->sample_interval;
    x.first_sample_sweep = w->first_sample_sweep;
    batch_exchange_kernel<<<pt->n_ladders, 128, 0, as_stream(stream)>>>(x);
    return check_launch("batch_exchange_kernel");
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
