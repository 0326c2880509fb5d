// Parallel-tempering replica exchange on the device.
//
// core/parallel_tempering.py:35-91 _exchange_kernel: one thread block strides
// over the disjoint neighbouring-temperature pairs (left, left+1) of one
// parity; the float64 log ratio (beta_a - beta_b)(E_a - E_b) uses the float32
// betas promoted before subtracting; exchange stream `left` supplies a
// float64 uniform only when both energies are finite; an accepted swap
// exchanges the walkers' betas and both index maps (states never move).
// After a barrier every walker updates its round-trip bookkeeping.
#include "mcgb_common.cuh"

namespace mcgb {

// One exchange round of one thread block (every thread of the block calls it).
__device__ void exchange_round(const double *__restrict__ energies, float *__restrict__ betas,
                               int32_t *__restrict__ w2t, int32_t *__restrict__ t2w, ulonglong2 *__restrict__ rng,
                               long long *__restrict__ counts, long long *__restrict__ trips, int R, int parity,
                               long long sweep)
{
    const int tid = threadIdx.x;
    long long *attempts = counts, *accepted = counts + (R - 1), *nonfinite = counts + 2 * (R - 1);
    for (int left = parity + 2 * tid; left < R - 1; left += 2 * blockDim.x) {
        const int right = left + 1;
        const int a = t2w[left], b = t2w[right];
        const double ea = energies[a], eb = energies[b];
        attempts[left] += 1;
        if (!isfinite(ea) || !isfinite(eb)) {
            nonfinite[left] += 1;
            continue;
        }
        const double log_ratio = ((double)betas[a] - (double)betas[b]) * (ea - eb);
        ulonglong2 st = rng[left];
        const double u = xoro_uniform_f64(st);
        rng[left] = st;
        if (log_ratio >= 0.0 || u == 0.0 || log(u) < log_ratio) {
            t2w[left] = b;
            t2w[right] = a;
            w2t[a] = right;
            w2t[b] = left;
            const float ba = betas[a];
            betas[a] = betas[b];
            betas[b] = ba;
            accepted[left] += 1;
        }
    }
    __syncthreads();
    long long *origin = trips, *visited = trips + R, *start = trips + 2 * R, *ntrips = trips + 3 * R,
              *tsweeps = trips + 4 * R;
    for (int w = tid; w < R; w += blockDim.x) {
        const int t = w2t[w];
        if (t != 0 && t != R - 1) continue;
        const long long o = origin[w];
        if (o < 0) {
            origin[w] = t;
            start[w] = sweep;
        } else if (t != o) {
            visited[w] = 1;
        } else if (visited[w]) {
            ntrips[w] += 1;
            tsweeps[w] += sweep - start[w];
            start[w] = sweep;
            visited[w] = 0;
        }
    }
}

__global__ void pt_exchange_kernel(const double *__restrict__ energies, float *__restrict__ betas,
                                   int32_t *__restrict__ w2t, int32_t *__restrict__ t2w,
                                   ulonglong2 *__restrict__ rng, long long *__restrict__ counts,
                                   long long *__restrict__ trips, int R, int parity, long long sweep)
{
    exchange_round(energies, betas, w2t, t2w, rng, counts, trips, R, parity, sweep);
}

// The same round with the schedule read from a device clock {sweeps,
// rounds}: the round happens after clock[0] + advance sweeps, its parity is
// rounds % 2 (0 for a two-walker ladder), and the clock is left at
// {clock[0] + advance, rounds + 1}.  A replayed CUDA graph then runs each
// round at its own sweep and parity.
__global__ void pt_exchange_clocked_kernel(const double *__restrict__ energies, float *__restrict__ betas,
                                           int32_t *__restrict__ w2t, int32_t *__restrict__ t2w,
                                           ulonglong2 *__restrict__ rng, long long *__restrict__ counts,
                                           long long *__restrict__ trips, int R, long long *__restrict__ clock,
                                           int advance)
{
    __shared__ long long s_sweep, s_rounds;
    if (threadIdx.x == 0) {
        s_sweep = clock[0] + advance;
        s_rounds = clock[1];
    }
    __syncthreads();
    const int parity = R > 2 ? (int)(s_rounds & 1) : 0;
    exchange_round(energies, betas, w2t, t2w, rng, counts, trips, R, parity, s_sweep);
    if (threadIdx.x == 0) {
        clock[0] = s_sweep;
        clock[1] = s_rounds + 1;
    }
}

// Append `n` float64 values to slot head[0] % capacity of a ring of
// [capacity][n] values, then advance head[0] (one block).
__global__ void ring_push_f64_kernel(const double *__restrict__ src, double *__restrict__ ring,
                                     long long *__restrict__ head, long long n, long long capacity)
{
    __shared__ long long s_slot;
    if (threadIdx.x == 0) s_slot = head[0] % capacity;
    __syncthreads();
    double *dst = ring + s_slot * n;
    for (long long k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    if (threadIdx.x == 0) head[0] += 1;
}

// Append the row w2t[ids[k]], k < n, to a ring of [capacity][n] int32 rows.
__global__ void ring_push_walkers_kernel(const int32_t *__restrict__ w2t, const int32_t *__restrict__ ids,
                                         int32_t *__restrict__ ring, long long *__restrict__ head, int n,
                                         long long capacity)
{
    __shared__ long long s_slot;
    if (threadIdx.x == 0) s_slot = head[0] % capacity;
    __syncthreads();
    int32_t *dst = ring + s_slot * n;
    for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = w2t[ids[k]];
    __syncthreads();
    if (threadIdx.x == 0) head[0] += 1;
}

__global__ void pt_record_kernel(const int32_t *__restrict__ w2t, const int32_t *__restrict__ ids,
                                 int32_t *__restrict__ row, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) row[k] = w2t[ids[k]];
}

}  // namespace mcgb

using namespace mcgb;

extern "C" int mcgb_pt_exchange(const double *energies, float *betas, int32_t *w2t, int32_t *t2w, void *rng,
                                int64_t *swap_counts, int64_t *trips, int R, int parity, int64_t sweep,
                                void *stream)
{
    MCGB_REQUIRE(R >= 2, "pt_exchange: R must be >= 2");
    MCGB_REQUIRE(parity == 0 || parity == 1, "pt_exchange: parity must be 0 or 1");
    MCGB_REQUIRE(energies && betas && w2t && t2w && rng && swap_counts && trips, "pt_exchange: null pointer");
    pt_exchange_kernel<<<1, 128, 0, as_stream(stream)>>>(energies, betas, w2t, t2w, static_cast<ulonglong2 *>(rng),
                                                         reinterpret_cast<long long *>(swap_counts),
                                                         reinterpret_cast<long long *>(trips), R, parity,
                                                         (long long)sweep);
    return check_launch("pt_exchange_kernel");
}

extern "C" int mcgb_pt_record_walkers(const int32_t *w2t, const int32_t *ids, int32_t *row, int n, void *stream)
{
    MCGB_REQUIRE(n >= 0, "pt_record_walkers: n must be >= 0");
    if (n == 0) return MCGB_OK;
    MCGB_REQUIRE(w2t && ids && row, "pt_record_walkers: null pointer");
    pt_record_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(w2t, ids, row, n);
    return check_launch("pt_record_kernel");
}

extern "C" int mcgb_pt_exchange_clocked(const double *energies, float *betas, int32_t *w2t, int32_t *t2w, void *rng,
                                        int64_t *swap_counts, int64_t *trips, int R, int64_t *clock, int advance,
                                        void *stream)
{
    MCGB_REQUIRE(R >= 2, "pt_exchange_clocked: R must be >= 2");
    MCGB_REQUIRE(advance >= 0, "pt_exchange_clocked: advance must be >= 0");
    MCGB_REQUIRE(energies && betas && w2t && t2w && rng && swap_counts && trips && clock,
                 "pt_exchange_clocked: null pointer");
    pt_exchange_clocked_kernel<<<1, 128, 0, as_stream(stream)>>>(
        energies, betas, w2t, t2w, static_cast<ulonglong2 *>(rng), reinterpret_cast<long long *>(swap_counts),
        reinterpret_cast<long long *>(trips), R, reinterpret_cast<long long *>(clock), advance);
    return check_launch("pt_exchange_clocked_kernel");
}

extern "C" int mcgb_ring_push(const double *src, double *ring, int64_t *head, int64_t n, int64_t capacity,
                              void *stream)
{
    MCGB_REQUIRE(n >= 1 && capacity >= 1, "ring_push: n and capacity must be >= 1");
    MCGB_REQUIRE(src && ring && head, "ring_push: null pointer");
    ring_push_f64_kernel<<<1, 256, 0, as_stream(stream)>>>(src, ring, reinterpret_cast<long long *>(head), n,
                                                          capacity);
    return check_launch("ring_push_f64_kernel");
}

extern "C" int mcgb_pt_record_walkers_ring(const int32_t *w2t, const int32_t *ids, int32_t *ring, int64_t *head,
                                           int n, int64_t capacity, void *stream)
{
    MCGB_REQUIRE(n >= 1 && capacity >= 1, "pt_record_walkers_ring: n and capacity must be >= 1");
    MCGB_REQUIRE(w2t && ids && ring && head, "pt_record_walkers_ring: null pointer");
    ring_push_walkers_kernel<<<1, 128, 0, as_stream(stream)>>>(w2t, ids, ring, reinterpret_cast<long long *>(head),
                                                              n, capacity);
    return check_launch("ring_push_walkers_kernel");
}
