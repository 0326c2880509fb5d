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

__global__ void pt_exchange_kernel(const double *__restrict__ energies, float *__restrict__ betas,
                                   int32_t *__restrict__ w2t, int32_t *__restrict__ t2w,
                                   ulonglong2 *__restrict__ rng, long long *__restrict__ counts,
                                   long long *__restrict__ trips, int R, int parity, long long sweep)
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
