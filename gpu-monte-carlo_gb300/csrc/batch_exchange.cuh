// Per-ladder replica exchange of the batched engine, as a block-cooperative
// device function: the stand-alone exchange kernel runs it with one block per
// ladder, and the fused window kernel runs it in the CTA that finishes a
// ladder's last replica.
#pragma once

#include "batch_common.cuh"

namespace mcgb {

// core/parallel_tempering.py:35-91 on ladder-local indices.  Replicas of
// ladder l are [start, start + n); its exchange streams and swap counters are
// at pair offset start - l.
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

// Every thread of the block calls this with the same l.  Everything it reads
// may have been written earlier in the same launch by another CTA (the
// energies and staged samples of this window; in a resident launch, the maps,
// counters and streams of the previous window's exchange, which another CTA
// may have run), ordered by fences and completion counts: so every read goes
// past L1 (ld.global.cg).
__device__ __forceinline__ void exchange_ladder(const ExchangeArgs &x, int l)
{
    const int start = x.starts[l], R = x.sizes[l];
    const long long sweep = __ldcg(x.clock) + x.window_sweeps;
    const int parity = R > 2 ? (int)(__ldcg(x.clock + 1) & 1) : 0;
    const int poff = start - l;
    const double *E = x.energies + start;
    float *B = x.betas + start;
    int32_t *W2T = x.w2t + start, *T2W = x.t2w + start;
    long long *attempts = x.counts + poff, *accepted = x.counts + x.n_pairs_total + poff,
              *nonfinite = x.counts + 2 * x.n_pairs_total + poff;
    for (int left = parity + 2 * (int)threadIdx.x; left < R - 1; left += 2 * blockDim.x) {
        const int right = left + 1;
        const int a = __ldcg(T2W + left), b = __ldcg(T2W + right);
        const double ea = __ldcg(E + a), eb = __ldcg(E + b);
        attempts[left] = __ldcg(attempts + left) + 1;
        if (!isfinite(ea) || !isfinite(eb)) {
            nonfinite[left] = __ldcg(nonfinite + left) + 1;
            continue;
        }
        const float ba = __ldcg(B + a), bb = __ldcg(B + b);
        const double log_ratio = ((double)ba - (double)bb) * (ea - eb);
        ulonglong2 st = __ldcg(x.rng + poff + left);
        const double u = xoro_uniform_f64(st);
        x.rng[poff + left] = st;
        if (log_ratio >= 0.0 || u == 0.0 || log(u) < log_ratio) {
            T2W[left] = b;
            T2W[right] = a;
            W2T[a] = right;
            W2T[b] = left;
            B[a] = bb;
            B[b] = ba;
            accepted[left] = __ldcg(accepted + left) + 1;
        }
    }
    __syncthreads();
    const int n = x.n_replicas;
    long long *origin = x.trips + start, *visited = x.trips + n + start, *sweep0 = x.trips + 2 * n + start,
              *ntrips = x.trips + 3 * n + start, *tsweeps = x.trips + 4 * n + start;
    for (int wk = threadIdx.x; wk < R; wk += blockDim.x) {
        const int t = __ldcg(W2T + wk);
        if (t != 0 && t != R - 1) continue;
        const long long o = __ldcg(origin + wk);
        if (o < 0) {
            origin[wk] = t;
            sweep0[wk] = sweep;
        } else if (t != o) {
            visited[wk] = 1;
        } else if (__ldcg(visited + wk)) {
            ntrips[wk] = __ldcg(ntrips + wk) + 1;
            tsweeps[wk] = __ldcg(tsweeps + wk) + (sweep - __ldcg(sweep0 + wk));
            sweep0[wk] = sweep;
            visited[wk] = 0;
        }
    }
    if (x.staging != nullptr && x.samples != nullptr) {
        const int slot = sample_slot(sweep, x.first_sample_sweep, x.sample_interval, x.n_slots);
        if (slot >= 0) {
            for (int wk = threadIdx.x; wk < R; wk += blockDim.x) {
                const int dst = start + __ldcg(W2T + wk);
                for (int q = 0; q < x.channels; ++q)
                    x.samples[((size_t)slot * x.channels + q) * x.n_temps_total + dst] =
                        __ldcg(x.staging + (size_t)q * n + start + wk);
            }
        }
    }
    __syncthreads();
}

// Completion bookkeeping of the fused window + exchange launch.  `sync` holds
// one counter per ladder, one for the launch, the resident launch's window
// epoch and its error flag; the counters and the epoch are zero between
// launches.
struct FusedExchange {
    ExchangeArgs ex;
    int32_t *ladder_done;  // [n_ladders]
    int32_t *launch_done;  // [1]
    int32_t *epoch;        // [1] resident launches: windows completed so far
    int32_t *error;        // [1] set when a wait for the epoch gave up
    int enabled;
    int n_windows;         // > 1: a resident launch (one replica per cluster, cooperative)
};

}  // namespace mcgb
