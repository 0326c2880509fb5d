// Per-ladder replica exchange of the batched engine, as a block-cooperative
// device function the stand-alone exchange kernel runs with one block per
// ladder, and the bookkeeping of the fused window kernel, which decides the
// same matching pair by pair (batch_window.cuh).
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
// Ladders of at most 32 temperatures: one warp, walker `lane` per lane.  All
// reads go out in one round trip; each pair's left lane decides, and the
// maps, betas, round-trip bookkeeping and the staged sample follow from the
// decisions by shuffles.  The same result as the general path below, with
// one memory round trip on the critical path instead of five.
constexpr int kWarpLadderChannels = 16;

__device__ __forceinline__ void exchange_ladder_warp(const ExchangeArgs &x, int l, int start, int R,
                                                     long long sweep, int parity)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int poff = start - l, n = x.n_replicas, np = x.n_pairs_total;
    const bool in = lane < R;
    // Slot roles: a left slot starts a pair of this round's matching.
    const bool left = in && lane >= parity && ((lane - parity) & 1) == 0 && lane < R - 1;
    const bool right = in && lane >= 1 + parity && ((lane - 1 - parity) & 1) == 0;

    // -- the one round of loads --
    const int t2w = in ? __ldcg(x.t2w + start + lane) : 0;       // walker at slot `lane`
    const int s = in ? __ldcg(x.w2t + start + lane) : 0;         // slot of walker `lane`
    const double e = in ? __ldcg(x.energies + start + lane) : 0.0;
    const float b = in ? __ldcg(x.betas + start + lane) : 0.0f;
    long long att = 0, acc = 0, nonf = 0;
    ulonglong2 st = make_ulonglong2(0, 0);
    if (left) {
        att = __ldcg(x.counts + poff + lane);
        acc = __ldcg(x.counts + np + poff + lane);
        nonf = __ldcg(x.counts + 2 * np + poff + lane);
        st = __ldcg(x.rng + poff + lane);
    }
    long long *tr = x.trips + start + lane;
    long long origin = 0, visited = 0, sweep0 = 0, ntrips = 0, tsweeps = 0;
    if (in) {
        origin = __ldcg(tr);
        visited = __ldcg(tr + n);
        sweep0 = __ldcg(tr + 2 * n);
        ntrips = __ldcg(tr + 3 * n);
        tsweeps = __ldcg(tr + 4 * n);
    }
    const bool scatter = x.staging != nullptr && x.samples != nullptr;
    const int slot = scatter ? sample_slot(sweep, x.first_sample_sweep, x.sample_interval, x.n_slots) : -1;
    double stg[kWarpLadderChannels];
#pragma unroll
    for (int q = 0; q < kWarpLadderChannels; ++q)
        stg[q] = (in && slot >= 0 && q < x.channels) ? __ldcg(x.staging + (size_t)q * n + start + lane) : 0.0;

    // -- decisions (left lanes), as in the general path --
    const int bw = __shfl_sync(full, t2w, (lane + 1) & 31);
    const double ea = __shfl_sync(full, e, t2w & 31), eb = __shfl_sync(full, e, bw & 31);
    const float ba = __shfl_sync(full, b, t2w & 31), bb = __shfl_sync(full, b, bw & 31);
    int swapped = 0;
    if (left) {
        att += 1;
        if (!isfinite(ea) || !isfinite(eb)) {
            nonf += 1;
        } else {
            const double log_ratio = ((double)ba - (double)bb) * (ea - eb);
            const double u = xoro_uniform_f64(st);
            if (log_ratio >= 0.0 || u == 0.0 || log(u) < log_ratio) {
                swapped = 1;
                acc += 1;
            }
        }
    }

    // -- new maps and betas --
    const int sw_prev = __shfl_sync(full, swapped, (lane + 31) & 31);
    const int t2w_prev = __shfl_sync(full, t2w, (lane + 31) & 31);
    int t2w_new = t2w;
    if (left && swapped) t2w_new = bw;
    if (right && sw_prev) t2w_new = t2w_prev;
    // walker `lane` sits at slot s: its pair starts at s (left) or s - 1 (right)
    const bool s_left = s >= parity && ((s - parity) & 1) == 0 && s < R - 1;
    const bool s_right = s >= 1 + parity && ((s - 1 - parity) & 1) == 0;
    const int q0 = s_left ? s : (s_right ? s - 1 : 0);
    const int swq = __shfl_sync(full, swapped, q0 & 31);
    const int partner_slot = s_left ? s + 1 : (s_right ? s - 1 : s);
    const int partner = __shfl_sync(full, t2w, partner_slot & 31);
    const float b_partner = __shfl_sync(full, b, partner & 31);
    const bool moved = in && (s_left || s_right) && swq;
    const int w2t_new = moved ? (s_left ? s + 1 : s - 1) : s;
    const float b_new = moved ? b_partner : b;

    // -- stores --
    if (in) {
        x.t2w[start + lane] = t2w_new;
        x.w2t[start + lane] = w2t_new;
        x.betas[start + lane] = b_new;
    }
    if (left) {
        x.counts[poff + lane] = att;
        x.counts[np + poff + lane] = acc;
        x.counts[2 * np + poff + lane] = nonf;
        x.rng[poff + lane] = st;
    }
    if (in && (w2t_new == 0 || w2t_new == R - 1)) {
        const int t = w2t_new;
        if (origin < 0) {
            tr[0] = t;
            tr[2 * n] = sweep;
        } else if (t != origin) {
            tr[n] = 1;
        } else if (visited) {
            tr[3 * n] = ntrips + 1;
            tr[4 * n] = tsweeps + (sweep - sweep0);
            tr[2 * n] = sweep;
            tr[n] = 0;
        }
    }
    if (in && slot >= 0) {
        double *out = x.samples + (size_t)slot * x.channels * x.n_temps_total + start + w2t_new;
#pragma unroll
        for (int q = 0; q < kWarpLadderChannels; ++q)
            if (q < x.channels) out[(size_t)q * x.n_temps_total] = stg[q];
    }
}

__device__ __forceinline__ void exchange_ladder(const ExchangeArgs &x, int l)
{
    const int start = x.starts[l], R = x.sizes[l];
    const long long sweep = __ldcg(x.clock) + x.window_sweeps;
    const int parity = R > 2 ? (int)(__ldcg(x.clock + 1) & 1) : 0;
    if (R <= 32 && x.channels <= kWarpLadderChannels) {
        if (threadIdx.x < 32) exchange_ladder_warp(x, l, start, R, sweep, parity);
        __syncthreads();
        return;
    }
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

// Bookkeeping of the fused window + exchange launch, carved out of one int32
// array `sync` of 5 * n_replicas + 2 entries (16-byte aligned, zero before
// the first launch):
//   mailbox [n_replicas] x 16 B  per pair, at its left global slot: empty
//                                (zero) or the first walker's post -- energy
//                                (double), then beta (float bits, low word)
//                                and 0x80000000 | local walker id (high word)
//   decided [n_replicas]         per pair: (round tag << 1) | swapped
//   launch_done [1], error [1]
struct FusedExchange {
    ExchangeArgs ex;
    double2 *mailbox;
    int32_t *decided;
    int32_t *launch_done;
    int32_t *error;        // set when a wait for a pair's decision gave up
    int enabled;
    int n_windows;         // > 1: a resident launch (one replica per cluster, cooperative)
    int hold_clock;        // another launch of the same windows advances the clock
    long long wait_limit;  // polls of a pair's decision before a wait gives up
};

inline FusedExchange make_fused(const ExchangeArgs &ex, int32_t *sync, int n_windows, int hold_clock,
                                long long wait_limit)
{
    const int n = ex.n_replicas;
    FusedExchange fx;
    fx.ex = ex;
    fx.mailbox = reinterpret_cast<double2 *>(sync);
    fx.decided = sync + 4ll * n;
    fx.launch_done = sync + 5ll * n;
    fx.error = sync + 5ll * n + 1;
    fx.enabled = 1;
    fx.n_windows = n_windows;
    fx.hold_clock = hold_clock;
    fx.wait_limit = wait_limit;
    return fx;
}

}  // namespace mcgb
