// Shared pieces of the batched ("ladder batch") engine.
//
// A batch is a table of replicas of possibly different L (mcgb_replica).  One
// launch runs a window of sweeps over every replica: a thread-block cluster
// of C CTAs owns one replica at a time, each CTA a strip of L/C rows, and a
// cluster walks its list of replicas (longest-processing-time order, built by
// the host).  Inside a window the state lives in shared memory and the RNG
// streams in registers, so HBM is touched once per window, not per sweep.
//
// Layout in HBM ("colour-major"): per replica, four planes, one per
// checkerboard colour c = 2*(i%2) + (j%2); plane c holds the sites
// (i, j) = (2*pr + c/2, 2*pc + c%2) in (pr, pc) row-major order, L/2 x L/2.
// The RNG array uses the same site order, so site (i, j) of replica r keeps
// the stream it has in the reference layout (r*L*L + i*L + j) after the
// permutation kernels convert between the two layouts.
//
// Neighbours of a colour-c site at plaquette (pr, pc), as (plane, dpr, dpc):
//   c=0: up (2,-1,0)  down (2,0,0)  left (1,0,-1) right (1,0,0)
//   c=1: up (3,-1,0)  down (3,0,0)  left (0,0,0)  right (0,0,+1)
//   c=2: up (0,0,0)   down (0,+1,0) left (3,0,-1) right (3,0,0)
//   c=3: up (1,0,0)   down (1,+1,0) left (2,0,0)  right (2,0,+1)
// Columns wrap within the strip (strips are whole rows); rows outside the
// strip are halo rows kept up to date by the neighbouring CTAs.
#pragma once

#include <cooperative_groups.h>

#include "mcgb_common.cuh"

namespace mcgb {

namespace cg = cooperative_groups;

// Plane and plaquette-row/column offsets of a neighbour.
struct NbrSpec {
    int plane, dpr, dpc;
};

// Knuth TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Kahan-style compensated accumulation of float terms (sum, comp).
__device__ __forceinline__ void comp_add(float &sum, float &comp, float x)
{
    float s, e;
    two_sum(sum, x, s, e);
    sum = s;
    comp += e;
}

// A compensated float32 sum hi + lo (about 48 significant bits; exact for
// integer terms).  The in-window sample reductions accumulate in these so
// they run on the FP32 pipe: GB300's float64 pipe issues a small fraction of
// the FP32 rate, and a per-site float64 accumulation dominated the cost of
// taking a sample.
struct FSum {
    float hi, lo;
    __device__ __forceinline__ FSum() : hi(0.0f), lo(0.0f) {}
    __device__ __forceinline__ FSum &operator+=(float x)
    {
        comp_add(hi, lo, x);
        return *this;
    }
    __device__ __forceinline__ void merge(float h, float l)
    {
        float s, e;
        two_sum(hi, h, s, e);
        hi = s;
        lo += l + e;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Warp reduce-scatter of P compensated sums (P a power of two <= 32): each of
// the first log2(P) shuffle levels halves the values a lane carries (the
// lane whose offset bit is set keeps the upper half and sends the lower),
// plain butterfly levels finish.  Lane l ends with the warp total of value
// l >> (5 - log2 P), in every lane of its group.  18 shuffles for 8 sums
// where one butterfly per sum takes 80.
template <int P>
__device__ __forceinline__ void warp_reduce_scatter(FSum (&u)[P], int lane)
{
    static_assert(P >= 1 && P <= 32 && (P & (P - 1)) == 0, "P must be a power of two <= 32");
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int half = P / 2, o = 16; half >= 1; half >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < half; ++k) {
            FSum keep = up ? u[k + half] : u[k];
            const FSum send = up ? u[k] : u[k + half];
            keep.merge(__shfl_xor_sync(full, send.hi, o), __shfl_xor_sync(full, send.lo, o));
            u[k] = keep;
        }
    }
#pragma unroll
    for (int o = 16 / P; o >= 1; o >>= 1) u[0].merge(__shfl_xor_sync(full, u[0].hi, o), __shfl_xor_sync(full, u[0].lo, o));
}

template <int N>
struct Pow2Ceil {
    static constexpr int value = N <= 1 ? 1 : 2 * Pow2Ceil<(N + 1) / 2>::value;
};
template <>
struct Pow2Ceil<1> {
    static constexpr int value = 1;
};

// Block reduction of N compensated sums (N <= 32) by warp reduce-scatters,
// the totals written to dst[0..N) by the lanes of warp 0 that hold them (a
// DSMEM address works).  `scratch` holds 32 * N float2.  All threads call;
// the same threads, values and order give the same bits every time.
template <int N>
__device__ __forceinline__ void block_fsum_push(const FSum (&v)[N], float2 *scratch, float2 *dst)
{
    constexpr int P = Pow2Ceil<N>::value;
    constexpr int shift = P == 1 ? 5 : (P == 2 ? 4 : (P == 4 ? 3 : (P == 8 ? 2 : (P == 16 ? 1 : 0))));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    FSum u[P];
#pragma unroll
    for (int q = 0; q < N; ++q) u[q] = v[q];
    warp_reduce_scatter<P>(u, lane);
    const int j = lane >> shift;
    if ((lane & ((1 << shift) - 1)) == 0 && j < N) scratch[j * 32 + warp] = make_float2(u[0].hi, u[0].lo);
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const float2 x = (q < N && lane < nwarps) ? scratch[q * 32 + lane] : make_float2(0.0f, 0.0f);
            u[q].hi = x.x;
            u[q].lo = x.y;
        }
        warp_reduce_scatter<P>(u, lane);
        if ((lane & ((1 << shift) - 1)) == 0 && j < N) dst[j] = make_float2(u[0].hi, u[0].lo);
    }
}

// The slot of the sample taken after sweep `sweep_no` (1-based, cumulative),
// or -1 when no sample is due.  The buffer is a ring of n_slots samples: a
// run longer than the buffer overwrites the oldest slots, so a replayed graph
// can keep writing into a fixed buffer that the host drains.
__device__ __forceinline__ int sample_slot(long long sweep_no, long long first, int interval, int n_slots)
{
    if (interval <= 0 || n_slots <= 0 || sweep_no < first) return -1;
    const long long d = sweep_no - first;
    if (d % interval) return -1;
    return (int)((d / interval) % n_slots);
}

// Block-wide double sums of NC values into `out` (thread 0 valid); scratch
// holds 32*NC doubles.  All threads of the block must call.
template <int NC>
__device__ __forceinline__ void block_reduce_to(double (&v)[NC], double *scratch)
{
    block_sum<NC>(v, scratch);
    __syncthreads();
}

}  // namespace mcgb
