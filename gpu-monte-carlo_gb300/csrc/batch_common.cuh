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
