// Shared device helpers for the mcgb CUDA library (sm_103a).
//
// - Status codes and the thread-local error message behind mcgb_last_error().
// - The per-site xoroshiro128+ stream (state = one 16-byte ulonglong2 {s0, s1},
//   the layout of numba.cuda.random's xoroshiro128p_dtype) with the
//   float32/float64 uniform conversions that the reference's kernels draw.
// - complex64 helpers with the operation order the reference's complex64
//   algebra uses (models/he3/update.py).
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mcgb.h"
#include "rng_convert.h"

namespace mcgb {

void set_error(const char *fmt, ...);
int cuda_status(cudaError_t err, const char *what);
int check_launch(const char *what);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

#define MCGB_REQUIRE(cond, ...)                       \
    do {                                              \
        if (!(cond)) {                                \
            ::mcgb::set_error(__VA_ARGS__);           \
            return MCGB_EINVAL;                       \
        }                                             \
    } while (0)

// ---------------------------------------------------------------- RNG

__device__ __forceinline__ uint64_t rotl64(uint64_t x, int k)
{
    return (x << k) | (x >> (64 - k));
}

// One xoroshiro128+ step (a=55, b=14, c=36); returns s0 + s1 of the old state.
__device__ __forceinline__ uint64_t xoro_next(ulonglong2 &s)
{
    uint64_t s0 = s.x, s1 = s.y;
    uint64_t result = s0 + s1;
    s1 ^= s0;
    s.x = rotl64(s0, 55) ^ s1 ^ (s1 << 14);
    s.y = rotl64(s1, 36);
    return result;
}

// (x >> 11) * 2^-53 in float64.
__device__ __forceinline__ double xoro_uniform_f64(ulonglong2 &s)
{
    return (double)(xoro_next(s) >> 11) * 0x1.0p-53;
}

// float32 of the float64 uniform, rounded in integer arithmetic (see
// rng_convert.h) so that no instruction issues to the float64 pipe.
__device__ __forceinline__ float xoro_uniform_f32(ulonglong2 &s)
{
    return mcgb_unit_f32(xoro_next(s));
}

// ---------------------------------------------------------------- colour grids
//
// The per-colour kernels run one thread per site of a colour on a 3D grid
// -- x over the L/2 columns, y over the L/2 rows of the colour's sublattice,
// z over the replicas (and, for a launch of two colours, a second layer of
// replicas for colour c0 + 1) -- the shape of the reference's
// cuda.grid(3) launches, so a thread finds its site without divisions.
struct ColourGrid {
    dim3 grid, block;
};

inline ColourGrid colour_grid(int R, int L, int ncol, int threads = 256)
{
    const int H = L >> 1;
    int bx = 32;
    while (bx > 1 && bx / 2 >= H) bx /= 2;  // no wider than the rows (small lattices)
    const int by = threads / bx;
    ColourGrid g;
    g.block = dim3((unsigned)bx, (unsigned)by, 1);
    g.grid = dim3((unsigned)((H + bx - 1) / bx), (unsigned)((H + by - 1) / by), (unsigned)(R * ncol));
    return g;
}

// Site (i, j) of replica r for this thread of a colour_grid(R, L, ncol)
// launch of colour c0 (and c0 + 1 on the second layer); false outside.
__device__ __forceinline__ bool colour_grid_site(int R, int L, int c0, int &r, int &i, int &j)
{
    const int H = L >> 1;
    const int col = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y * blockDim.y + threadIdx.y;
    if (col >= H || row >= H) return false;
    const int z = blockIdx.z, extra = z >= R ? 1 : 0;
    r = z - extra * R;
    i = 2 * row + ((c0 + extra) >> 1);
    j = 2 * col + ((c0 + extra) & 1);
    return true;
}

// ---------------------------------------------------------------- XY visit (reference arithmetic)
//
// models/xy/update.py:19-54 in two halves, shared by the per-colour kernel
// and the reference-layout window so both produce the same bits.  Every
// float32 operation is rounded on its own (the __f*_rn intrinsics are never
// contracted into fused multiply-adds), as in the reference's arithmetic.

// The proposal theta + delta (2u - 1), wrapped once into [-pi, pi) (delta <=
// pi and theta in [-pi, pi)), and the acceptance uniform v, in the
// reference's draw order.
__device__ __forceinline__ float xy_ref_propose(float th, ulonglong2 &st, float delta, float &v)
{
    const float pi = 3.14159265358979323846f, two_pi = 6.28318530717958647692f;
    const float u = xoro_uniform_f32(st);
    float p = __fadd_rn(th, __fmul_rn(delta, __fsub_rn(__fmul_rn(2.0f, u), 1.0f)));
    if (p >= pi)
        p = __fsub_rn(p, two_pi);
    else if (p < -pi)
        p = __fadd_rn(p, two_pi);
    v = xoro_uniform_f32(st);
    return p;
}

// -J times the bond cosines of angle t with its four neighbours, in the
// reference's order (up, down, left, right).
__device__ __forceinline__ float xy_ref_site_energy(float t, float up, float down, float left, float right, float J)
{
    const float c = __fadd_rn(__fadd_rn(__fadd_rn(cosf(__fsub_rn(t, up)), cosf(__fsub_rn(t, down))),
                                        cosf(__fsub_rn(t, left))),
                              cosf(__fsub_rn(t, right)));
    return __fmul_rn(-J, c);
}

// The Metropolis decision of proposal p for angle th; dE the energy change.
__device__ __forceinline__ bool xy_ref_accept(float th, float p, float v, float up, float down, float left,
                                              float right, float beta, float J, float &dE)
{
    dE = __fsub_rn(xy_ref_site_energy(p, up, down, left, right, J), xy_ref_site_energy(th, up, down, left, right, J));
    return dE <= 0.0f || v < expf(__fmul_rn(-beta, dE));
}

// ---------------------------------------------------------------- complex64

struct c32 {
    float re, im;
};

__device__ __forceinline__ c32 cmk(float a, float b) { return c32{a, b}; }
__device__ __forceinline__ c32 operator+(c32 a, c32 b) { return cmk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ c32 operator-(c32 a, c32 b) { return cmk(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ c32 operator-(c32 a) { return cmk(-a.re, -a.im); }
__device__ __forceinline__ c32 operator*(c32 a, c32 b)
{
    return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ c32 operator*(float s, c32 a) { return cmk(s * a.re, s * a.im); }
__device__ __forceinline__ c32 conj(c32 a) { return cmk(a.re, -a.im); }
__device__ __forceinline__ float norm2(c32 z) { return z.re * z.re + z.im * z.im; }

// ---------------------------------------------------------------- reductions

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NC channels (blockDim.x a multiple of 32, <= 1024).
// Result valid in thread 0.  `scratch` holds 32*NC doubles.
template <int NC>
__device__ __forceinline__ void block_sum(double (&v)[NC], double *scratch)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < NC; ++c) v[c] = warp_sum(v[c]);
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) scratch[c * 32 + warp] = v[c];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            double x = lane < nwarps ? scratch[c * 32 + lane] : 0.0;
            v[c] = warp_sum(x);
        }
    }
}

__host__ __device__ __forceinline__ int wrapi(int i, int L) { return i < 0 ? i + L : (i >= L ? i - L : i); }

// ---------------------------------------------------------------- per-replica reductions on a cluster
//
// A per-replica reduction launched by launch_replica_reduce runs one
// thread-block cluster of C CTAs per replica (blockIdx.x / C): CTA `rank`
// takes sites k = rank * blockDim.x + threadIdx.x, k + C * blockDim.x, ...;
// cluster_sum adds the CTAs' block sums in rank order through distributed
// shared memory.  The order of every addition is fixed by the launch shape,
// so results are reproducible, and no global scratch is needed.

struct ReplicaSpan {
    int r, rank, first, step;
};

__device__ __forceinline__ ReplicaSpan replica_span()
{
    namespace cg = cooperative_groups;
    const cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks();
    return ReplicaSpan{(int)(blockIdx.x / C), (int)cl.block_rank(), (int)(cl.block_rank() * blockDim.x + threadIdx.x),
                       (int)(C * blockDim.x)};
}

// Sum of NC channels over the CTA (block_sum), then over the cluster's CTAs
// in rank order: valid in thread 0 of rank 0.  `scratch` holds 32*NC
// doubles, `part` NC doubles of shared memory.  Every thread must call it.
template <int NC>
__device__ __forceinline__ void cluster_sum(double (&v)[NC], double *scratch, double *part)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    block_sum<NC>(v, scratch);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) part[c] = v[c];
    }
    cl.sync();
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) v[c] = part[c];
        for (unsigned k = 1; k < cl.num_blocks(); ++k) {
            const double *pk = cl.map_shared_rank(part, k);
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] += pk[c];
        }
    }
    // Peers keep their shared memory until rank 0 has read it.
    cl.sync();
}

// CTAs per replica: enough clusters to give every SM about two CTAs, at
// most 8 (the portable cluster size) and at most one CTA per `threads`
// sites.
int replica_reduce_cluster(int R, int L, int threads);

// Launch `kern` as one cluster of replica_reduce_cluster(R, L, threads) CTAs
// per replica.
template <typename... KArgs, typename... Args>
int launch_replica_reduce(void (*kern)(KArgs...), int R, int L, int threads, cudaStream_t s, const char *name,
                          Args... args)
{
    const int C = replica_reduce_cluster(R, L, threads);
    if (C < 0) return C;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(R * C));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t err = cudaLaunchKernelEx(&cfg, kern, args...);
    if (err != cudaSuccess) {
        (void)cudaGetLastError();  // a refused configuration is not sticky
        return cuda_status(err, name);
    }
    return check_launch(name);
}

}  // namespace mcgb
