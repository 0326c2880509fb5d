// Error plumbing of the C ABI and the per-site xoroshiro128+ streams.
//
// numba.cuda.random (the reference's RNG, called at core/runtime.py:51-53)
// seeds stream 0 with one SplitMix64 output in both words and derives stream
// k by k sequential 2^64-step jumps on the host: O(n) host work and an H2D
// copy of n*16 bytes.  Here every stream is computed on the device: the jump
// is a linear map J on the 128-bit state over GF(2), so stream k is J^k s0.
// The host builds J^(2^b) for b < 48 once per device (column form, 96 KB in
// a __device__ table); each thread applies the set bits of its first stream
// index, then steps J for the following streams of its chunk.
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "mcgb_common.cuh"

namespace mcgb {

static thread_local std::string g_error;

void set_error(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
}

int cuda_status(cudaError_t err, const char *what)
{
    if (err == cudaSuccess) return MCGB_OK;
    set_error("%s: %s", what, cudaGetErrorString(err));
    return err == cudaErrorMemoryAllocation ? MCGB_ENOMEM : MCGB_ECUDA;
}

int check_launch(const char *what)
{
    g_error.clear();
    return cuda_status(cudaGetLastError(), what);
}

int replica_reduce_cluster(int R, int L, int threads)
{
    int dev = 0, sms = 0;
    int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    st = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                     "cudaDeviceGetAttribute(multiprocessors)");
    if (st) return st;
    long long C = (2LL * sms + R - 1) / R;
    const long long by_sites = (long long)L * L / threads;
    if (C > by_sites) C = by_sites;
    if (C > 8) C = 8;
    if (C < 1) C = 1;
    return (int)C;
}

// ------------------------------------------------------------ jump tables

constexpr int kJumpLevels = 48;
__device__ ulonglong2 g_jump_cols[kJumpLevels][128];  // column c of J^(2^b)

static uint64_t host_next(uint64_t s[2])
{
    uint64_t s0 = s[0], s1 = s[1], r = s0 + s1;
    s1 ^= s0;
    s[0] = ((s0 << 55) | (s0 >> 9)) ^ s1 ^ (s1 << 14);
    s[1] = (s1 << 36) | (s1 >> 28);
    return r;
}

static void host_jump(uint64_t s[2])
{
    static const uint64_t JUMP[2] = {0xbeac0467eba5facbull, 0xd86b048b86aa9922ull};
    uint64_t a = 0, b = 0;
    for (int w = 0; w < 2; ++w)
        for (int bit = 0; bit < 64; ++bit) {
            if (JUMP[w] & (1ull << bit)) {
                a ^= s[0];
                b ^= s[1];
            }
            host_next(s);
        }
    s[0] = a;
    s[1] = b;
}

// y = M x for a column-form matrix M (cols[c] = image of basis vector c).
static void host_apply(const uint64_t (*cols)[2], const uint64_t x[2], uint64_t y[2])
{
    uint64_t a = 0, b = 0;
    for (int c = 0; c < 128; ++c)
        if ((x[c >> 6] >> (c & 63)) & 1) {
            a ^= cols[c][0];
            b ^= cols[c][1];
        }
    y[0] = a;
    y[1] = b;
}

static int ensure_jump_tables(cudaStream_t stream)
{
    static std::mutex mu;
    static bool ready[128] = {};
    int dev = 0;
    int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 128 && ready[dev]) return MCGB_OK;
    static uint64_t tables[kJumpLevels][128][2];
    static bool built = false;
    if (!built) {
        for (int c = 0; c < 128; ++c) {
            uint64_t s[2] = {0, 0};
            s[c >> 6] = 1ull << (c & 63);
            host_jump(s);
            tables[0][c][0] = s[0];
            tables[0][c][1] = s[1];
        }
        for (int b = 1; b < kJumpLevels; ++b)
            for (int c = 0; c < 128; ++c) host_apply(tables[b - 1], tables[b - 1][c], tables[b][c]);
        built = true;
    }
    st = cuda_status(cudaMemcpyToSymbolAsync(g_jump_cols, tables, sizeof tables, 0,
                                             cudaMemcpyHostToDevice, stream),
                     "upload RNG jump tables");
    if (st) return st;
    st = cuda_status(cudaStreamSynchronize(stream), "upload RNG jump tables");
    if (st) return st;
    if (dev < 128) ready[dev] = true;
    return MCGB_OK;
}

__device__ __forceinline__ ulonglong2 apply_level(int level, ulonglong2 x)
{
    uint64_t a = 0, b = 0;
#pragma unroll 4
    for (int c = 0; c < 64; ++c)
        if ((x.x >> c) & 1) {
            ulonglong2 col = g_jump_cols[level][c];
            a ^= col.x;
            b ^= col.y;
        }
#pragma unroll 4
    for (int c = 0; c < 64; ++c)
        if ((x.y >> c) & 1) {
            ulonglong2 col = g_jump_cols[level][64 + c];
            a ^= col.x;
            b ^= col.y;
        }
    return make_ulonglong2(a, b);
}

__host__ __device__ inline uint64_t splitmix64_first(uint64_t seed)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

constexpr int kInitChunk = 32;

__global__ void rng_init_kernel(ulonglong2 *states, int64_t n, uint64_t seed, uint64_t sub)
{
    int64_t chunk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t first = chunk * kInitChunk;
    if (first >= n) return;
    uint64_t z = splitmix64_first(seed);
    ulonglong2 v = make_ulonglong2(z, z);
    uint64_t k = sub + (uint64_t)first;
    for (int b = 0; b < kJumpLevels && k; ++b, k >>= 1)
        if (k & 1) v = apply_level(b, v);
    int64_t last = first + kInitChunk < n ? first + kInitChunk : n;
    for (int64_t i = first; i < last; ++i) {
        states[i] = v;
        if (i + 1 < last) v = apply_level(0, v);
    }
}

__global__ void rng_draw_kernel(ulonglong2 *states, int64_t index, int count, int kind, void *out)
{
    ulonglong2 s = states[index];
    for (int k = 0; k < count; ++k) {
        if (kind == 0)
            static_cast<float *>(out)[k] = xoro_uniform_f32(s);
        else
            static_cast<double *>(out)[k] = xoro_uniform_f64(s);
    }
    states[index] = s;
}

__global__ void expf_kernel(const float *x, float *y, int64_t n)
{
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) y[t] = expf(x[t]);
}

}  // namespace mcgb

using namespace mcgb;

extern "C" const char *mcgb_last_error(void) { return g_error.c_str(); }

extern "C" const char *mcgb_version(void) { return "mcgb 0.1 sm_103a"; }

extern "C" int mcgb_rng_init(void *states, int64_t n, uint64_t seed, uint64_t sub, void *stream)
{
    MCGB_REQUIRE(n >= 0, "rng_init: n must be >= 0");
    if (n == 0) return MCGB_OK;
    MCGB_REQUIRE(states != nullptr, "rng_init: null states");
    MCGB_REQUIRE(sub < (1ull << 47) && (uint64_t)n < (1ull << 47),
                 "rng_init: subsequence_start + n must be < 2^48");
    cudaStream_t s = as_stream(stream);
    int st = ensure_jump_tables(s);
    if (st) return st;
    int64_t chunks = (n + kInitChunk - 1) / kInitChunk;
    int threads = 128;
    int64_t blocks = (chunks + threads - 1) / threads;
    rng_init_kernel<<<(unsigned)blocks, threads, 0, s>>>(static_cast<ulonglong2 *>(states), n, seed, sub);
    return check_launch("rng_init_kernel");
}

extern "C" int mcgb_rng_draw(void *states, int64_t index, int count, int kind, void *out, void *stream)
{
    MCGB_REQUIRE(states && out, "rng_draw: null pointer");
    MCGB_REQUIRE(index >= 0 && count >= 0 && (kind == 0 || kind == 1), "rng_draw: bad arguments");
    rng_draw_kernel<<<1, 1, 0, as_stream(stream)>>>(static_cast<ulonglong2 *>(states), index, count, kind, out);
    return check_launch("rng_draw_kernel");
}

extern "C" int mcgb_expf(const float *x, float *out, int64_t n, void *stream)
{
    MCGB_REQUIRE(n >= 0, "expf: n must be >= 0");
    if (n == 0) return MCGB_OK;
    MCGB_REQUIRE(x && out, "expf: null pointer");
    expf_kernel<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(x, out, n);
    return check_launch("expf_kernel");
}
