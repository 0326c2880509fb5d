// Exact float32 uniform from a 64-bit xoroshiro128+ output, in integer
// arithmetic only.
//
// numba.cuda.random's xoroshiro128p_uniform_float32 returns
// float32((x >> 11) * 2^-53): the 53-bit integer m = x >> 11 scaled to
// [0, 1) in float64, then rounded to float32 (round to nearest, ties to even).
// A uint64 -> float conversion instruction would compute the same value, but
// on GB300 it issues to the float64 pipe, whose throughput is a small fraction
// of the integer pipe's.  Here the rounding is done on the integer bits:
//   lz  = leading zeros of m (m < 2^53, so lz >= 11 when m != 0)
//   y   = m << lz                      (most significant bit at bit 63)
//   sig = y >> 40                      (24 significant bits, implicit bit set)
//   round up when bit 39 of y is set and (any lower bit of y is set or sig
//   is odd)
//   value = sig * 2^(40 - lz - 53), assembled as float bits
//   ((136 - lz) << 23) + sig, where a carry of sig into 2^24 bumps the
//   exponent exactly as IEEE rounding does.
// Compiles as host C++ (the unit test checks it bit for bit against the
// float64 route) and as CUDA device code.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define MCGB_HD __host__ __device__ __forceinline__
#else
#define MCGB_HD static inline
#endif

MCGB_HD int mcgb_clz64(uint64_t v)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

MCGB_HD float mcgb_bits_to_float(uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, sizeof f);
    return f;
#endif
}

MCGB_HD float mcgb_unit_f32(uint64_t x)
{
    const uint64_t m = x >> 11;
    if (m == 0) return 0.0f;
    const int lz = mcgb_clz64(m);
    const uint64_t y = m << lz;
    const uint32_t hi = (uint32_t)(y >> 32);
    const uint32_t lo = (uint32_t)y;
    uint32_t sig = hi >> 8;                      // bits 63..40 of y
    const uint32_t round = (hi >> 7) & 1u;       // bit 39
    const uint32_t sticky = (hi & 0x7fu) | lo;   // bits 38..0
    sig += round & ((sticky != 0u) | (sig & 1u));
    return mcgb_bits_to_float(((uint32_t)(136 - lz) << 23) + sig);
}

// Integer acceptance threshold.  For a float t, returns the smallest integer
// M in [0, 2^53] such that mcgb_unit_f32(x) >= t exactly when (x >> 11) >= M.
// mcgb_unit_f32 is monotone in m = x >> 11, so `u < t` for the float32 uniform
// u of x is `(x >> 11) < M`: one 64-bit compare instead of a conversion.
// t <= 0 or NaN gives 0 (never below), t > 1 gives 2^53 (always below).
//
// With T = t * 2^53 (exact), RN24(m) >= T holds for the integers m above the
// midpoint between T and its float predecessor q; a midpoint that is itself
// an integer rounds to T only when T's 24-bit significand is even.  Below
// 2^24 every integer is representable, so M = ceil(T).
MCGB_HD uint64_t mcgb_unit_threshold(float t)
{
    if (!(t > 0.0f)) return 0;
    if (t > 1.0f) return 1ull << 53;
    uint32_t b;
#if defined(__CUDA_ARCH__)
    b = __float_as_uint(t);
#else
    memcpy(&b, &t, sizeof b);
#endif
    int e = (int)(b >> 23);          // biased exponent of t
    uint32_t sig = b & 0x7fffffu;
    if (e == 0) {                    // subnormal t < 2^-126: T < 2^-73 < 1
        return 1;
    }
    sig |= 0x800000u;                // 24-bit significand, t = sig * 2^(e - 150)
    // T = sig * 2^(e - 150 + 53) = sig * 2^s, s = e - 97.
    const int s = e - 97;
    if (s <= 0) {
        // T < 2^24: M = ceil(T) = ceil(sig / 2^-s).
        const int sh = -s;
        if (sh >= 25) return 1;      // 0 < T < 1
        const uint64_t q = sig >> sh;
        return q + ((uint64_t)(sig & ((1u << sh) - 1u)) != 0);
    }
    // T >= 2^24: T = sig << s, an integer; ulp(T) = 2^s.
    const uint64_t T = (uint64_t)sig << s;
    uint64_t half;                   // T - midpoint(pred, T)
    if (sig == 0x800000u) {
        // A power of two: the predecessor is 2^(s-1) below.
        half = 1ull << (s - 1 > 0 ? s - 2 : 0);
        if (s == 1) {
            // pred = T - 1, midpoint T - 0.5 is not an integer.
            return T;
        }
        // midpoint T - 2^(s-2) is an integer; the tie goes to the even
        // significand, which is T's (1.000...).
        return T - half;
    }
    half = 1ull << (s - 1);
    if (s == 1) {
        // midpoint T - 1 is the integer between pred = T - 2 and T: a tie,
        // won by T only if its significand is even.
        return (sig & 1u) ? T : T - 1;
    }
    return (sig & 1u) ? T - half + 1 : T - half;
}

// Fast float32 uniform in [0, 1) from the top 23 bits of x (a float in
// [1, 2) minus one); used where the exact numba-compatible rounding is not
// needed (proposal noise and acceptance in the mixed-precision forms).
MCGB_HD float mcgb_fast_unit(uint64_t x)
{
    return mcgb_bits_to_float(0x3f800000u | (uint32_t)(x >> 41)) - 1.0f;
}

// The same from bits 40..18 of x, the next 23 bits below mcgb_fast_unit's:
// one draw yields two independent 23-bit uniforms (both away from the
// generator's weak lowest bits).
MCGB_HD float mcgb_fast_unit_mid(uint64_t x)
{
    return mcgb_bits_to_float(0x3f800000u | ((uint32_t)(x >> 18) & 0x7fffffu)) - 1.0f;
}

// The three uniforms of a Gaussian Metropolis visit of an XY spin, all from
// one draw x (each exact in float32):
//   u1 = (2k + 1) 2^-22, k = bits 63..43  -- strictly inside (0, 1), the
//        Box-Muller radius draw (no logarithm of zero, no clamp);
//   u2 = k 2^-21,        k = bits 42..22  -- the Box-Muller angle draw;
//   v  = k 2^-21,        k = bits 21..1   -- the acceptance draw (bit 0, the
//        generator's weakest, unused).
// The proposal is a Gaussian truncated at 5.4 sigma on a 2^-21 grid,
// symmetric, so Metropolis acceptance keeps detailed balance.
MCGB_HD float mcgb_visit_u1(uint64_t x)
{
    return mcgb_bits_to_float(0x3f800000u | ((uint32_t)(x >> 43) << 2) | 2u) - 1.0f;
}
MCGB_HD float mcgb_visit_u2(uint64_t x)
{
    return mcgb_bits_to_float(0x3f800000u | (((uint32_t)(x >> 22) & 0x1fffffu) << 2)) - 1.0f;
}
MCGB_HD float mcgb_visit_v(uint64_t x)
{
    return mcgb_bits_to_float(0x3f800000u | (((uint32_t)(x >> 1) & 0x1fffffu) << 2)) - 1.0f;
}
