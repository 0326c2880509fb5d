// Float-float ("double-float") arithmetic and a float-float sine/cosine.
//
// GB300 issues float64 arithmetic at a small fraction of its float32 rate,
// and a float64 cos or sin takes dozens of float64 instructions.  The
// reference's measurements evaluate them in float64 per site; here the same
// values come from the float32 pipe: a value is the unevaluated sum hi + lo
// of two floats (about 48 significant bits), built from the error-free
// transformations of Knuth (two_sum) and Dekker (fast_two_sum), with the
// product's rounding error from one fused multiply-add (two_prod).
//
// ff_sincos(x) evaluates sin and cos of a float-float x with |x| <= 2^20:
// Cody-Waite reduction x = k pi/2 + r with pi/2 split into three floats
// (each product k * part exact through two_prod, |r| <= pi/4 + tiny), then
// the Taylor series of sin and cos at 0 (coefficients 1/n!, the first
// terms as float-float pairs) by Horner's rule, float-float where a term's
// rounding would exceed about 1e-16 and plain float for the small tail
// (from r^11 for sin, r^12 for cos), and the quadrant's signs and swap.
// Absolute error of either result below 6e-15 over float angles, exact
// differences of two angles and |x| up to 2^20 (a host check against the C
// library's float64 sin and cos asserts 8e-15).
//
// Compiles as host C++ (the check) and as CUDA device code.  Host builds
// must not reassociate float expressions (no -ffast-math).
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define FF_HD __host__ __device__ __forceinline__
#else
#define FF_HD static inline
#endif

struct ff {
    float hi, lo;
};

FF_HD ff ff_make(float hi, float lo)
{
    ff r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

// a + b = s + e exactly (Knuth).
FF_HD ff ff_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return ff_make(s, (a - (s - bb)) + (b - bb));
}

// a + b = s + e exactly when |a| >= |b| (Dekker).
FF_HD ff ff_fast_two_sum(float a, float b)
{
    const float s = a + b;
    return ff_make(s, b - (s - a));
}

// a * b = p + e exactly (one fused multiply-add for the error).
FF_HD ff ff_two_prod(float a, float b)
{
    const float p = a * b;
    return ff_make(p, fmaf(a, b, -p));
}

FF_HD ff ff_add(ff a, ff b)
{
    ff s = ff_two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return ff_fast_two_sum(s.hi, s.lo);
}

FF_HD ff ff_add_f(ff a, float b)
{
    ff s = ff_two_sum(a.hi, b);
    s.lo += a.lo;
    return ff_fast_two_sum(s.hi, s.lo);
}

FF_HD ff ff_mul(ff a, ff b)
{
    ff p = ff_two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return ff_fast_two_sum(p.hi, p.lo);
}

FF_HD ff ff_mul_f(ff a, float b)
{
    ff p = ff_two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return ff_fast_two_sum(p.hi, p.lo);
}

FF_HD ff ff_neg(ff a) { return ff_make(-a.hi, -a.lo); }

FF_HD double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// a - b of two floats, exactly.
FF_HD ff ff_diff(float a, float b) { return ff_two_sum(a, -b); }

// sin and cos of x (|x| <= 2^20), each within 8e-15 of the exact value.
FF_HD void ff_sincos(ff x, ff *s, ff *c)
{
    // pi/2 = P0 + P1 + P2 + O(1e-23); 2/pi rounded to float.
    const float P0 = 0x1.921fb6p+0f, P1 = -0x1.777a5cp-25f, P2 = -0x1.ee59dap-50f;
    const float two_over_pi = 0x1.45f306p-1f;
    const float k = rintf(x.hi * two_over_pi);
    // r = x - k (P0 + P1 + P2): each k * Pi exact as a float-float.
    ff r = ff_add(x, ff_neg(ff_two_prod(k, P0)));
    r = ff_add(r, ff_neg(ff_two_prod(k, P1)));
    r = ff_add_f(r, -k * P2);
    const ff z = ff_mul(r, r);
    const float zf = z.hi;

    // sin r = r + r z (-1/3! + z (1/5! + z (-1/7! + z (1/9! + z T)))),
    // T = -1/11! + z (1/13! + z (-1/15! + z / 17!)) in float.
    float t = 0x1.952c78p-49f;
    t = fmaf(zf, t, -0x1.ae7f3ep-41f);
    t = fmaf(zf, t, 0x1.612462p-33f);
    t = fmaf(zf, t, -0x1.ae6456p-26f);
    ff p = ff_add(ff_make(0x1.71de3ap-19f, 0x1.55b1ccp-45f), ff_mul_f(z, t));
    p = ff_add(ff_make(-0x1.a01a02p-13f, 0x1.7f97fap-39f), ff_mul(z, p));
    p = ff_add(ff_make(0x1.111112p-7f, -0x1.dddddep-32f), ff_mul(z, p));
    p = ff_add(ff_make(-0x1.555556p-3f, 0x1.555556p-28f), ff_mul(z, p));
    const ff sn = ff_add(r, ff_mul(ff_mul(r, z), p));

    // cos r = 1 - z/2 + z^2 (1/4! + z (-1/6! + z (1/8! + z (-1/10! + z T)))),
    // T = 1/12! + z (-1/14! + z (1/16! - z / 18!)) in float.
    t = -0x1.682786p-53f;
    t = fmaf(zf, t, 0x1.ae7f3ep-45f);
    t = fmaf(zf, t, -0x1.93974ap-37f);
    t = fmaf(zf, t, 0x1.1eed8ep-29f);
    ff q = ff_add(ff_make(-0x1.27e4fcp-22f, 0x1.10ec14p-47f), ff_mul_f(z, t));
    q = ff_add(ff_make(0x1.a01a02p-16f, -0x1.7f97fap-42f), ff_mul(z, q));
    q = ff_add(ff_make(-0x1.6c16c2p-10f, 0x1.27d27ep-35f), ff_mul(z, q));
    q = ff_add(ff_make(0x1.555556p-5f, -0x1.555556p-30f), ff_mul(z, q));
    ff cs = ff_add(ff_mul(ff_mul(z, z), q), ff_mul_f(z, -0.5f));
    cs = ff_add_f(cs, 1.0f);

    // Quadrant k mod 4: (sin, cos) of x = (s, c), (c, -s), (-s, -c), (-c, s).
    const int quad = ((int)k) & 3;
    const ff a = (quad & 1) ? cs : sn;
    const ff b = (quad & 1) ? sn : cs;
    *s = (quad & 2) ? ff_neg(a) : a;
    *c = ((quad + 1) & 2) ? ff_neg(b) : b;
}
