// Host check of mcgb_unit_threshold (rng_convert.h): for many floats t, the
// returned M separates the integers m = x >> 11 with mcgb_unit_f32 < t
// (m < M) from those with mcgb_unit_f32 >= t (m >= M).  Built and run by
// tests/test_rng_convert.py.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cmath>

#include "rng_convert.h"

static float unit_of_m(uint64_t m) { return mcgb_unit_f32(m << 11); }

static int check(float t)
{
    const uint64_t M = mcgb_unit_threshold(t);
    if (M > (1ull << 53)) { std::printf("M out of range for t=%a\n", t); return 1; }
    // m = M - 1 must be below t, m = M must not be (when in range).
    if (M > 0 && !(unit_of_m(M - 1) < t)) {
        std::printf("t=%a M=%llu: unit(M-1)=%a not < t\n", t, (unsigned long long)M, unit_of_m(M - 1));
        return 1;
    }
    if (M < (1ull << 53) && (unit_of_m(M) < t)) {
        std::printf("t=%a M=%llu: unit(M)=%a < t\n", t, (unsigned long long)M, unit_of_m(M));
        return 1;
    }
    return 0;
}

static float from_bits(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }

int main()
{
    int bad = 0;
    // Every float in [2^-30, 1] with a stride, plus dense ranges near
    // exponent boundaries, tiny values, and the special cases.
    for (uint32_t b = 0x30800000u; b <= 0x3f800000u && bad < 5; b += 97) bad += check(from_bits(b));
    for (int e = 1; e < 255 && bad < 5; ++e)
        for (uint32_t k = 0; k < 2048; ++k) {
            const uint32_t base = (uint32_t)e << 23;
            bad += check(from_bits(base + k));
            bad += check(from_bits(base + 0x7fffffu - k));
        }
    const float specials[] = {0.0f, -0.0f, -1.0f, 1.0f, 2.0f, 1e-45f, 1e-38f, 1.0f - 1e-7f, NAN, INFINITY};
    for (float t : specials) bad += check(t);
    std::printf(bad ? "FAIL\n" : "OK\n");
    return bad ? 1 : 0;
}
