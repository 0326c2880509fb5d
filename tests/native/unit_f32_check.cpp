// Host check of mcgb_unit_f32 (rng_convert.h) against the float64 route
// float((double)(x >> 11) * 2^-53), built and run by tests/test_rng_convert.py.
#include <cstdio>
#include <cstdint>

#include "rng_convert.h"

static uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static int check(uint64_t x)
{
    const float ref = (float)((double)(x >> 11) * (1.0 / 9007199254740992.0));
    const float got = mcgb_unit_f32(x);
    if (!(ref == got) && !(ref != ref && got != got)) {
        std::printf("mismatch x=%016llx ref=%a got=%a\n", (unsigned long long)x, ref, got);
        return 1;
    }
    return 0;
}

int main()
{
    int bad = 0;
    uint64_t s = 12345;
    for (long i = 0; i < 20000000 && bad < 5; ++i) {
        uint64_t x = splitmix(s);
        bad += check(x);
        // Short mantissas, ties and values near 1 and 0.
        const int shift = (int)(x & 63);
        bad += check(x >> shift);
        bad += check((x | 0x7FFull) >> (shift & 31));
        bad += check(~0ull - (x & 0xFFFFFull));
    }
    for (int b = 0; b < 64; ++b) {
        bad += check(1ull << b);
        bad += check((1ull << b) - 1);
        bad += check((3ull << b) >> 1);
    }
    // Exact ties: bit 39 of the normalised value set, nothing below.
    for (int lz = 11; lz < 40; ++lz)
        for (uint64_t sig = (1u << 23); sig < (1u << 23) + 64; ++sig) {
            const uint64_t y = (sig << 40) | (1ull << 39);
            bad += check((y >> lz) << 11);
        }
    std::printf(bad ? "FAIL\n" : "OK\n");
    return bad ? 1 : 0;
}
