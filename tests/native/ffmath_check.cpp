// Host check of the float-float sine/cosine (ffmath.h) against the C
// library's float64 sin and cos: the largest absolute error over random
// float and float-float arguments in several ranges, and at the points
// nearest multiples of pi/2, stays within the stated bounds.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <random>

#include "ffmath.h"

static double worst = 0.0;

static bool check(ff x, double bound)
{
    ff s, c;
    ff_sincos(x, &s, &c);
    const double xd = (double)x.hi + (double)x.lo;
    const double es = std::fabs(ff_to_double(s) - std::sin(xd));
    const double ec = std::fabs(ff_to_double(c) - std::cos(xd));
    const double e = es > ec ? es : ec;
    if (e > worst) worst = e;
    if (!(e <= bound)) {
        std::printf("FAIL x=%.17g (hi %a lo %a): sin err %.3g cos err %.3g bound %.3g\n", xd, x.hi, x.lo, es, ec,
                    bound);
        return false;
    }
    return true;
}

int main()
{
    std::mt19937_64 gen(12345);
    std::uniform_real_distribution<float> angle(-3.14159265f, 3.14159265f);
    bool ok = true;
    // Angles of float spins and exact differences of two of them.
    for (int n = 0; n < 2000000 && ok; ++n) {
        const float a = angle(gen), b = angle(gen);
        ok = check(ff_make(a, 0.0f), 8e-15) && check(ff_diff(a, b), 8e-15);
    }
    const double small_worst = worst;
    // Wider ranges: the reduction's error grows with |x|.
    const float ranges[] = {10.0f, 100.0f, 1000.0f, 65536.0f, 1048576.0f};
    for (float R : ranges) {
        std::uniform_real_distribution<float> wide(-R, R);
        for (int n = 0; n < 200000 && ok; ++n) ok = check(ff_make(wide(gen), 0.0f), 8e-15 + 4e-17 * R);
    }
    // The floats nearest k pi/2 (cancellation in the reduction).
    for (int k = -4096; k <= 4096 && ok; ++k) {
        const float x = (float)(k * 1.5707963267948966);
        ok = check(ff_make(x, 0.0f), 8e-15 + 4e-17 * std::fabs(x)) &&
             check(ff_make(std::nextafter(x, 1e30f), 0.0f), 8e-15 + 4e-17 * std::fabs(x)) &&
             check(ff_make(std::nextafter(x, -1e30f), 0.0f), 8e-15 + 4e-17 * std::fabs(x));
    }
    std::printf("worst |err| for |x| <= 2 pi: %.3g; overall %.3g\n", small_worst, worst);
    if (ok) std::printf("OK\n");
    return ok ? 0 : 1;
}
