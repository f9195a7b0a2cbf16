// Checks div_by_known (start_gb300/csrc/exact_div.h) against IEEE division:
// random dividends over many binades, dividends just around midpoints of the
// quotient grid, and the particle masses the workloads use as divisors.
// Prints the number of mismatches (0 expected) and exits non-zero on any.
#include <cstdio>
#include <cstdint>
#include <random>

#include "exact_div.h"

int main(int argc, char **argv) {
    const long long n = argc > 1 ? std::atoll(argv[1]) : 2000000;
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    const double masses[] = {7.95e-26, 7.9485017e-26, 6.6335209e-26, 1.0, 3.0, 1.6726e-27, 9.1093837e-31};
    long long bad = 0, tested = 0;
    for (double m : masses) {
        const double r = 1.0 / m;
        for (long long i = 0; i < n; ++i) {
            // dividend: random mantissa, exponent spread over +-60 binades around q E ~ 1e-17..1e-12
            double x = std::ldexp(1.0 + u(g), int(u(g) * 120.0) - 120);
            if (i & 1) x = -x;
            if (i % 7 == 0) {
                // a dividend that puts x/m next to a midpoint between two doubles
                const double q = std::ldexp(1.0 + u(g), int(u(g) * 60.0) - 30);
                const double mid = q + 0.5 * (std::nextafter(q, 2.0 * q) - q);
                x = mid * m;
                x = std::nextafter(x, (i % 2) ? 0.0 : 2.0 * x);
            }
            const double a = spg::div_by_known(x, m, r), b = x / m;
            if (spg::as_bits(a) != spg::as_bits(b)) {
                if (bad < 10) std::printf("mismatch m=%.17g x=%.17g got %.17g want %.17g\n", m, x, a, b);
                bad++;
            }
            tested++;
        }
    }
    std::printf("tested %lld mismatches %lld\n", tested, bad);
    return bad ? 1 : 0;
}
