// Correctly rounded division by a divisor known in advance, shared by the
// FP64 field kernel and a host-side exhaustive check of its rounding.
#ifndef SPG_EXACT_DIV_H
#define SPG_EXACT_DIV_H

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SPG_XHD __host__ __device__
#else
#define SPG_XHD
#endif

namespace spg {

SPG_XHD inline long long as_bits(double x) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    long long b;
    std::memcpy(&b, &x, 8);
    return b;
#endif
}

SPG_XHD inline double from_bits(long long b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    std::memcpy(&x, &b, 8);
    return x;
#endif
}

// Correctly rounded x / m for a divisor known in advance, without the FP64
// division sequence (the FMA-based correction of Markstein, IBM J. Res. Dev.
// 34(1), 1990): with r = RN(1/m), q0 = RN(x r) is within two ulps of x/m and
// q1 = RN(q0 + RN(x - q0 m) r) within one, so the remainder x - q1 m is exact
// as one FMA. q1 is the nearest double unless that remainder exceeds
// m ulp/2 (m ulp/4 toward zero when q1 is a power of two, where the ulp
// below is half the ulp above); then the neighbour in the remainder's
// direction is taken, and an exact half-way remainder keeps the even one.
// Comparisons and the ulp step are integer operations on the bit patterns.
// Zero and quotients or thresholds near the subnormal or overflow range take
// the division itself.
SPG_XHD inline double div_by_known(double x, double m, double r) {
    const long long qb0 = as_bits(x * r);
    const int eq = int((qb0 >> 52) & 0x7ff);
    const long long mb = as_bits(m);
    const int em = int((mb >> 52) & 0x7ff);
    // (x == 0 is a zero exponent of x r; the tests below are integer operations)
    if (eq < 64 || eq > 2000 || em + eq < 1140 || em + eq > 3000) return x / m;
    const double q0 = from_bits(qb0);
    const double q1 = std::fma(std::fma(-q0, m, x), r, q0);
    const double e1 = std::fma(-q1, m, x);  // exact: q1 is faithful
    const long long b1 = as_bits(q1), be = as_bits(e1);
    const int e = int((b1 >> 52) & 0x7ff);
    // the true quotient lies farther from zero: e1 nonzero with the sign of q1
    const bool away = (be << 1) != 0 && ((be ^ b1) >= 0);
    const bool pow2 = (b1 & 0xFFFFFFFFFFFFFLL) == 0;
    // m ulp(q1) / 2 = m 2^(e - 1076); toward zero from a power of two: m 2^(e - 1077)
    const int sh = (!away && pow2) ? e - 1077 : e - 1076;
    const long long lim = (mb & 0x7fffffffffffffffLL) + ((long long)sh << 52);
    const long long ae = be & 0x7fffffffffffffffLL;
    if (ae < lim || (ae == lim && (pow2 || !(b1 & 1)))) return q1;
    return from_bits(away ? b1 + 1 : b1 - 1);
}

}  // namespace spg

#endif
