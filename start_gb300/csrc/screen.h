// FP32 screens of the FP64 step: the truncated-float view of a double and the
// per-tet record of the inside screen. Shared by the step kernel and the host
// code that builds the records, so both truncate with the same integer ops.
#ifndef SPG_SCREEN_H
#define SPG_SCREEN_H

#include "exact_div.h"

namespace spg {

// Float from the high word of a double (sign, exponent, top 20 mantissa
// bits), integer ops only: |f - x| <= 2^-20 |x| for 2^-126 <= |x| < 2^128;
// 0 below that range, +-inf above.
SPG_XHD inline float hi_float(double x) {
    const int hi = int(as_bits(x) >> 32);
    const int a = hi & 0x7fffffff;
    const int r = a < (897 << 20) ? 0 : (a >= (1151 << 20) ? 0x7f800000 : ((a - (896 << 20)) << 3));
    const int bits = r | (hi & int(0x80000000));
#ifdef __CUDA_ARCH__
    return __int_as_float(bits);
#else
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
#endif
}

// hi_float of a tet's barycentric map (M row-major, origin x0): what the
// inside screen reads, 48 bytes instead of the 96 of the FP64 map.
struct alignas(16) TetScreen {
    float M[9];
    float x0[3];
};
static_assert(sizeof(TetScreen) == 48, "TetScreen is three 16-byte words");

}  // namespace spg

#endif
