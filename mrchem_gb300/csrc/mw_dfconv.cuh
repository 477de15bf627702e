// mw_dfconv.cuh -- FP64 <-> FP32-pair conversions on the integer and FP32 pipes.
//
// The double-FP32 kernels (post-processing, tree multiply) read FP64 blocks, compute on FP32
// pairs and write FP64 blocks.  The CUDA conversions between double and float, and the double
// addition that joins a pair, execute on the FP64 pipe, which on GB300 runs at 1/64 of the FP32
// rate: for a node of the multiply they kept that pipe about a quarter busy beside the FP32 work.
// These helpers do the same conversions with integer operations on the bit patterns.
//
//   df_split(d, h, l): h = d truncated to 24 significant bits, l = the remainder (d - h, exact in
//                      29 bits) truncated to 24 bits; |d - h - l| < 2^-47 |d|.  Values whose
//                      exponent lies outside [2^-74, 2^127), zeros included, take the CUDA
//                      conversions instead (round-to-nearest split).
//   df_widen(f):       the float's value as a double, exactly (normal floats by bit patterns,
//                      zeros, subnormals, infinities and NaNs by the CUDA conversion).
#pragma once

#include <cstdint>

namespace mwg {

__device__ __forceinline__ void df_split(double d, float &h, float &l) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    if (e >= 949u && e <= 1150u) {
        const unsigned s = (unsigned)(u >> 63) << 31;
        // hi: the sign, the exponent rebiased for FP32 and the top 23 mantissa bits
        h = __uint_as_float(s | ((e - 896u) << 23) | ((unsigned)(u >> 29) & 0x7fffffu));
        const unsigned r = (unsigned)u & 0x1fffffffu;  // the remainder: r * 2^(e - 1075)
        if (r == 0u) {
            l = 0.0f;
        } else {
            const int p = 31 - __clz((int)r);  // leading bit of r, 0 .. 28
            const unsigned m = p >= 23 ? r >> (p - 23) : r << (23 - p);
            l = __uint_as_float(s | ((unsigned)(p + (int)e - 948) << 23) | (m & 0x7fffffu));
        }
    } else {
        h = __double2float_rn(d);
        l = __double2float_rn(d - (double)h);
    }
}

__device__ __forceinline__ double df_widen(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)f;
    const unsigned long long u = ((unsigned long long)(b >> 31) << 63) | ((unsigned long long)(e + 896u) << 52) |
                                 ((unsigned long long)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)u);
}

}  // namespace mwg
