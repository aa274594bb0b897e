// Exact FP32 <-> FP64 conversions with integer operations.  On this part the
// conversion instructions run on the FP64 pipe, whose rate is a small
// fraction of the FP32 one, so kernels that widen or narrow one value per
// output element spend most of their time there.  Both functions move the
// IEEE-754 fields (sign, exponent rebiased between 127 and 1023, mantissa
// shifted between 23 and 52 bits, rounded to nearest even when narrowing)
// and give the conversion instruction's result bit for bit; the values they
// do not handle (zeros, subnormals, infinities, NaNs, and narrowing results
// outside the normal FP32 range) take the instruction.
#pragma once
#include <cstdint>

namespace slfmm {

__device__ __forceinline__ double f64_of_f32(float x) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;
    const uint64_t r = ((uint64_t)(b >> 31) << 63) | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)r);
}

__device__ __forceinline__ float f32_of_f64(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ffu);
    const int ef = e - 896;
    if (e == 0x7ff || ef <= 0 || ef >= 255) return (float)x;
    const uint64_t m = b & 0xfffffffffffffull;
    const uint32_t mf = (uint32_t)(m >> 29), rest = (uint32_t)(m & 0x1fffffffu);
    uint32_t r = ((uint32_t)(b >> 63) << 31) | ((uint32_t)ef << 23) | mf;
    if (rest > 0x10000000u || (rest == 0x10000000u && (mf & 1u))) r += 1u;  // a carry moves into the exponent
    return __uint_as_float(r);
}

}  // namespace slfmm
