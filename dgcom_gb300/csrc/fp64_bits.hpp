// Comparisons, minima and maxima of doubles on the integer pipes.
//
// GB300 executes two FP64 operations per SM per clock, a sixty-fourth of
// its FP32 and integer rate, and a compare or min/max of doubles (DSETP,
// DMNMX) holds the FP64 pipe as long as a multiply-add does. The stage is
// bound by that pipe, so these helpers compare bit patterns instead.
//
// For every non-NaN argument, ±0, subnormals and infinities included, each
// helper returns exactly what its IEEE counterpart written beside it
// returns; lmax/lmin return the same operand as `a > b ? a : b` and
// `a < b ? a : b`. With a NaN argument the result may differ from IEEE:
// a state that is not finite is caught by the stage's finiteness check and
// fails the step either way.
//
// Host and device both compile this header (the host for its unit test).
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DG_HD __host__ __device__ __forceinline__
#else
#define DG_HD inline
#endif

namespace dgswe {
namespace fp {

DG_HD int64_t bits(double x) {
#if defined(__CUDA_ARCH__)
    return (int64_t)__double_as_longlong(x);
#else
    int64_t b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

DG_HD double from_bits(int64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}

// A signed key in the order of the values: the sign-magnitude pattern as a
// two's-complement integer, with −0 and +0 both mapped to 0
DG_HD int64_t key(double x) {
    const int64_t b = bits(x);
    return b < 0 ? -(b & INT64_MAX) : b;
}

constexpr uint64_t kNegZero = 0x8000000000000000ull;

DG_HD bool gt0(double x) { return bits(x) > 0; }                       // x > 0
DG_HD bool le0(double x) { return bits(x) <= 0; }                      // x <= 0
DG_HD bool lt0(double x) { return (uint64_t)bits(x) > kNegZero; }      // x < 0
DG_HD bool ge0(double x) { return (uint64_t)bits(x) <= kNegZero; }     // x >= 0
DG_HD bool nz(double x) { return (bits(x) & INT64_MAX) != 0; }         // x != 0
DG_HD bool finite(double x) {                                          // isfinite(x)
    return (bits(x) & 0x7FF0000000000000ll) != 0x7FF0000000000000ll;
}

DG_HD bool gt(double a, double b) { return key(a) > key(b); }  // a > b
DG_HD bool ge(double a, double b) { return key(a) >= key(b); }  // a >= b
DG_HD bool lt(double a, double b) { return key(a) < key(b); }  // a < b
DG_HD bool le(double a, double b) { return key(a) <= key(b); }  // a <= b

// a > b ? a : b and a < b ? a : b
DG_HD double lmax(double a, double b) { return gt(a, b) ? a : b; }
DG_HD double lmin(double a, double b) { return lt(a, b) ? a : b; }
// x > 0 ? x : +0 (the depth floor max(x, 0) of the reference's selects)
DG_HD double max0(double x) { return gt0(x) ? x : 0.0; }

// Both operands non-negative (sign bit clear, e.g. after max0, or depths
// known to be ≥ +0): the raw patterns already order as the values
DG_HD bool gt_nn(double a, double b) { return bits(a) > bits(b); }
DG_HD double max_nn(double a, double b) { return bits(a) > bits(b) ? a : b; }
DG_HD double min_nn(double a, double b) { return bits(a) < bits(b) ? a : b; }

// The float at or toward zero from a double: sign, rebiased exponent and
// the top 23 bits of the mantissa, by integer operations (on the device a
// conversion instruction would run on the FP64 pipe); ±0 below 2^-126, ±∞
// from 2^128. The same bits on the host (tables built there) and on the
// device.
DG_HD float f32_trunc(double x) {
    const uint64_t b = (uint64_t)bits(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    const uint32_t mag = (uint32_t)(b >> 29) - (896u << 23);
    const uint32_t out = sign | (e <= 896u ? 0u : (e >= 1151u ? 0x7F800000u : mag));
#if defined(__CUDA_ARCH__)
    return __uint_as_float(out);
#else
    float f;
    memcpy(&f, &out, sizeof f);
    return f;
#endif
}

}  // namespace fp
}  // namespace dgswe
