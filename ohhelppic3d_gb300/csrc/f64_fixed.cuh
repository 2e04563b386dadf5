// f64_fixed.cuh -- cell, offset and 2^-48 fixed-point CIC weights of FP64
// coordinates, shared by the FP64 tile kernels (push_f64.cu) and the subdomain
// kernels (subdomain.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr unsigned long long kOne48 = 1ull << 48;

// Cell index and in-cell offset of a coordinate by integer operations on its
// bit pattern.  On GB300 the FP64 pipe bounds this form, and (int)x,
// (double)ix, x - ix and the 48-bit rounding were six of its operations per axis.
// A coordinate is kept as (fr, e): for x >= 1, e is its binary exponent and fr
// the mantissa bits below the binary point, so the offset is fr * 2^(e-52); for
// x in [0, 1) (and -0.0), e = -1 and fr holds the bits of x itself.
struct Split {
    unsigned long long fr;
    int e;
};

// floor(x) for x in [0, 2^30); -1 for anything else (negative, NaN, too large).
__device__ __forceinline__ int split_cell(double x, Split &s)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)(b >> 52);                       // the sign bit makes negatives >= 2048
    if (E < 1023 || b == 0x8000000000000000ull) {       // [0, 1) and -0.0: cell 0, offset x
        s.fr = b;
        s.e = -1;
        return 0;
    }
    s.e = E - 1023;
    if (s.e > 29) return -1;
    const unsigned long long F = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = 52 - s.e;
    s.fr = F & ((1ull << sh) - 1);
    return (int)(F >> sh);
}

// The offset x - floor(x) as a double, exact (the same bits FP64 subtraction gives).
__device__ __forceinline__ double split_frac(const Split &s)
{
    if (s.e < 0) return __longlong_as_double((long long)s.fr);
    if (s.fr == 0) return 0.0;
    const int p = 63 - __clzll((long long)s.fr);       // top set bit; the value is 2^(p+e-52) * 1.m
    const unsigned long long mant = (s.fr << (52 - p)) & ((1ull << 52) - 1);
    return __longlong_as_double((long long)(((unsigned long long)(p + s.e + 971) << 52) | mant));
}

// round(offset * 2^48), ties up.
__device__ __forceinline__ unsigned long long split_frac48(const Split &s)
{
    if (s.e >= 4) return s.fr << (s.e - 4);
    if (s.e >= 0) {
        const int sh = 4 - s.e;
        return (s.fr + (1ull << (sh - 1))) >> sh;
    }
    const int E = (int)((s.fr >> 52) & 0x7ff);           // x in [0, 1): x * 2^48 = F * 2^(E - 1027)
    if (E == 0) return 0;
    const int sh = 1027 - E;                            // >= 5
    if (sh > 54) return 0;
    const unsigned long long F = (s.fr & ((1ull << 52) - 1)) | (1ull << 52);
    return (F + (1ull << (sh - 1))) >> sh;
}

// round(p * w / 2^48) for p, w <= 2^48, from the 96-bit product.
__device__ __forceinline__ unsigned long long mul48(unsigned long long p, unsigned long long w)
{
    const unsigned long long hi = __umul64hi(p, w), lo = p * w;
    const unsigned long long q = (hi << 16) | (lo >> 48);
    return q + ((lo >> 47) & 1ull);
}

// The 8 weights of a particle whose offsets are Rx, Ry, Rz (units of 2^-48), in
// units of 2^-48, summing to exactly 2^48; order x fastest as in add8 / deposit_global.
__device__ __forceinline__ void fixed_weights48(int conv, unsigned long long Rx, unsigned long long Ry,
                                                unsigned long long Rz, unsigned long long u[8])
{
    const bool ref = conv == OHPIC_WEIGHTS_REFERENCE;   // node floor(x) takes r (linear_scatter.f90:41-42)
    const unsigned long long X1 = ref ? kOne48 - Rx : Rx, X0 = kOne48 - X1;
    const unsigned long long wy1 = ref ? kOne48 - Ry : Ry, wz1 = ref ? kOne48 - Rz : Rz;
    const unsigned long long Y01 = min(mul48(X0, wy1), X0), Y11 = min(mul48(X1, wy1), X1);
    const unsigned long long Y00 = X0 - Y01, Y10 = X1 - Y11;
    const unsigned long long Z00 = min(mul48(Y00, wz1), Y00), Z10 = min(mul48(Y10, wz1), Y10);
    const unsigned long long Z01 = min(mul48(Y01, wz1), Y01), Z11 = min(mul48(Y11, wz1), Y11);
    u[0] = Y00 - Z00; u[1] = Y10 - Z10; u[2] = Y01 - Z01; u[3] = Y11 - Z11;
    u[4] = Z00; u[5] = Z10; u[6] = Z01; u[7] = Z11;
}

}  // namespace
}  // namespace ohpic
