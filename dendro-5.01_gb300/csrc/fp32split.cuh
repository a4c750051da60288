// FP32 arithmetic on split doubles, shared by the mixed-precision stencils
// of the BSSN (6th order) and CCZ4 (4th order) kernels.
//
// A double u is held as (hi, lo) floats with u = hi + lo up to 2^-48
// relative, split and widened back by integer bit operations only (no FP64
// pipe work).  On the hi part the stencils run compensated: every value is
// carried as s + e through error-free transformations (Knuth's TwoSum for
// differences and sums, the FMA TwoProduct for tap products) with explicit
// round-to-nearest intrinsics, and reaches FP64 as widen(s) + widen(e).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dgb {
namespace {

// A double u is held as (hi, lo) floats with u = hi + lo up to 2^-48 relative:
// hi = u with its mantissa truncated to 23 bits, lo = the remaining 29 bits,
// rounded to float.  Built with integer operations only.
struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 split_double(double u)
{
    const unsigned long long b = __double_as_longlong(u);
    const unsigned int sign = (unsigned int)(b >> 63);
    const int e = (int)((b >> 52) & 0x7FF);
    F2 r;
    if (e < 1023 - 126 + 1 || e > 1023 + 127) {  // |u| outside normal float range
        r.hi = 0.0f;
        r.lo = 0.0f;
        if (e > 1023 + 127) r.hi = __int_as_float((sign << 31) | 0x7F800000u);
        return r;
    }
    const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    r.hi = __int_as_float((sign << 31) | ((unsigned int)(e - 1023 + 127) << 23)
                          | (unsigned int)(mant >> 29));
    // remaining 29 mantissa bits times 2^(e-1023-52)
    const unsigned int rest = (unsigned int)(mant & 0x1FFFFFFFull);
    const int se = e - 1023 - 52;  // exponent of the lowest mantissa bit
    float scale;
    if (se >= -126) {
        scale = __int_as_float((unsigned int)(se + 127) << 23);
        r.lo = (float)rest * scale;
    } else {
        // scale below the normal float range: two steps
        scale = __int_as_float((unsigned int)(se + 64 + 127) << 23);
        r.lo = ((float)rest * scale) * 5.421010862427522e-20f;  // 2^-64
    }
    if (sign) r.lo = -r.lo;
    return r;
}

// float -> double by bit manipulation (exact; zero and normal floats).
__device__ __forceinline__ double widen(float f)
{
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xFF;
    if (e == 0) return 0.0;  // zero (float subnormals flush; never reached by derivative data)
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    const unsigned long long exp = (unsigned long long)(e - 127 + 1023) << 52;
    const unsigned long long man = (unsigned long long)(b & 0x7FFFFF) << 29;
    return __longlong_as_double(sign | exp | man);
}

// KO numerator: -(t3) + 6 t2 - 15 t1 with t_k = (u[k]-u0)+(u[-k]-u0)
// (the 20 u0 term is absorbed: -2 + 12 - 30 + 20 = 0)
__device__ __forceinline__ float nko_32(const float *u, int s)
{
    const float c = u[0];
    const float t1 = (u[s] - c) + (u[-s] - c), t2 = (u[2 * s] - c) + (u[-2 * s] - c),
                t3 = (u[3 * s] - c) + (u[-3 * s] - c);
    return fmaf(-15.0f, t1, fmaf(6.0f, t2, -t3));
}

// Compensated FP32 stencils for the hi plane.  A value is carried as s + e
// (|e| <= ulp(s)/2) through error-free transformations: Knuth's TwoSum for
// every difference and sum, the FMA TwoProduct for every tap product, all
// in FP32 with explicit round-to-nearest intrinsics (no contraction, no
// reassociation).  The numerator then reaches FP64 as widen(s) + widen(e),
// so neither the differences of nearly equal hi values nor the final float
// rounding of the sum limits the accuracy; the FP64 side is one add and the
// scale multiply per stencil.
struct FP2 {
    float s, e;
};
__device__ __forceinline__ FP2 two_sum(float a, float b)
{
    FP2 r;
    r.s = __fadd_rn(a, b);
    const float bb = __fsub_rn(r.s, a);
    r.e = __fadd_rn(__fsub_rn(a, __fsub_rn(r.s, bb)), __fsub_rn(b, bb));
    return r;
}
__device__ __forceinline__ FP2 add2(FP2 x, FP2 y)
{
    FP2 r = two_sum(x.s, y.s);
    r.e = __fadd_rn(r.e, __fadd_rn(x.e, y.e));
    return r;
}
__device__ __forceinline__ FP2 mulc2(float c, FP2 x)
{
    FP2 r;
    r.s = __fmul_rn(c, x.s);
    r.e = __fadd_rn(__fmaf_rn(c, x.s, -r.s), __fmul_rn(c, x.e));
    return r;
}
// (u[k] - c) + (u[-k] - c)
__device__ __forceinline__ FP2 sym2(const float *u, int k, float c)
{
    return add2(two_sum(u[k], -c), two_sum(u[-k], -c));
}
__device__ __forceinline__ FP2 nko_c(const float *u, int s)
{
    const float c = u[0];
    FP2 t3 = sym2(u, 3 * s, c);
    t3.s = -t3.s;
    t3.e = -t3.e;
    return add2(add2(mulc2(-15.0f, sym2(u, s, c)), mulc2(6.0f, sym2(u, 2 * s, c))), t3);
}
__device__ __forceinline__ double fp2_widen(FP2 h) { return __dadd_rn(widen(h.s), widen(h.e)); }

// A double scale held as a float pair c = hi + lo (2^-48 relative), so that
// the scaling of a stencil numerator stays on the FP32 pipes: TwoProduct for
// s * hi, the small cross terms in FP32; the FP64 side is the one add of
// fp2_widen.  Built once per tile.
struct FC {
    float hi, lo;
};
__device__ __forceinline__ FC split_const(double c)
{
    FC r;
    r.hi = __double2float_rn(c);
    r.lo = __double2float_rn(c - (double)r.hi);
    return r;
}
__device__ __forceinline__ FP2 mulfc(FP2 x, FC c)
{
    FP2 r;
    r.s = __fmul_rn(x.s, c.hi);
    r.e = __fadd_rn(__fmaf_rn(x.s, c.hi, -r.s), __fadd_rn(__fmul_rn(x.s, c.lo), __fmul_rn(x.e, c.hi)));
    return r;
}

}  // namespace
}  // namespace dgb
