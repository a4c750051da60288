// Correctly rounded product of a double and a small positive integer
// constant, computed on the integer pipes.
//
// On GB300 the FP64 pipe retires 2 lanes per clock per SM while the integer
// ALU / IMAD pipes retire 64, so the stencil tap products RN(c * u)
// (c in {2, 6, 9, 15, 20, 27, 45, 270, 490}) are cheaper as integer
// arithmetic than as DMUL.  The result is bit-identical to the IEEE-754
// round-to-nearest-even product (the rounding the reference's stencils use):
// for x = m * 2^(e-1075) with a 53-bit significand m, c*m is an exact integer
// below 2^63; it is shifted back to 53 bits with round-half-even on the
// dropped bits.  Zero keeps its bits; subnormal, infinite/NaN inputs and
// results that could leave the normal range take the hardware multiply.
// Products by powers of two (2^K: the 4th-order stencils' 4, 8, 16) are an
// exponent shift (dgb_mul_pow2).
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DGB_XM_HD __host__ __device__ __forceinline__
#else
#define DGB_XM_HD static inline
#endif

DGB_XM_HD uint64_t dgb_dbits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

DGB_XM_HD double dgb_bitsd(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

// The hardware multiply for the rare inputs (subnormal, huge, non-finite),
// out of line on the device: inlined behind the exponent test, the compiler
// may turn the branch into a select and issue the DMUL on every call, which
// occupies the FP64 pipe (predicated off or not) and defeats the purpose.
#if defined(__CUDA_ARCH__)
template <uint32_t C>
__device__ __noinline__ double dgb_mul_hw(double x)
{
    return __dmul_rn((double)C, x);
}
#define DGB_XM_SLOW(C, x) dgb_mul_hw<C>(x)
#else
#define DGB_XM_SLOW(C, x) ((double)(C) * (x))
#endif

// 2^K as a double, exact for |K| < 31
template <int K>
struct dgb_pow2 {
    static constexpr double value = K >= 0 ? (double)(1u << (K >= 0 ? K : 0))
                                           : 1.0 / (double)(1u << (K < 0 ? -K : 0));
};

#if defined(__CUDA_ARCH__)
template <int K>
__device__ __noinline__ double dgb_mul_hw_pow2(double x)
{
    return __dmul_rn(dgb_pow2<K>::value, x);
}
#define DGB_XM_SLOW_POW2(K, x) dgb_mul_hw_pow2<K>(x)
#else
#define DGB_XM_SLOW_POW2(K, x) (dgb_pow2<K>::value * (x))
#endif

// RN(2^K * x) for a compile-time K, 1 <= |K| <= 8: exact, an exponent shift
// for normal x whose product stays normal; +-0 keeps its bits; subnormal,
// infinite/NaN inputs and products that would leave the normal range take
// the hardware multiply.
template <int K>
DGB_XM_HD double dgb_mul_pow2(double x)
{
    static_assert(K != 0 && K >= -8 && K <= 8, "small powers of two only");
    const uint64_t b = dgb_dbits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    const bool fast = K > 0 ? (e != 0u && e < 0x7FFu - (uint32_t)(K > 0 ? K : 0))
                            : (e > (uint32_t)(K < 0 ? -K : 0) && e != 0x7FFu);
    if (!fast) {
        if ((b << 1) == 0ull) return x;  // 2^K * (+-0) = +-0
        return DGB_XM_SLOW_POW2(K, x);
    }
    return dgb_bitsd(b + ((uint64_t)(int64_t)K << 52));
}

// 2 * x: exact, an exponent increment for normal x; +-0 stays +-0.
DGB_XM_HD double dgb_mul2(double x)
{
    const uint64_t b = dgb_dbits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    if (e == 0u || e >= 0x7FEu) {
        if ((b << 1) == 0ull) return x;
        return DGB_XM_SLOW(2u, x);
    }
    return dgb_bitsd(b + (1ull << 52));
}

// bit length of a constant: 2^(L-1) <= C < 2^L
constexpr int dgb_bitlen(uint32_t c) { return c ? 1 + dgb_bitlen(c >> 1) : 0; }

// RN(C * x) for a compile-time constant 2 <= C < 1024, with L = bitlen(C).
// The significand product p = m * C (m in [2^52, 2^53)) lies in
// [2^(51+L), 2^(53+L)); doubling it when it is below 2^(52+L) puts every
// product in [2^(52+L), 2^(53+L)), so the return to 53 bits is one fixed
// shift by L.  Round-half-even is an add before the shift: the dropped bits
// plus 2^(L-1) - 1 plus the kept lsb carry into the kept bits exactly when
// they exceed half, or equal it with the lsb odd.  The result's bits are
// the input's sign and exponent plus (shift - 1) << 52 plus the rounded
// significand, whose implicit bit (or its carry to 2^53) lifts the exponent
// by the remaining one (or two).  All shifts are by constants: about 20
// integer instructions, no count-leading-zeros, no variable 64-bit shifts.
template <uint32_t C>
DGB_XM_HD double dgb_mul_const(double x)
{
    static_assert(C >= 2 && C < 1024, "small integer constants only");
    constexpr int L = dgb_bitlen(C);
    const uint64_t b = dgb_dbits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    if (e - 1u >= 0x7FFu - 11u) {        // e == 0 (wraps) or e >= 0x7FF - 10
        if ((b << 1) == 0ull) return x;  // C * (+-0) = +-0
        return DGB_XM_SLOW(C, x);
    }
    const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    const uint64_t p = m * (uint64_t)C;  // exact, < 2^63
    const bool big = p >= (1ull << (52 + L));
    const uint64_t pn = big ? p : p << 1;
    const uint64_t t = pn + ((1ull << (L - 1)) - 1ull) + ((pn >> L) & 1ull);
    const uint64_t q = t >> L;           // in [2^52, 2^53]
    const uint64_t se = (b & 0xFFF0000000000000ull) + ((uint64_t)(big ? L - 1 : L - 2) << 52);
    return dgb_bitsd(se + q);
}
