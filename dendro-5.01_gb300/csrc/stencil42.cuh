// 4th-order finite-difference stencils on staged (shared-memory) lines, in
// the reference's rounding order: one rounding per operation, left to
// right, products by 2, 4, 8, 16 (exponent shifts) and the other integer tap
// products formed exactly on the integer pipes (exact_mul.cuh).  `c` points at the
// value of the current point, `s` is the stride along the axis, `pos` the
// point's index along an axis of n points (interior [3, n-3)), lo / hi the
// block's domain-boundary flags on that axis.
//
//   d1_42_at    deriv42_{x,y,z}  (BSSN_GR/src/derivs.cpp:11-242; identical in
//               CCZ4_GR/src/derivs.cpp), closures at 3,4 / n-5,n-4
//   d2_42_at    deriv42_{xx,yy,zz} (:244-490)
//   adv42_at    the upwind deriv42adv_{x,y,z} (CCZ4_GR/src/derivs.cpp:495-915;
//               BSSN_GR/src/derivs.cpp:494-913 differs in one closure test),
//               biased by sign(beta)
//   ko42c_at    the CCZ4 solver's ko_deriv42_{x,y,z}
//               (CCZ4_GR/src/derivs.cpp:917-1347): the centred stencil of
//               the neighbouring point at the first and last interior
//               point, closures on flagged faces
#pragma once
#include <cuda_runtime.h>

#include "exact_mul.cuh"

namespace dgb {
namespace {

struct Ax4 {
    double c12, half, c12sq, sq;   // (1/h)/12, 0.5/h, (1/h^2)/12, 1/h^2
    double pre, smr3, smr2, smr1;  // KO: -1/64/h, {59,43,49}/48*64*h
};
__device__ __forceinline__ Ax4 ax4(double h)
{
    Ax4 a;
    const double ih = 1.0 / h, ih2 = 1.0 / (h * h);
    a.c12 = ih / 12.0;
    a.half = 0.5 * ih;
    a.c12sq = ih2 / 12.0;
    a.sq = ih2;
    a.pre = -1.0 / 64.0 / h;
    a.smr3 = __dmul_rn(59.0 / 48.0 * 64, h);
    a.smr2 = __dmul_rn(43.0 / 48.0 * 64, h);
    a.smr1 = __dmul_rn(49.0 / 48.0 * 64, h);
    return a;
}

__device__ __forceinline__ double d1_42(const double *u, int s, double c12)
{
    double t = __dsub_rn(u[-2 * s], dgb_mul_pow2<3>(u[-s]));
    t = __dadd_rn(t, dgb_mul_pow2<3>(u[s]));
    t = __dsub_rn(t, u[2 * s]);
    return __dmul_rn(t, c12);
}
__device__ __forceinline__ double d2_42(const double *u, int s, double c12sq)
{
    double t = __dadd_rn(-u[-2 * s], dgb_mul_pow2<4>(u[-s]));
    t = __dsub_rn(t, dgb_mul_const<30>(u[0]));
    t = __dadd_rn(t, dgb_mul_pow2<4>(u[s]));
    t = __dsub_rn(t, u[2 * s]);
    return __dmul_rn(t, c12sq);
}

// (-3 u0 + 4 u1 - u2) * (0.5/h): the one-sided first derivative, forward
__device__ __forceinline__ double fwd3(const double *c, int s, double half)
{
    const double t = __dadd_rn(-dgb_mul_const<3>(c[0]), dgb_mul_pow2<2>(c[s]));
    return __dmul_rn(__dsub_rn(t, c[2 * s]), half);
}
// (u_-2 - 4 u_-1 + 3 u0) * (0.5/h): backward
__device__ __forceinline__ double bwd3(const double *c, int s, double half)
{
    const double t = __dsub_rn(c[-2 * s], dgb_mul_pow2<2>(c[-s]));
    return __dmul_rn(__dadd_rn(t, dgb_mul_const<3>(c[0])), half);
}
// (-u_-1 + u1) * (0.5/h)
__device__ __forceinline__ double ctr2(const double *c, int s, double half)
{
    return __dmul_rn(__dadd_rn(-c[-s], c[s]), half);
}

__device__ __forceinline__ double d1_42_at(const double *c, int s, int pos, int n, bool lo, bool hi,
                                           const Ax4 &a)
{
    if (lo && pos == 3) return fwd3(c, s, a.half);
    if (lo && pos == 4) return ctr2(c, s, a.half);
    if (hi && pos == n - 5) return ctr2(c, s, a.half);
    if (hi && pos == n - 4) return bwd3(c, s, a.half);
    return d1_42(c, s, a.c12);
}
__device__ __forceinline__ double d2_42_at(const double *c, int s, int pos, int n, bool lo, bool hi,
                                           const Ax4 &a)
{
    if (lo && pos == 3) {
        double t = __dsub_rn(dgb_mul2(c[0]), dgb_mul_const<5>(c[s]));
        t = __dadd_rn(t, dgb_mul_pow2<2>(c[2 * s]));
        return __dmul_rn(__dsub_rn(t, c[3 * s]), a.sq);
    }
    if ((lo && pos == 4) || (hi && pos == n - 5)) {
        const double t = __dsub_rn(c[-s], dgb_mul2(c[0]));
        return __dmul_rn(__dadd_rn(t, c[s]), a.sq);
    }
    if (hi && pos == n - 4) {
        double t = __dadd_rn(-c[-3 * s], dgb_mul_pow2<2>(c[-2 * s]));
        t = __dsub_rn(t, dgb_mul_const<5>(c[-s]));
        return __dmul_rn(__dadd_rn(t, dgb_mul2(c[0])), a.sq);
    }
    return d2_42(c, s, a.c12sq);
}

// upwind interior forms
__device__ __forceinline__ double adv42_pos(const double *c, int s, double c12)
{
    // (-3 u_-1 - 10 u0 + 18 u1 - 6 u2 + u3) / (12 h)
    double t = __dsub_rn(-dgb_mul_const<3>(c[-s]), dgb_mul_const<10>(c[0]));
    t = __dadd_rn(t, dgb_mul_const<18>(c[s]));
    t = __dsub_rn(t, dgb_mul_const<6>(c[2 * s]));
    t = __dadd_rn(t, c[3 * s]);
    return __dmul_rn(t, c12);
}
__device__ __forceinline__ double adv42_neg(const double *c, int s, double c12)
{
    // (-u_-3 + 6 u_-2 - 18 u_-1 + 10 u0 + 3 u1) / (12 h)
    double t = __dadd_rn(-c[-3 * s], dgb_mul_const<6>(c[-2 * s]));
    t = __dsub_rn(t, dgb_mul_const<18>(c[-s]));
    t = __dadd_rn(t, dgb_mul_const<10>(c[0]));
    t = __dadd_rn(t, dgb_mul_const<3>(c[s]));
    return __dmul_rn(t, c12);
}
// ccz4_hi: the CCZ4 file's test at the point ie-3 of a flagged high face
// (forward form where beta < 0); false: the BSSN_GR / QuadGrav files' test
// (forward form where beta > 0, BSSN_GR/src/derivs.cpp:579).
__device__ __forceinline__ double adv42_at(const double *c, int s, int pos, int n, bool lo, bool hi,
                                           double beta, const Ax4 &a, bool ccz4_hi = true)
{
    const int ie = n - 3;
    if (lo && pos <= 5) {
        if (pos == 3) return fwd3(c, s, a.half);
        if (pos == 4) return beta > 0.0 ? fwd3(c, s, a.half) : ctr2(c, s, a.half);
        return beta > 0.0 ? adv42_pos(c, s, a.c12) : bwd3(c, s, a.half);
    }
    if (hi && pos >= ie - 3) {
        if (pos == ie - 3)
            return (ccz4_hi ? beta < 0.0 : beta > 0.0) ? fwd3(c, s, a.half) : adv42_neg(c, s, a.c12);
        if (pos == ie - 2) return beta > 0.0 ? ctr2(c, s, a.half) : bwd3(c, s, a.half);
        return bwd3(c, s, a.half);
    }
    return beta > 0.0 ? adv42_pos(c, s, a.c12) : adv42_neg(c, s, a.c12);
}

// 7-point KO numerator  -u_-3 + 6 u_-2 - 15 u_-1 + 20 u0 - 15 u1 + 6 u2 - u3
// read from the line with step `st` (st = -s: the mirrored order the
// reference writes at the first interior point), centred at c
__device__ __forceinline__ double ko7(const double *c, int st)
{
    double t = __dadd_rn(-c[-3 * st], dgb_mul_const<6>(c[-2 * st]));
    t = __dsub_rn(t, dgb_mul_const<15>(c[-st]));
    t = __dadd_rn(t, dgb_mul_const<20>(c[0]));
    t = __dsub_rn(t, dgb_mul_const<15>(c[st]));
    t = __dadd_rn(t, dgb_mul_const<6>(c[2 * st]));
    return __dsub_rn(t, c[3 * st]);
}
__device__ __forceinline__ double ko42c_at(const double *c, int s, int pos, int n, bool lo, bool hi,
                                           const Ax4 &a)
{
    const int ie = n - 3;
    if (lo && pos <= 5) {
        if (pos == 3) {  // (u6 - 3 u5 + 3 u4 - u3) / smr3
            double t = __dsub_rn(c[3 * s], dgb_mul_const<3>(c[2 * s]));
            t = __dadd_rn(t, dgb_mul_const<3>(c[s]));
            return __ddiv_rn(__dsub_rn(t, c[0]), a.smr3);
        }
        if (pos == 4) {  // (u7 - 6 u6 + 12 u5 - 10 u4 + 3 u3) / smr2
            double t = __dsub_rn(c[3 * s], dgb_mul_const<6>(c[2 * s]));
            t = __dadd_rn(t, dgb_mul_const<12>(c[s]));
            t = __dsub_rn(t, dgb_mul_const<10>(c[0]));
            return __ddiv_rn(__dadd_rn(t, dgb_mul_const<3>(c[-s])), a.smr2);
        }
        // (u8 - 6 u7 + 15 u6 - 19 u5 + 12 u4 - 3 u3) / smr1
        double t = __dsub_rn(c[3 * s], dgb_mul_const<6>(c[2 * s]));
        t = __dadd_rn(t, dgb_mul_const<15>(c[s]));
        t = __dsub_rn(t, dgb_mul_const<19>(c[0]));
        t = __dadd_rn(t, dgb_mul_const<12>(c[-s]));
        return __ddiv_rn(__dsub_rn(t, dgb_mul_const<3>(c[-2 * s])), a.smr1);
    }
    if (hi && pos >= ie - 3) {
        if (pos == ie - 3) {  // (u-3 - 6 u-2 + 15 u-1 - 19 u0 + 12 u1 - 3 u2) / spr1
            double t = __dsub_rn(c[-3 * s], dgb_mul_const<6>(c[-2 * s]));
            t = __dadd_rn(t, dgb_mul_const<15>(c[-s]));
            t = __dsub_rn(t, dgb_mul_const<19>(c[0]));
            t = __dadd_rn(t, dgb_mul_const<12>(c[s]));
            return __ddiv_rn(__dsub_rn(t, dgb_mul_const<3>(c[2 * s])), a.smr1);
        }
        if (pos == ie - 2) {  // (u-3 - 6 u-2 + 12 u-1 - 10 u0 + 3 u1) / spr2
            double t = __dsub_rn(c[-3 * s], dgb_mul_const<6>(c[-2 * s]));
            t = __dadd_rn(t, dgb_mul_const<12>(c[-s]));
            t = __dsub_rn(t, dgb_mul_const<10>(c[0]));
            return __ddiv_rn(__dadd_rn(t, dgb_mul_const<3>(c[s])), a.smr2);
        }
        // (u-3 - 3 u-2 + 3 u-1 - u0) / spr3
        double t = __dsub_rn(c[-3 * s], dgb_mul_const<3>(c[-2 * s]));
        t = __dadd_rn(t, dgb_mul_const<3>(c[-s]));
        return __ddiv_rn(__dsub_rn(t, c[0]), a.smr3);
    }
    // first interior point: the stencil of pos 4, written from u7 down to u1;
    // last interior point: the stencil of pos n-5, written from u[n-2] down.
    // Centre and step are selected, not branched on, so a warp that holds an
    // end point of a line does not diverge.
    const int sh = pos == 3 ? s : (pos == ie - 1 ? -s : 0);
    return __dmul_rn(a.pre, ko7(c + sh, sh != 0 ? -s : s));
}

}  // namespace
}  // namespace dgb
