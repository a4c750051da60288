// BSSN right-hand side on padded octant blocks: one persistent, work-queued
// launch over all blocks of a plan, whatever their sizes.
//
// Work item = a rectangular tile (<= TX x TY x TZ interior points) of one
// block.  A CTA takes items from a global atomic queue and, per item:
//   phase D  for each of the 24 fields: stage the padded tile region
//            (tile + 3 on each side) in shared memory (cp.async, double
//            buffered: field v+1 lands while field v is differentiated),
//            then write every derivative the algebra reads, plus the KO sum
//            kx+ky+kz, to the CTA's slice of the derivative workspace;
//   phase A  one thread per tile point: the generated algebra
//            (bssn_algebra.cuh) reads the fields and the workspace and
//            writes rhs = algebra + sigma * KO for the interior point.
//
// Reference behaviour reproduced (BSSN_GR/src/rhs.cpp:86-392 with the
// QuadGrav 6th-order binding, QuadGrav/include/derivs.h:80-97):
//   first derivatives  deriv64_{x,y,z}   (QuadGrav/src/derivs.cpp:2141-2560)
//   second             deriv64_{xx,yy,zz} (:2569-2910)
//   mixed              d_y(d_x u), d_z(d_x u), d_z(d_y u)
//                      (BSSN_GR/scripts/bssnrhs_derivs.h), so d_x u is formed
//                      on the tile plus 3 rows in y and z, d_y u plus 3 in z
//   advective          deriv64adv_* = centred deriv64 (:2913-2953), hence the
//                      advective slots alias the first-derivative slots
//   KO                 ko_deriv42_{x,y,z} (BSSN_GR/src/derivs.cpp:914-1410),
//                      rhs += sigma * (kx + ky + kz) (rhs.cpp:336-373)
// Domain-boundary blocks (bflag != 0) take the one-sided closures in phase D
// and the outgoing-radiation condition bssn_bcs on their flagged faces in
// phase A (BSSN_GR/src/rhs.cpp:838-982), in FP64 in both precisions.
//
// The mixed-precision variant (MIXED = true) splits each staged FP64 value
// into a float pair hi + lo by integer bit operations (no FP64 pipe work)
// and evaluates every stencil in FP32 on symmetric differences
// (u[+k] - u[-k], (u[k] - u0) + (u[-k] - u0)): compensated (TwoSum /
// FMA TwoProduct) on the hi part, plain on the lo part.  Each stencil's
// float pair is scaled by its float-pair scale (and KO summed over the three
// directions) in FP32 pairs and widened to FP64 by integer bit operations
// with one FP64 add; the algebra, the RK update and all field I/O stay FP64.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bssn_algebra.cuh"
#include "dgb_internal.h"
#include "exact_mul.cuh"
#include "fp32split.cuh"
#include "tile_index.cuh"

namespace dgb {
namespace {

#ifndef DGB_RHS_THREADS
#define DGB_RHS_THREADS 256
#endif
constexpr int kThreads = DGB_RHS_THREADS;
#ifndef DGB_RHS_MIN_CTAS
#define DGB_RHS_MIN_CTAS 2
#endif
// CTAs per SM the register budget is sized for (255 registers at 1, 128 at 2)
constexpr int kMinBlocks = DGB_RHS_MIN_CTAS;

// fields with second derivatives, VAR order -> D2 index (or -1)
__constant__ int8_t c_d2index[NV] = {0, 1, -1, -1, -1, -1, 2, 3, 4, -1, -1, -1,
                                     5, 6, 7, 8, 9, 10, -1, -1, -1, -1, -1, -1};

// ---------------------------------------------------------------- FP64 stencils
// The reference's rounding sequence, operation by operation: every tap is a
// rounded product added left to right, then one rounded scale
// (QuadGrav/src/derivs.cpp:2164-2170, :2592-2598; BSSN_GR/src/derivs.cpp:963-971).
// Explicit _rn intrinsics keep nvcc from contracting to FMA: an FMA rounds
// once where the reference rounds twice, and on fields of size ~1 whose
// right-hand side is ~1e-6 that difference alone reaches 1e-11 normwise.
// Multiplications by -1, 1 are exact and are not issued; the tap products
// by the integer coefficients are formed on the integer pipes, bit-identical
// to DMUL (exact_mul.cuh), which leaves the FP64 pipe the adds and the scale.
__device__ __forceinline__ double d1_64(const double *u, int s, double c60)
{
    double t = __dadd_rn(-u[-3 * s], dgb_mul_const<9>(u[-2 * s]));
    t = __dsub_rn(t, dgb_mul_const<45>(u[-s]));
    t = __dadd_rn(t, dgb_mul_const<45>(u[s]));
    t = __dsub_rn(t, dgb_mul_const<9>(u[2 * s]));
    t = __dadd_rn(t, u[3 * s]);
    return __dmul_rn(t, c60);
}
__device__ __forceinline__ double d2_64(const double *u, int s, double c180)
{
    double t = __dsub_rn(dgb_mul2(u[-3 * s]), dgb_mul_const<27>(u[-2 * s]));
    t = __dadd_rn(t, dgb_mul_const<270>(u[-s]));
    t = __dsub_rn(t, dgb_mul_const<490>(u[0]));
    t = __dadd_rn(t, dgb_mul_const<270>(u[s]));
    t = __dsub_rn(t, dgb_mul_const<27>(u[2 * s]));
    t = __dadd_rn(t, dgb_mul2(u[3 * s]));
    return __dmul_rn(t, c180);
}
__device__ __forceinline__ double ko_64(const double *u, int s, double pre)
{
    double t = __dadd_rn(-u[-3 * s], dgb_mul_const<6>(u[-2 * s]));
    t = __dsub_rn(t, dgb_mul_const<15>(u[-s]));
    t = __dadd_rn(t, dgb_mul_const<20>(u[0]));
    t = __dsub_rn(t, dgb_mul_const<15>(u[s]));
    t = __dadd_rn(t, dgb_mul_const<6>(u[2 * s]));
    t = __dsub_rn(t, u[3 * s]);
    return __dmul_rn(pre, t);
}

// ---------------------------------------------------------------- boundary closures
// One-sided stencils at domain-boundary faces (bflag bit 2a: low side of
// axis a, bit 2a+1: high side; OCT_DIR_* of include/dendro.h:84-89), as the
// reference writes them: first derivative QuadGrav/src/derivs.cpp:2174-2230
// (scale (1/h)/12), second :2602-2650 (scale (1/h^2)/12), KO
// BSSN_GR/src/derivs.cpp:997-1075 (divided by {59,43,49}/48*64*h).  Taps are
// (index along the axis, coefficient) in evaluation order; low-side indices
// are absolute (3..8), high-side ones relative to ie = n - 3.  Rounded
// product per tap, added left to right: the reference's rounding.
struct Taps {
    int n;
    int idx[6];
    double c[6];
};
__constant__ Taps c_d1lo[3] = {{5, {3, 4, 5, 6, 7}, {-25.0, 48.0, -36.0, 16.0, -3.0}},
                               {5, {3, 4, 5, 6, 7}, {-3.0, -10.0, 18.0, -6.0, 1.0}},
                               {4, {3, 4, 6, 7}, {1.0, -8.0, 8.0, -1.0}}};
__constant__ Taps c_d1hi[3] = {{4, {-5, -4, -2, -1}, {1.0, -8.0, 8.0, -1.0}},
                               {5, {-5, -4, -3, -2, -1}, {-1.0, 6.0, -18.0, 10.0, 3.0}},
                               {5, {-5, -4, -3, -2, -1}, {3.0, -16.0, 36.0, -48.0, 25.0}}};
__constant__ Taps c_d2lo[3] = {{5, {3, 4, 5, 6, 7}, {35.0, -104.0, 114.0, -56.0, 11.0}},
                               {5, {3, 4, 5, 6, 7}, {11.0, -20.0, 6.0, 4.0, -1.0}},
                               {5, {3, 4, 5, 6, 7}, {-1.0, 16.0, -30.0, 16.0, -1.0}}};
__constant__ Taps c_d2hi[3] = {{5, {-5, -4, -3, -2, -1}, {-1.0, 16.0, -30.0, 16.0, -1.0}},
                               {5, {-5, -4, -3, -2, -1}, {-1.0, 4.0, 6.0, -20.0, 11.0}},
                               {5, {-5, -4, -3, -2, -1}, {11.0, -56.0, 114.0, -104.0, 35.0}}};
__constant__ Taps c_kolo[3] = {{4, {6, 5, 4, 3}, {1.0, -3.0, 3.0, -1.0}},
                               {5, {7, 6, 5, 4, 3}, {1.0, -6.0, 12.0, -10.0, 3.0}},
                               {6, {8, 7, 6, 5, 4, 3}, {1.0, -6.0, 15.0, -19.0, 12.0, -3.0}}};
__constant__ Taps c_kohi[3] = {{6, {-6, -5, -4, -3, -2, -1}, {1.0, -6.0, 15.0, -19.0, 12.0, -3.0}},
                               {5, {-5, -4, -3, -2, -1}, {1.0, -6.0, 12.0, -10.0, 3.0}},
                               {4, {-4, -3, -2, -1}, {1.0, -3.0, 3.0, -1.0}}};

// c points at the value of the current point (index pos along the axis,
// stride s); tap index a is read at c[(a + base - pos) * s].
__device__ __forceinline__ double eval_taps(const double *c, int s, int shift, const Taps &t)
{
    double acc = __dmul_rn(t.c[0], c[(t.idx[0] + shift) * s]);
    for (int q = 1; q < t.n; q++) acc = __dadd_rn(acc, __dmul_rn(t.c[q], c[(t.idx[q] + shift) * s]));
    return acc;
}

// Per-axis scales of one block (h = block spacing along the axis).
struct AxisScale {
    double c60, c12, c180, c12sq, pre, smr[3];
};

__device__ __forceinline__ AxisScale axis_scale(double h)
{
    AxisScale a;
    a.c60 = (1.0 / h) / 60.0;
    a.c12 = (1.0 / h) / 12.0;
    a.c180 = (1.0 / (h * h)) / 180.0;
    a.c12sq = (1.0 / (h * h)) / 12.0;
    a.pre = -1.0 / 64.0 / h;
    a.smr[0] = __dmul_rn(59.0 / 48.0 * 64, h);  // point 3 / ie-1
    a.smr[1] = __dmul_rn(43.0 / 48.0 * 64, h);  // point 4 / ie-2
    a.smr[2] = __dmul_rn(49.0 / 48.0 * 64, h);  // point 5 / ie-3
    return a;
}

// Stencils at index pos of an axis of n points with boundary flags lo/hi.
__device__ __forceinline__ double d1_at(const double *c, int s, int pos, int n, bool lo, bool hi,
                                        const AxisScale &a)
{
    if (lo && pos < 6) return __dmul_rn(eval_taps(c, s, -pos, c_d1lo[pos - 3]), a.c12);
    if (hi && pos >= n - 6) return __dmul_rn(eval_taps(c, s, n - 3 - pos, c_d1hi[pos - (n - 6)]), a.c12);
    return d1_64(c, s, a.c60);
}
__device__ __forceinline__ double d2_at(const double *c, int s, int pos, int n, bool lo, bool hi,
                                        const AxisScale &a)
{
    if (lo && pos < 6) return __dmul_rn(eval_taps(c, s, -pos, c_d2lo[pos - 3]), a.c12sq);
    if (hi && pos >= n - 6) return __dmul_rn(eval_taps(c, s, n - 3 - pos, c_d2hi[pos - (n - 6)]), a.c12sq);
    return d2_64(c, s, a.c180);
}
__device__ __forceinline__ double ko_at(const double *c, int s, int pos, int n, bool lo, bool hi,
                                        const AxisScale &a)
{
    if (lo && pos < 6) return __ddiv_rn(eval_taps(c, s, -pos, c_kolo[pos - 3]), a.smr[pos - 3]);
    if (hi && pos >= n - 6) {
        const int q = pos - (n - 6);
        return __ddiv_rn(eval_taps(c, s, n - 3 - pos, c_kohi[q]), a.smr[2 - q]);
    }
    return ko_64(c, s, a.pre);
}

// bssn_bcs falloff / asymptotic value per variable (BSSN_GR/src/rhs.cpp:269-321).
__constant__ double c_bc_falloff[NV] = {1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1,
                                        1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2};
__constant__ double c_bc_asym[NV] = {1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     1, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0, 0};

// ---------------------------------------------------------------- FP32 stencils (6th order)
// first derivative numerator on a float row: 45 a1 - 9 a2 + a3, a_k = u[k]-u[-k]
__device__ __forceinline__ float n1_32(const float *u, int s)
{
    const float a1 = u[s] - u[-s], a2 = u[2 * s] - u[-2 * s], a3 = u[3 * s] - u[-3 * s];
    return fmaf(45.0f, a1, fmaf(-9.0f, a2, a3));
}
// second derivative numerator: 270 s1 - 27 s2 + 2 s3, s_k = (u[k]-u0)+(u[-k]-u0)
__device__ __forceinline__ float n2_32(const float *u, int s)
{
    const float c = u[0];
    const float s1 = (u[s] - c) + (u[-s] - c), s2 = (u[2 * s] - c) + (u[-2 * s] - c),
                s3 = (u[3 * s] - c) + (u[-3 * s] - c);
    return fmaf(270.0f, s1, fmaf(-27.0f, s2, 2.0f * s3));
}
__device__ __forceinline__ FP2 n1_c(const float *u, int s)
{
    const FP2 a1 = two_sum(u[s], -u[-s]), a2 = two_sum(u[2 * s], -u[-2 * s]),
              a3 = two_sum(u[3 * s], -u[-3 * s]);
    return add2(add2(mulc2(45.0f, a1), mulc2(-9.0f, a2)), a3);
}
__device__ __forceinline__ FP2 n2_c(const float *u, int s)
{
    const float c = u[0];
    return add2(add2(mulc2(270.0f, sym2(u, s, c)), mulc2(-27.0f, sym2(u, 2 * s, c))),
                mulc2(2.0f, sym2(u, 3 * s, c)));
}
// ---------------------------------------------------------------- cp.async
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned int s = (unsigned int)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ---------------------------------------------------------------- algebra I/O
struct AlgIOw {
    const double *const *uu;
    double *const *rr;
    const double *S;
    int pmax, p;
    uint64_t gi;
    double sigma;
    __device__ __forceinline__ double u(int v) const { return __ldg(uu[v] + gi); }
    __device__ __forceinline__ double d(int s) const { return S[(size_t)s * pmax + p]; }
    // rhs += sigma * (kx + ky + kz) with the reference's two roundings
    // (BSSN_GR/src/rhs.cpp:336-373); the KO sum is stored pre-added.
    __device__ __forceinline__ void out(int v, double x) const
    {
        rr[v][gi] = __dadd_rn(x, __dmul_rn(sigma, S[(size_t)(DGB_NUM_DERIV + v) * pmax + p]));
    }
};

// Gather mode (fused unzip): the fields are the zipped state and the
// interpolated-point buffer, read through the padded point's gather index;
// the RHS at a padded point goes to its zipped node when the point owns it.
// The algebra's results are stored unconditionally (into the KO slot each
// one has just consumed) and copied to the owned node afterwards: a store
// behind a branch would split the algebra into other basic blocks than in
// the plain kernel, where the compiler may contract other multiply-adds,
// and the fused step would no longer give the unfused step's bits.
__device__ __forceinline__ const double *gather_src(const RhsArgs &a, int v, uint32_t g)
{
    return g < a.ndof ? a.u[v] + g : a.ib[v] + (g - a.ndof);
}

struct AlgIOg {
    const RhsArgs *a;
    double *S;
    int pmax, p;
    uint32_t g, o;  // gather index and owned zipped node (0xFFFFFFFF: none) of the point
    double sigma;
    __device__ __forceinline__ double u(int v) const { return __ldg(gather_src(*a, v, g)); }
    __device__ __forceinline__ double d(int s) const { return S[(size_t)s * pmax + p]; }
    __device__ __forceinline__ void out(int v, double x) const
    {
        double *ko = S + (size_t)(DGB_NUM_DERIV + v) * pmax + p;
        *ko = __dadd_rn(x, __dmul_rn(sigma, *ko));
    }
    __device__ __forceinline__ void flush() const
    {
        if (o == 0xFFFFFFFFu) return;
        for (int v = 0; v < NV; v++) a->rhs[v][o] = S[(size_t)(DGB_NUM_DERIV + v) * pmax + p];
    }
};

struct AlgPrm {
    double l1, l2, l3, l4, lf0, lf1;
};

template <int TX, int TY, int TZ>
struct Geo {
    static constexpr int PX = TX + 6, PY = TY + 6, PZ = TZ + 6;
    static constexpr int FBUF = PX * PY * PZ;        // staged field (doubles)
    static constexpr int DXB = TX * PY * PZ;         // d_x box (cross region)
    static constexpr int DYB = TX * TY * PZ;         // d_y box
    static constexpr int PMAX = TX * TY * TZ;
    // DivBy (tile_index.cuh) splits indices q < FBUF by extents < 32 exactly
    static_assert(FBUF < (1 << 13) && PX < 32 && PY < 32 && PZ < 32, "tile too large for DivBy");
};

template <int TX, int TY, int TZ, bool MIXED, bool GATHER = false>
struct Smem {
    using G = Geo<TX, TY, TZ>;
    // FP64: two field buffers + d_x box + d_y box (doubles)
    // MIXED: two field buffers (doubles) + hi/lo float planes + float-pair boxes
    // GATHER: + the staged region's gather indices (uint32)
    static constexpr size_t base = MIXED
        ? (2 * G::FBUF * 8 + 2 * G::FBUF * 4 + 2 * (G::DXB + G::DYB) * 4)
        : (2 * G::FBUF * 8 + (G::DXB + G::DYB) * 8);
    // the gather indices are staged only where two CTAs per SM still fit
    // (228 KB per SM, 1 KB of it reserved per CTA); deeper tiles read them
    // from global memory (L1-resident) once per field instead
    static constexpr bool gidx_smem = GATHER && 2 * (base + G::FBUF * 4 + 1024) <= 228 * 1024;
    static constexpr size_t bytes = base + (gidx_smem ? G::FBUF * 4 : 0);
};

// One work item (a tile of one block): phase D then phase A.  S is this
// CTA's slice of the derivative workspace.
template <int TX, int TY, int TZ, bool MIXED, bool GATHER = false>
__device__ __forceinline__ void rhs_item(const RhsArgs &args, const WorkItem &w,
                                         const DevBlock &blk, double *S, const AlgPrm &aprm)
{
    using G = Geo<TX, TY, TZ>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *fb0 = reinterpret_cast<double *>(smem_raw);
    double *fb1 = fb0 + G::FBUF;
    // FP64 boxes
    double *dxb = fb1 + G::FBUF;
    double *dyb = dxb + G::DXB;
    // FP32 planes (MIXED): split field, and the d_x / d_y boxes as s + e pairs
    float *fhi = reinterpret_cast<float *>(fb1 + G::FBUF);
    float *flo = fhi + G::FBUF;
    float *dxs = flo + G::FBUF;
    float *dxe = dxs + G::DXB;
    float *dys = dxe + G::DXB;
    float *dye = dys + G::DYB;
    const int tid = threadIdx.x;

    const int nx = blk.sz[0], ny = blk.sz[1];
    const int ex = w.e[0], ey = w.e[1], ez = w.e[2];
    const int px = ex + 6, py = ey + 6, pz = ez + 6;
    const int npad = px * py * pz;
    const int P = ex * ey * ez;
    const DivBy dex(ex), dey(ey), dbx(ey + 6), dpx(px), dpy(py);
    // region start in padded block coordinates = interior origin
    const uint64_t rbase = blk.offset + (uint64_t)w.o[0]
                         + (uint64_t)nx * ((uint64_t)w.o[1] + (uint64_t)ny * w.o[2]);
    const double hx = blk.h[0], hy = blk.h[1], hz = blk.h[2];
    const double c60[3] = {(1.0 / hx) / 60.0, (1.0 / hy) / 60.0, (1.0 / hz) / 60.0};
    const double c180[3] = {(1.0 / (hx * hx)) / 180.0, (1.0 / (hy * hy)) / 180.0,
                            (1.0 / (hz * hz)) / 180.0};
    const double ko[3] = {-1.0 / 64.0 / hx, -1.0 / 64.0 / hy, -1.0 / 64.0 / hz};
    const int sy = px, sz = px * py;  // strides in the staged region
    const int nz = blk.sz[2];
    const uint32_t bflag = blk.bflag;
    const bool blo[3] = {(bflag & 1u) != 0, (bflag & 4u) != 0, (bflag & 16u) != 0};
    const bool bhi[3] = {(bflag & 2u) != 0, (bflag & 8u) != 0, (bflag & 32u) != 0};
    AxisScale ax[3];
    if (bflag != 0) {
        ax[0] = axis_scale(hx);
        ax[1] = axis_scale(hy);
        ax[2] = axis_scale(hz);
    }

    // gather mode: the staged region's gather indices, loaded once per item
    constexpr bool kGidxSmem = Smem<TX, TY, TZ, MIXED, GATHER>::gidx_smem;
    uint32_t *gidx = reinterpret_cast<uint32_t *>(smem_raw + Smem<TX, TY, TZ, MIXED>::base);
    if (GATHER && kGidxSmem) {
        const uint32_t *gm = args.gmap + rbase;
        for (int q = tid; q < npad; q += kThreads) {
            int i, j, k;
            split3(q, dpx, dpy, i, j, k);
            gidx[q] = __ldg(gm + i + (uint64_t)nx * (j + (uint64_t)ny * k));
        }
        __syncthreads();
    }
    auto issue_load = [&](int v, double *dst) {
        if (GATHER && kGidxSmem) {
            for (int q = tid; q < npad; q += kThreads) cp_async8(dst + q, gather_src(args, v, gidx[q]));
        } else if (GATHER) {
            const uint32_t *gm = args.gmap + rbase;
            for (int q = tid; q < npad; q += kThreads) {
                int i, j, k;
                split3(q, dpx, dpy, i, j, k);
                cp_async8(dst + q, gather_src(args, v, __ldg(gm + i + (uint64_t)nx * (j + (uint64_t)ny * k))));
            }
        } else {
            const double *src = args.u[v] + rbase;
            for (int q = tid; q < npad; q += kThreads) {
                int i, j, k;
                split3(q, dpx, dpy, i, j, k);
                cp_async8(dst + q, src + i + (uint64_t)nx * (j + (uint64_t)ny * k));
            }
        }
        cp_async_commit();
    };

    // ------------------------------------------------------------ phase D
    issue_load(0, fb0);
    for (int v = 0; v < NV; v++) {
        double *F = (v & 1) ? fb1 : fb0;
        cp_async_wait<0>();
        // one barrier per field: field v is staged and visible, and every
        // thread is done with field v-1 (its buffer, the boxes); the next
        // field's load then goes into field v-1's buffer
        __syncthreads();
        if (v + 1 < NV) issue_load(v + 1, (v & 1) ? fb0 : fb1);
        const int q2 = c_d2index[v];
        double *Sg = S + (size_t)(3 * v) * G::PMAX;
        double *Sko = S + (size_t)(DGB_NUM_DERIV + v) * G::PMAX;
        if (bflag != 0) {
            // ---------------- domain-boundary block: closures, FP64 in both precisions
            if (q2 < 0) {
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int pi = w.o[0] + ti + 3, pj = w.o[1] + tj + 3, pk = w.o[2] + tk + 3;
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sg[p] = d1_at(c, 1, pi, nx, blo[0], bhi[0], ax[0]);
                    Sg[G::PMAX + p] = d1_at(c, sy, pj, ny, blo[1], bhi[1], ax[1]);
                    Sg[2 * G::PMAX + p] = d1_at(c, sz, pk, nz, blo[2], bhi[2], ax[2]);
                    Sko[p] = ko_at(c, 1, pi, nx, blo[0], bhi[0], ax[0])
                           + ko_at(c, sy, pj, ny, blo[1], bhi[1], ax[1])
                           + ko_at(c, sz, pk, nz, blo[2], bhi[2], ax[2]);
                }
            } else {
                double *S2 = S + (size_t)(DGB_NUM_GRAD + 6 * q2) * G::PMAX;
                const int bx_y = ey + 6;
                const int nA = ex * bx_y * ez, nB = ex * ey * 6;
                for (int q = tid; q < nA + nB; q += kThreads) {
                    int ti, tj, tk;
                    if (q < nA) {
                        split3(q, dex, dbx, ti, tj, tk);
                        tk += 3;
                    } else {
                        const int q3 = q - nA;
                        int kk;  // 0..5
                        split3(q3, dex, dey, ti, tj, kk);
                        tj += 3;
                        tk = kk < 3 ? kk : ez + kk;
                    }
                    const double *c = F + (ti + 3) + sy * tj + sz * tk;
                    dxb[ti + ex * (tj + bx_y * tk)] = d1_at(c, 1, w.o[0] + ti + 3, nx, blo[0], bhi[0], ax[0]);
                }
                const int nC = ex * ey * pz;
                for (int q = tid; q < nC; q += kThreads) {
                    int ti, tj, tk;
                    split3(q, dex, dey, ti, tj, tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * tk;
                    dyb[q] = d1_at(c, sy, w.o[1] + tj + 3, ny, blo[1], bhi[1], ax[1]);
                }
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int pi = w.o[0] + ti + 3, pj = w.o[1] + tj + 3, pk = w.o[2] + tk + 3;
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sg[2 * G::PMAX + p] = d1_at(c, sz, pk, nz, blo[2], bhi[2], ax[2]);
                    S2[0 * G::PMAX + p] = d2_at(c, 1, pi, nx, blo[0], bhi[0], ax[0]);
                    S2[3 * G::PMAX + p] = d2_at(c, sy, pj, ny, blo[1], bhi[1], ax[1]);
                    S2[5 * G::PMAX + p] = d2_at(c, sz, pk, nz, blo[2], bhi[2], ax[2]);
                    Sko[p] = ko_at(c, 1, pi, nx, blo[0], bhi[0], ax[0])
                           + ko_at(c, sy, pj, ny, blo[1], bhi[1], ax[1])
                           + ko_at(c, sz, pk, nz, blo[2], bhi[2], ax[2]);
                }
                __syncthreads();
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int pj = w.o[1] + tj + 3, pk = w.o[2] + tk + 3;
                    const double *cx = dxb + ti + ex * ((tj + 3) + bx_y * (tk + 3));
                    const double *cy = dyb + ti + ex * (tj + ey * (tk + 3));
                    Sg[p] = cx[0];
                    Sg[G::PMAX + p] = cy[0];
                    S2[1 * G::PMAX + p] = d1_at(cx, ex, pj, ny, blo[1], bhi[1], ax[1]);
                    S2[2 * G::PMAX + p] = d1_at(cx, ex * bx_y, pk, nz, blo[2], bhi[2], ax[2]);
                    S2[4 * G::PMAX + p] = d1_at(cy, ex * ey, pk, nz, blo[2], bhi[2], ax[2]);
                }
            }
        } else if constexpr (!MIXED) {
            if (q2 < 0) {
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sg[p] = d1_64(c, 1, c60[0]);
                    Sg[G::PMAX + p] = d1_64(c, sy, c60[1]);
                    Sg[2 * G::PMAX + p] = d1_64(c, sz, c60[2]);
                    Sko[p] = ko_64(c, 1, ko[0]) + ko_64(c, sy, ko[1]) + ko_64(c, sz, ko[2]);
                }
            } else {
                double *S2 = S + (size_t)(DGB_NUM_GRAD + 6 * q2) * G::PMAX;
                // (1a) d_x on the cross region: x in tile, (y ext, z tile) or (y tile, z ext),
                // and (1b) d_y on x, y in tile, z extended, in one pass: every item is one
                // first-derivative stencil, so the threads share the two boxes evenly
                const int bx_y = ey + 6;  // d_x box rows
                const int nA = ex * bx_y * ez, nB = ex * ey * 6;
                const int nC = ex * ey * pz;
                for (int q = tid; q < nA + nB + nC; q += kThreads) {
                    int ti, tj, tk;  // box coords: tj in [0,ey+6), tk in [0,ez+6)
                    if (q < nA + nB) {
                        if (q < nA) {
                            split3(q, dex, dbx, ti, tj, tk);
                            tk += 3;
                        } else {
                            const int q3 = q - nA;
                            int kk;  // 0..5
                            split3(q3, dex, dey, ti, tj, kk);
                            tj += 3;
                            tk = kk < 3 ? kk : ez + kk;
                        }
                        const double *c = F + (ti + 3) + sy * tj + sz * tk;
                        dxb[ti + ex * (tj + bx_y * tk)] = d1_64(c, 1, c60[0]);
                    } else {
                        const int qc = q - nA - nB;
                        split3(qc, dex, dey, ti, tj, tk);
                        const double *c = F + (ti + 3) + sy * (tj + 3) + sz * tk;
                        dyb[qc] = d1_64(c, sy, c60[1]);
                    }
                }
                // (1c) pointwise: d_z, xx, yy, zz, KO
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sg[2 * G::PMAX + p] = d1_64(c, sz, c60[2]);
                    S2[0 * G::PMAX + p] = d2_64(c, 1, c180[0]);
                    S2[3 * G::PMAX + p] = d2_64(c, sy, c180[1]);
                    S2[5 * G::PMAX + p] = d2_64(c, sz, c180[2]);
                    Sko[p] = ko_64(c, 1, ko[0]) + ko_64(c, sy, ko[1]) + ko_64(c, sz, ko[2]);
                }
                __syncthreads();
                // (2) mixed from the boxes; d_x, d_y at tile points
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const double *cx = dxb + ti + ex * ((tj + 3) + bx_y * (tk + 3));
                    const double *cy = dyb + ti + ex * (tj + ey * (tk + 3));
                    Sg[p] = cx[0];
                    Sg[G::PMAX + p] = cy[0];
                    S2[1 * G::PMAX + p] = d1_64(cx, ex, c60[1]);
                    S2[2 * G::PMAX + p] = d1_64(cx, ex * bx_y, c60[2]);
                    S2[4 * G::PMAX + p] = d1_64(cy, ex * ey, c60[2]);
                }
            }
        } else {
            // ---------------- mixed precision: split staged doubles into float pairs
            for (int q = tid; q < npad; q += kThreads) {
                const F2 f2 = split_double(F[q]);
                fhi[q] = f2.hi;
                flo[q] = f2.lo;
            }
            __syncthreads();
            // numerators: compensated on the hi plane, plain FP32 on the lo
            // plane (its rounding is 2^-24 of a 2^-24 residue), as s + e
            auto N1 = [&](int off, int s) {
                FP2 h = n1_c(fhi + off, s);
                h.e = __fadd_rn(h.e, n1_32(flo + off, s));
                return h;
            };
            auto N2 = [&](int off, int s) {
                FP2 h = n2_c(fhi + off, s);
                h.e = __fadd_rn(h.e, n2_32(flo + off, s));
                return h;
            };
            auto NK = [&](int off, int s) {
                FP2 h = nko_c(fhi + off, s);
                h.e = __fadd_rn(h.e, nko_32(flo + off, s));
                return h;
            };
            // scales as float pairs: the scaling and the KO sum across the three
            // directions stay in FP32 pairs, one FP64 add per result
            const FC f60[3] = {split_const(c60[0]), split_const(c60[1]), split_const(c60[2])};
            const FC f180[3] = {split_const(c180[0]), split_const(c180[1]), split_const(c180[2])};
            const FC fko[3] = {split_const(ko[0]), split_const(ko[1]), split_const(ko[2])};
            auto KO3 = [&](int off) {
                return fp2_widen(add2(add2(mulfc(NK(off, 1), fko[0]), mulfc(NK(off, sy), fko[1])),
                                      mulfc(NK(off, sz), fko[2])));
            };
            if (q2 < 0) {
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int off = (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sg[p] = fp2_widen(mulfc(N1(off, 1), f60[0]));
                    Sg[G::PMAX + p] = fp2_widen(mulfc(N1(off, sy), f60[1]));
                    Sg[2 * G::PMAX + p] = fp2_widen(mulfc(N1(off, sz), f60[2]));
                    Sko[p] = KO3(off);
                }
            } else {
                double *S2 = S + (size_t)(DGB_NUM_GRAD + 6 * q2) * G::PMAX;
                const int bx_y = ey + 6;
                const int nA = ex * bx_y * ez, nB = ex * ey * 6;
                // (1a) x-numerators on the cross region, kept as s + e pairs
                for (int q = tid; q < nA + nB; q += kThreads) {
                    int ti, tj, tk;
                    if (q < nA) {
                        split3(q, dex, dbx, ti, tj, tk);
                        tk += 3;
                    } else {
                        const int q3 = q - nA;
                        int kk;  // 0..5
                        split3(q3, dex, dey, ti, tj, kk);
                        tj += 3;
                        tk = kk < 3 ? kk : ez + kk;
                    }
                    const FP2 h = N1((ti + 3) + sy * tj + sz * tk, 1);
                    const int b = ti + ex * (tj + bx_y * tk);
                    dxs[b] = h.s;
                    dxe[b] = h.e;
                }
                // (1b) y-numerators, z extended
                const int nC = ex * ey * pz;
                for (int q = tid; q < nC; q += kThreads) {
                    int ti, tj, tk;
                    split3(q, dex, dey, ti, tj, tk);
                    const FP2 h = N1((ti + 3) + sy * (tj + 3) + sz * tk, sy);
                    dys[q] = h.s;
                    dye[q] = h.e;
                }
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int off = (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sg[2 * G::PMAX + p] = fp2_widen(mulfc(N1(off, sz), f60[2]));
                    S2[0 * G::PMAX + p] = fp2_widen(mulfc(N2(off, 1), f180[0]));
                    S2[3 * G::PMAX + p] = fp2_widen(mulfc(N2(off, sy), f180[1]));
                    S2[5 * G::PMAX + p] = fp2_widen(mulfc(N2(off, sz), f180[2]));
                    Sko[p] = KO3(off);
                }
                __syncthreads();
                // (2) mixed: the pair boxes differentiated again (compensated on s,
                // plain on e), both scales applied in FP64
                const FC fxy = split_const(c60[0] * c60[1]), fxz = split_const(c60[0] * c60[2]),
                         fyz = split_const(c60[1] * c60[2]);
                for (int p = tid; p < P; p += kThreads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int bxi = ti + ex * ((tj + 3) + bx_y * (tk + 3));
                    const int byi = ti + ex * (tj + ey * (tk + 3));
                    Sg[p] = fp2_widen(mulfc(FP2{dxs[bxi], dxe[bxi]}, f60[0]));
                    Sg[G::PMAX + p] = fp2_widen(mulfc(FP2{dys[byi], dye[byi]}, f60[1]));
                    FP2 h = n1_c(dxs + bxi, ex);
                    h.e = __fadd_rn(h.e, n1_32(dxe + bxi, ex));
                    S2[1 * G::PMAX + p] = fp2_widen(mulfc(h, fxy));
                    h = n1_c(dxs + bxi, ex * bx_y);
                    h.e = __fadd_rn(h.e, n1_32(dxe + bxi, ex * bx_y));
                    S2[2 * G::PMAX + p] = fp2_widen(mulfc(h, fxz));
                    h = n1_c(dys + byi, ex * ey);
                    h.e = __fadd_rn(h.e, n1_32(dye + byi, ex * ey));
                    S2[4 * G::PMAX + p] = fp2_widen(mulfc(h, fyz));
                }
            }
        }
    }
    __syncthreads();

    // ------------------------------------------------------------ phase A
    for (int p = tid; p < P; p += kThreads) {
        int ti, tj, tk;
        split3(p, dex, dey, ti, tj, tk);
        const int i = w.o[0] + ti + 3, j = w.o[1] + tj + 3, k = w.o[2] + tk + 3;
        const uint64_t gi = blk.offset + (uint64_t)i + (uint64_t)nx * ((uint64_t)j + (uint64_t)ny * k);
        // coordinates and radius with the reference's roundings (rhs.cpp:210-219)
        const double x = __dadd_rn(blk.pmin[0], __dmul_rn((double)i, hx));
        const double y = __dadd_rn(blk.pmin[1], __dmul_rn((double)j, hy));
        const double z = __dadd_rn(blk.pmin[2], __dmul_rn((double)k, hz));
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
        if (bflag != 0 && ((blo[0] && i == 3) || (bhi[0] && i == nx - 4) || (blo[1] && j == 3) ||
                           (bhi[1] && j == ny - 4) || (blo[2] && k == 3) || (bhi[2] && k == nz - 4))) {
            // outgoing-radiation condition on a domain face (BSSN_GR/src/rhs.cpp:838-982):
            // rhs = -(1/r)(x f_x + y f_y + z f_z + falloff (f - asymptotic)),
            // replacing the algebra at this point, then + sigma * KO as elsewhere
            const double ninv_r = -__ddiv_rn(1.0, __dsqrt_rn(r2));
            const uint32_t gg = GATHER ? __ldg(args.gmap + gi) : 0u;
            const uint32_t go = GATHER ? __ldg(args.zmap + gi) : 0u;
            for (int v = 0; v < NV; v++) {
                const double f = GATHER ? __ldg(gather_src(args, v, gg)) : __ldg(args.u[v] + gi);
                const double *g = S + (size_t)(3 * v) * G::PMAX + p;
                double t = __dadd_rn(__dmul_rn(x, g[0]), __dmul_rn(y, g[G::PMAX]));
                t = __dadd_rn(t, __dmul_rn(z, g[2 * G::PMAX]));
                t = __dadd_rn(t, __dmul_rn(c_bc_falloff[v], __dsub_rn(f, c_bc_asym[v])));
                const double ko_sum = S[(size_t)(DGB_NUM_DERIV + v) * G::PMAX + p];
                const double out = __dadd_rn(__dmul_rn(ninv_r, t), __dmul_rn(args.prm.sigma, ko_sum));
                if (!GATHER)
                    args.rhs[v][gi] = out;
                else if (go != 0xFFFFFFFFu)
                    args.rhs[v][go] = out;
            }
            continue;
        }
        const double rr = __dsqrt_rn(r2);
        double eta = args.prm.eta_const;
        if (rr >= args.prm.eta_r0) {
            const double q = args.prm.eta_r0 / rr;
            eta *= (args.prm.eta_exp == 1.0) ? q : pow(q, args.prm.eta_exp);
        }
        if (GATHER) {
            AlgIOg io{&args, S, G::PMAX, p, __ldg(args.gmap + gi), __ldg(args.zmap + gi),
                      args.prm.sigma};
            dgb_bssn_algebra(io, aprm, eta);
            io.flush();
        } else {
            AlgIOw io{args.u, args.rhs, S, G::PMAX, p, gi, args.prm.sigma};
            dgb_bssn_algebra(io, aprm, eta);
        }
    }
}

}  // namespace
}  // namespace dgb
