// CCZ4 right-hand side on padded octant blocks (ccz4rhs,
// CCZ4_GR/src/rhs.cpp:12-298): one persistent, work-queued launch over all
// blocks of a plan, the structure of the BSSN kernel (rhs_item.cuh) with
// the CCZ4 solver's 4th-order stencil family (stencil42.cuh).
//
// Per work item (a tile of <= 8x8x8 interior points of one block):
//   the shift components at the tile points are staged once (the upwind
//   direction of every advective derivative);
//   phase D  for each of the 25 fields: stage tile + 3 in shared memory
//            (cp.async, double buffered) and write to the CTA's workspace
//            slice the first derivatives (deriv42), the upwind advective
//            derivatives (deriv42adv), for alpha, psi, beta0-2, gt0-5 the
//            second and mixed derivatives (mixed = d_y(d_x u), d_z(d_x u),
//            d_z(d_y u) as CCZ4_GR/scripts/ccz4rhs_derivs.h composes them),
//            and for every field but theta_z4 the KO sum kx + ky + kz;
//   phase A  one thread per tile point: the generated algebra
//            (ccz4_algebra.cuh), ccz4_bcs on flagged faces (every variable
//            but theta_z4) and rhs += sigma * KO (every variable but
//            theta_z4, CCZ4_GR/src/rhs.cpp:241-283).
// The first derivatives of At0-5 and B0-2 feed only the boundary condition
// and are formed on domain-boundary blocks only.
//
// Mixed precision (MIXED = true, interior blocks): every stencil runs in
// FP32 on the split doubles (fp32split.cuh), compensated on the hi part and
// plain on the lo part, is scaled by its float-pair scale and (KO) summed
// across directions as float pairs, and reaches FP64 with one add; the
// algebra, the boundary condition and all field I/O stay FP64.
// Domain-boundary blocks take the FP64 stencils.
#include <cuda_runtime.h>
#include <stdint.h>

#include "ccz4_algebra.cuh"
#include "dgb_internal.h"
#include "exact_mul.cuh"
#include "fp32split.cuh"
#include "stencil42.cuh"
#include "tile_index.cuh"

namespace dgb {
namespace {

constexpr int kC4Threads = 256;
#ifndef DGB_C4_MIN_CTAS
#define DGB_C4_MIN_CTAS 2
#endif
// CTAs per SM the register budget is sized for (255 registers at 1, 128 at 2)
constexpr int kC4MinBlocks = DGB_C4_MIN_CTAS;
constexpr int kC4Theta = 24;
// VAR -> second-derivative group (alpha, psi, beta0-2, gt0-5) or -1
__constant__ int8_t c_c4d2[NV4] = {0, 1, -1, -1, -1, -1, 2, 3, 4, -1, -1, -1,
                                   5, 6, 7, 8, 9, 10, -1, -1, -1, -1, -1, -1, -1};
// ccz4_bcs falloff / asymptotic per variable (CCZ4_GR/src/rhs.cpp:168-231)
__constant__ double c_c4fall[NV4] = {1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 0};
__constant__ double c_c4asym[NV4] = {1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     1, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0};

__device__ __forceinline__ void c4_cp_async8(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void c4_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void c4_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ---- 4th-order numerators on float lines (hi: compensated, lo: plain)
__device__ __forceinline__ FP2 neg2(FP2 x)
{
    x.s = -x.s;
    x.e = -x.e;
    return x;
}
// first derivative: 8 (u1 - u-1) - (u2 - u-2)
__device__ __forceinline__ FP2 n1_4c(const float *u, int s)
{
    return add2(mulc2(8.0f, two_sum(u[s], -u[-s])), neg2(two_sum(u[2 * s], -u[-2 * s])));
}
__device__ __forceinline__ float n1_4(const float *u, int s)
{
    return fmaf(8.0f, u[s] - u[-s], -(u[2 * s] - u[-2 * s]));
}
// second derivative: 16 s1 - s2, s_k = (u_k - u0) + (u_-k - u0)
__device__ __forceinline__ FP2 n2_4c(const float *u, int s)
{
    const float c = u[0];
    return add2(mulc2(16.0f, sym2(u, s, c)), neg2(sym2(u, 2 * s, c)));
}
__device__ __forceinline__ float n2_4(const float *u, int s)
{
    const float c = u[0];
    return fmaf(16.0f, (u[s] - c) + (u[-s] - c), -((u[2 * s] - c) + (u[-2 * s] - c)));
}
// upwind, beta > 0: -3 d_-1 + 18 d_1 - 6 d_2 + d_3 with d_k = u_k - u0
__device__ __forceinline__ FP2 nadvp_c(const float *u, int s)
{
    const float c = u[0];
    FP2 t = add2(mulc2(-3.0f, two_sum(u[-s], -c)), mulc2(18.0f, two_sum(u[s], -c)));
    t = add2(t, mulc2(-6.0f, two_sum(u[2 * s], -c)));
    return add2(t, two_sum(u[3 * s], -c));
}
__device__ __forceinline__ float nadvp(const float *u, int s)
{
    const float c = u[0];
    return fmaf(-3.0f, u[-s] - c, fmaf(18.0f, u[s] - c, fmaf(-6.0f, u[2 * s] - c, u[3 * s] - c)));
}
// upwind, beta <= 0: -d_-3 + 6 d_-2 - 18 d_-1 + 3 d_1
__device__ __forceinline__ FP2 nadvn_c(const float *u, int s)
{
    const float c = u[0];
    FP2 t = add2(neg2(two_sum(u[-3 * s], -c)), mulc2(6.0f, two_sum(u[-2 * s], -c)));
    t = add2(t, mulc2(-18.0f, two_sum(u[-s], -c)));
    return add2(t, mulc2(3.0f, two_sum(u[s], -c)));
}
__device__ __forceinline__ float nadvn(const float *u, int s)
{
    const float c = u[0];
    return fmaf(6.0f, u[-2 * s] - c, fmaf(-18.0f, u[-s] - c, fmaf(3.0f, u[s] - c, -(u[-3 * s] - c))));
}

template <int TX, int TY, int TZ>
struct C4Geo {
    static constexpr int PX = TX + 6, PY = TY + 6, PZ = TZ + 6;
    static constexpr int FBUF = PX * PY * PZ;
    static constexpr int DXB = TX * (TY + 4) * (TZ + 4);  // d_x on the +-2 cross region
    static constexpr int DYB = TX * TY * (TZ + 4);
    static constexpr int PMAX = TX * TY * TZ;
    // doubles: two staged fields, the d_x / d_y boxes, the shift at the tile
    // points; then per direction the tile points ordered by the sign of the shift
    static constexpr size_t bytes = (size_t)(2 * FBUF + DXB + DYB + 3 * PMAX) * 8 + 3 * PMAX * 2;
    // + hi/lo planes of the staged field and the s + e pair boxes (floats)
    static constexpr size_t bytes_mixed = bytes + (size_t)(2 * FBUF + 2 * DXB + 2 * DYB) * 4;
    // DivBy (tile_index.cuh) splits indices q < FBUF by extents < 32 exactly
    static_assert(FBUF < (1 << 13) && TX + 6 < 32 && TY + 6 < 32 && TZ + 6 < 32, "tile too large for DivBy");
};

struct C4AlgPrm {
    double l1, l2, l3, l4, lf0, lf1, k1, k2, p;
};

struct C4IO {
    const double *const *uu;
    double *const *rr;
    const double *S;
    int pmax, p;
    uint64_t gi;
    double sigma;
    bool face;            // on a flagged domain face: ccz4_bcs replaces the algebra
    double x, y, z, ninv_r;
    __device__ __forceinline__ double u(int v) const { return __ldg(uu[v] + gi); }
    __device__ __forceinline__ double d(int s) const { return S[(size_t)s * pmax + p]; }
    __device__ __forceinline__ void out(int v, double val) const
    {
        if (v == kC4Theta) {
            rr[v][gi] = val;
            return;
        }
        if (face) {
            // -(1/r)(x f_x + y f_y + z f_z + falloff (f - asymptotic))
            const double f = __ldg(uu[v] + gi);
            double t = __dadd_rn(__dmul_rn(x, d(3 * v)), __dmul_rn(y, d(3 * v + 1)));
            t = __dadd_rn(t, __dmul_rn(z, d(3 * v + 2)));
            t = __dadd_rn(t, __dmul_rn(c_c4fall[v], __dsub_rn(f, c_c4asym[v])));
            val = __dmul_rn(ninv_r, t);
        }
        rr[v][gi] = __dadd_rn(val, __dmul_rn(sigma, d(DGB_CCZ4_NUM_DERIV + v)));
    }
};

// Phase D of a work item: stage each field, write its derivatives and KO sum
// to the workspace.  BDY: the block touches a domain face.  Interior blocks
// are compiled with the closure tests constant-false, so the one-sided
// stencils (and the KO closures' divisions) are not issued under a false
// predicate on every point, and the upwind forms are split by the sorted
// point lists.
template <int TX, int TY, int TZ, bool MIXED, bool BDY>
__device__ __forceinline__ void c4_item(const C4Args &args, const WorkItem &w, const DevBlock &blk,
                                        double *S)
{
    using G = C4Geo<TX, TY, TZ>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *fb0 = reinterpret_cast<double *>(smem_raw);
    double *fb1 = fb0 + G::FBUF;
    double *dxb = fb1 + G::FBUF;
    double *dyb = dxb + G::DXB;
    double *bet = dyb + G::DYB;  // beta0..2 at the tile points
    // per direction d: tile points with beta_d > 0 first, then the others
    uint16_t *advl = reinterpret_cast<uint16_t *>(bet + 3 * G::PMAX);
    float *fhi = reinterpret_cast<float *>(advl + 3 * G::PMAX);  // MIXED only
    float *flo = fhi + G::FBUF;
    float *dxs = flo + G::FBUF;
    float *dxe = dxs + G::DXB;
    float *dys = dxe + G::DXB;
    float *dye = dys + G::DYB;
    const int tid = threadIdx.x;
    const int nx = blk.sz[0], ny = blk.sz[1], nz = blk.sz[2];
    const int ex = w.e[0], ey = w.e[1], ez = w.e[2];
    const int px = ex + 6, py = ey + 6, pz = ez + 6;
    const int npad = px * py * pz;
    const DivBy dpx(px), dpy(py);
    const int P = ex * ey * ez;
    const DivBy dex(ex), dey(ey);
    const int sy = px, sz = px * py;
    const uint64_t rbase = blk.offset + (uint64_t)w.o[0]
                         + (uint64_t)nx * ((uint64_t)w.o[1] + (uint64_t)ny * w.o[2]);
    const uint32_t bflag = BDY ? blk.bflag : 0u;
    const bool lo[3] = {(bflag & 1u) != 0, (bflag & 4u) != 0, (bflag & 16u) != 0};
    const bool hi[3] = {(bflag & 2u) != 0, (bflag & 8u) != 0, (bflag & 32u) != 0};
    const Ax4 ax[3] = {ax4(blk.h[0]), ax4(blk.h[1]), ax4(blk.h[2])};
    const int nn[3] = {nx, ny, nz};

    // The upwind direction of every advective derivative is the sign of the
    // shift at the point; with points ordered by that sign per direction, a
    // warp evaluates one upwind form instead of both (the order of the points
    // does not change any result: each writes its own slot).
    __shared__ int s_cnt[6];
    if (tid < 6) s_cnt[tid] = 0;
    __syncthreads();
    for (int p = tid; p < P; p += kC4Threads) {
        int ti, tj, tk;
        split3(p, dex, dey, ti, tj, tk);
        const uint64_t gi = blk.offset + (uint64_t)(w.o[0] + ti + 3)
                          + (uint64_t)nx * ((uint64_t)(w.o[1] + tj + 3) + (uint64_t)ny * (w.o[2] + tk + 3));
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double b = __ldg(args.u[6 + d] + gi);
            bet[d * G::PMAX + p] = b;
            const int q = b > 0.0 ? atomicAdd(&s_cnt[2 * d], 1) : P - 1 - atomicAdd(&s_cnt[2 * d + 1], 1);
            advl[d * G::PMAX + q] = (uint16_t)p;
        }
    }
    const int st3[3] = {1, sy, sz};
    auto tile_pos = [&](int p, int d, int *ti_, int *tj_, int *tk_) {
        int ti, tj, tk;
        split3(p, dex, dey, ti, tj, tk);
        *ti_ = ti; *tj_ = tj; *tk_ = tk;
        return (d == 0 ? w.o[0] + ti : d == 1 ? w.o[1] + tj : w.o[2] + tk) + 3;
    };

    // FP64 upwind derivatives over the tile points ordered by the sign of the
    // shift; interior blocks: the first s_cnt[2d] points take the forward
    // form, the rest the backward one, each in a loop of its own
    auto adv64_sorted = [&](const double *F, double *Sa) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (BDY) {
                for (int q = tid; q < P; q += kC4Threads) {
                    const int p = advl[d * G::PMAX + q];
                    int ti, tj, tk;
                    const int pos = tile_pos(p, d, &ti, &tj, &tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sa[d * G::PMAX + p] = adv42_at(c, st3[d], pos, nn[d], lo[d], hi[d],
                                                   bet[d * G::PMAX + p], ax[d]);
                }
            } else {
                const int npos = s_cnt[2 * d];
                for (int q = tid; q < npos; q += kC4Threads) {
                    const int p = advl[d * G::PMAX + q];
                    int ti, tj, tk;
                    tile_pos(p, d, &ti, &tj, &tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sa[d * G::PMAX + p] = adv42_pos(c, st3[d], ax[d].c12);
                }
                for (int q = npos + tid; q < P; q += kC4Threads) {
                    const int p = advl[d * G::PMAX + q];
                    int ti, tj, tk;
                    tile_pos(p, d, &ti, &tj, &tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sa[d * G::PMAX + p] = adv42_neg(c, st3[d], ax[d].c12);
                }
            }
        }
    };

    auto issue_load = [&](int v, double *dst) {
        const double *src = args.u[v] + rbase;
        for (int q = tid; q < npad; q += kC4Threads) {
            int i, j, k;
            split3(q, dpx, dpy, i, j, k);
            c4_cp_async8(dst + q, src + i + (uint64_t)nx * (j + (uint64_t)ny * k));
        }
        c4_commit();
    };

    issue_load(0, fb0);
    for (int v = 0; v < NV4; v++) {
        double *F = (v & 1) ? fb1 : fb0;
        if (v + 1 < NV4) {
            issue_load(v + 1, (v & 1) ? fb0 : fb1);
            c4_wait<1>();
        } else {
            c4_wait<0>();
        }
        __syncthreads();
        const int q2 = c_c4d2[v];
        double *Sg = S + (size_t)(3 * v) * G::PMAX;
        double *Sa = S + (size_t)(DGB_CCZ4_ADV0 + 3 * v) * G::PMAX;
        double *Sko = S + (size_t)(DGB_CCZ4_NUM_DERIV + v) * G::PMAX;
        // At0-5, B0-2: first derivatives only for the boundary condition
        const bool want_grad = bflag != 0 || !((v >= 9 && v <= 11) || (v >= 18 && v <= 23));
        if (MIXED && bflag == 0) {
            for (int q = tid; q < npad; q += kC4Threads) {
                const F2 f2 = split_double(F[q]);
                fhi[q] = f2.hi;
                flo[q] = f2.lo;
            }
            __syncthreads();
            auto N1 = [&](const float *h, const float *l, int s) {
                FP2 r = n1_4c(h, s);
                r.e = __fadd_rn(r.e, n1_4(l, s));
                return r;
            };
            // scales as float pairs: scaling and the KO sum stay in FP32 pairs
            const FC f12[3] = {split_const(ax[0].c12), split_const(ax[1].c12), split_const(ax[2].c12)};
            const FC f12sq[3] = {split_const(ax[0].c12sq), split_const(ax[1].c12sq),
                                 split_const(ax[2].c12sq)};
            const FC fpre[3] = {split_const(ax[0].pre), split_const(ax[1].pre), split_const(ax[2].pre)};
            auto to64 = [](FP2 r, FC f) { return fp2_widen(mulfc(r, f)); };
            // one point: KO (theta excluded) in FP32, scaled and summed in FP64
            auto adv_ko = [&](int p, int off, const int *pos) {
                const int st[3] = {1, sy, sz};
                if (v == kC4Theta) return;
                FP2 ko{0.0f, 0.0f};
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    // the first / last interior point takes its neighbour's stencil
                    const int sh = pos[d] == 3 ? st[d] : (pos[d] == nn[d] - 4 ? -st[d] : 0);
                    FP2 k = nko_c(fhi + off + sh, st[d]);
                    k.e = __fadd_rn(k.e, nko_32(flo + off + sh, st[d]));
                    const FP2 kd = mulfc(k, fpre[d]);
                    ko = d == 0 ? kd : add2(ko, kd);
                }
                Sko[p] = fp2_widen(ko);
            };
            // upwind derivatives over the tile points ordered by the sign of the
            // shift: forward form on the first s_cnt[2d], backward on the rest
            auto adv_sorted = [&]() {
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const int npos = s_cnt[2 * d];
                    for (int q = tid; q < npos; q += kC4Threads) {
                        const int p = advl[d * G::PMAX + q];
                        int ti, tj, tk;
                        tile_pos(p, d, &ti, &tj, &tk);
                        const int off = (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                        FP2 a = nadvp_c(fhi + off, st3[d]);
                        a.e = __fadd_rn(a.e, nadvp(flo + off, st3[d]));
                        Sa[d * G::PMAX + p] = to64(a, f12[d]);
                    }
                    for (int q = npos + tid; q < P; q += kC4Threads) {
                        const int p = advl[d * G::PMAX + q];
                        int ti, tj, tk;
                        tile_pos(p, d, &ti, &tj, &tk);
                        const int off = (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                        FP2 a = nadvn_c(fhi + off, st3[d]);
                        a.e = __fadd_rn(a.e, nadvn(flo + off, st3[d]));
                        Sa[d * G::PMAX + p] = to64(a, f12[d]);
                    }
                }
            };
            if (q2 < 0) {
                for (int p = tid; p < P; p += kC4Threads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int pos[3] = {w.o[0] + ti + 3, w.o[1] + tj + 3, w.o[2] + tk + 3};
                    const int off = (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    if (want_grad) {
                        Sg[p] = to64(N1(fhi + off, flo + off, 1), f12[0]);
                        Sg[G::PMAX + p] = to64(N1(fhi + off, flo + off, sy), f12[1]);
                        Sg[2 * G::PMAX + p] = to64(N1(fhi + off, flo + off, sz), f12[2]);
                    }
                    adv_ko(p, off, pos);
                }
                adv_sorted();
            } else {
                double *S2 = S + (size_t)(DGB_CCZ4_D20 + 6 * q2) * G::PMAX;
                const int by = ey + 4;
                const DivBy dby(by);
                const int nA = ex * by * ez, nB = ex * ey * 4;
                for (int q = tid; q < nA + nB; q += kC4Threads) {
                    int ti, tj, tk;
                    if (q < nA) {
                        split3(q, dex, dby, ti, tj, tk);
                        tk += 2;
                    } else {
                        const int q3 = q - nA;
                        int kk;
                        split3(q3, dex, dey, ti, tj, kk);
                        tj += 2;
                        tk = kk < 2 ? kk : ez + kk;
                    }
                    const int off = (ti + 3) + sy * (tj + 1) + sz * (tk + 1);
                    const FP2 h = N1(fhi + off, flo + off, 1);
                    const int b = ti + ex * (tj + by * tk);
                    dxs[b] = h.s;
                    dxe[b] = h.e;
                }
                const int nC = ex * ey * (ez + 4);
                for (int q = tid; q < nC; q += kC4Threads) {
                    int ti, tj, tk;
                    split3(q, dex, dey, ti, tj, tk);
                    const int off = (ti + 3) + sy * (tj + 3) + sz * (tk + 1);
                    const FP2 h = N1(fhi + off, flo + off, sy);
                    dys[q] = h.s;
                    dye[q] = h.e;
                }
                for (int p = tid; p < P; p += kC4Threads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int pos[3] = {w.o[0] + ti + 3, w.o[1] + tj + 3, w.o[2] + tk + 3};
                    const int off = (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    Sg[2 * G::PMAX + p] = to64(N1(fhi + off, flo + off, sz), f12[2]);
                    const int st[3] = {1, sy, sz};
                    const int slot[3] = {0, 3, 5};
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        FP2 h = n2_4c(fhi + off, st[d]);
                        h.e = __fadd_rn(h.e, n2_4(flo + off, st[d]));
                        S2[slot[d] * G::PMAX + p] = to64(h, f12sq[d]);
                    }
                    adv_ko(p, off, pos);
                }
                adv_sorted();
                __syncthreads();
                const FC fxy = split_const(ax[0].c12 * ax[1].c12), fxz = split_const(ax[0].c12 * ax[2].c12),
                         fyz = split_const(ax[1].c12 * ax[2].c12);
                for (int p = tid; p < P; p += kC4Threads) {
                    int ti, tj, tk;
                    split3(p, dex, dey, ti, tj, tk);
                    const int bxi = ti + ex * ((tj + 2) + by * (tk + 2));
                    const int byi = ti + ex * (tj + ey * (tk + 2));
                    Sg[p] = to64(FP2{dxs[bxi], dxe[bxi]}, f12[0]);
                    Sg[G::PMAX + p] = to64(FP2{dys[byi], dye[byi]}, f12[1]);
                    S2[1 * G::PMAX + p] = to64(N1(dxs + bxi, dxe + bxi, ex), fxy);
                    S2[2 * G::PMAX + p] = to64(N1(dxs + bxi, dxe + bxi, ex * by), fxz);
                    S2[4 * G::PMAX + p] = to64(N1(dys + byi, dye + byi, ex * ey), fyz);
                }
            }
        } else if (q2 < 0) {
            for (int p = tid; p < P; p += kC4Threads) {
                int ti, tj, tk;
                split3(p, dex, dey, ti, tj, tk);
                const int pos[3] = {w.o[0] + ti + 3, w.o[1] + tj + 3, w.o[2] + tk + 3};
                const int st[3] = {1, sy, sz};
                const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                double ko = 0.0;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    if (want_grad) Sg[d * G::PMAX + p] = d1_42_at(c, st[d], pos[d], nn[d], lo[d], hi[d], ax[d]);
                    if (v != kC4Theta) {
                        const double k = ko42c_at(c, st[d], pos[d], nn[d], lo[d], hi[d], ax[d]);
                        ko = d == 0 ? k : __dadd_rn(ko, k);
                    }
                }
                if (v != kC4Theta) Sko[p] = ko;
            }
            adv64_sorted(F, Sa);
        } else {
            double *S2 = S + (size_t)(DGB_CCZ4_D20 + 6 * q2) * G::PMAX;
            // (1a) d_x on x in tile and (y in tile +- 2, z in tile) or (y in tile, z halo of 2)
            const int by = ey + 4;
            const DivBy dby(by);
            const int nA = ex * by * ez, nB = ex * ey * 4;
            for (int q = tid; q < nA + nB; q += kC4Threads) {
                int ti, tj, tk;  // box coordinates: tj in [0, ey+4), tk in [0, ez+4)
                if (q < nA) {
                    split3(q, dex, dby, ti, tj, tk);
                    tk += 2;
                } else {
                    const int q3 = q - nA;
                    int kk;  // 0..3
                    split3(q3, dex, dey, ti, tj, kk);
                    tj += 2;
                    tk = kk < 2 ? kk : ez + kk;
                }
                const double *c = F + (ti + 3) + sy * (tj + 1) + sz * (tk + 1);
                dxb[ti + ex * (tj + by * tk)] = d1_42_at(c, 1, w.o[0] + ti + 3, nx, lo[0], hi[0], ax[0]);
            }
            // (1b) d_y on x, y in tile, z in tile +- 2
            const int nC = ex * ey * (ez + 4);
            for (int q = tid; q < nC; q += kC4Threads) {
                int ti, tj, tk;
                split3(q, dex, dey, ti, tj, tk);
                const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 1);
                dyb[q] = d1_42_at(c, sy, w.o[1] + tj + 3, ny, lo[1], hi[1], ax[1]);
            }
            // (1c) pointwise: d_z, xx, yy, zz, advective, KO
            for (int p = tid; p < P; p += kC4Threads) {
                int ti, tj, tk;
                split3(p, dex, dey, ti, tj, tk);
                const int pos[3] = {w.o[0] + ti + 3, w.o[1] + tj + 3, w.o[2] + tk + 3};
                const int st[3] = {1, sy, sz};
                const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                Sg[2 * G::PMAX + p] = d1_42_at(c, sz, pos[2], nz, lo[2], hi[2], ax[2]);
                S2[0 * G::PMAX + p] = d2_42_at(c, 1, pos[0], nx, lo[0], hi[0], ax[0]);
                S2[3 * G::PMAX + p] = d2_42_at(c, sy, pos[1], ny, lo[1], hi[1], ax[1]);
                S2[5 * G::PMAX + p] = d2_42_at(c, sz, pos[2], nz, lo[2], hi[2], ax[2]);
                double ko = 0.0;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const double k = ko42c_at(c, st[d], pos[d], nn[d], lo[d], hi[d], ax[d]);
                    ko = d == 0 ? k : __dadd_rn(ko, k);
                }
                Sko[p] = ko;
            }
            adv64_sorted(F, Sa);
            __syncthreads();
            // (2) mixed from the boxes; d_x, d_y at the tile points
            for (int p = tid; p < P; p += kC4Threads) {
                int ti, tj, tk;
                split3(p, dex, dey, ti, tj, tk);
                const int pj = w.o[1] + tj + 3, pk = w.o[2] + tk + 3;
                const double *cx = dxb + ti + ex * ((tj + 2) + by * (tk + 2));
                const double *cy = dyb + ti + ex * (tj + ey * (tk + 2));
                Sg[p] = cx[0];
                Sg[G::PMAX + p] = cy[0];
                S2[1 * G::PMAX + p] = d1_42_at(cx, ex, pj, ny, lo[1], hi[1], ax[1]);
                S2[2 * G::PMAX + p] = d1_42_at(cx, ex * by, pk, nz, lo[2], hi[2], ax[2]);
                S2[4 * G::PMAX + p] = d1_42_at(cy, ex * ey, pk, nz, lo[2], hi[2], ax[2]);
            }
        }
        __syncthreads();  // F and the boxes are reused
    }
}

// Phase A of a work item (one thread per tile point), shared by interior and
// boundary blocks: the algebra, the boundary condition on flagged faces, KO.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void c4_points(const C4Args &args, const WorkItem &w, const DevBlock &blk,
                                          const double *S)
{
    using G = C4Geo<TX, TY, TZ>;
    const int tid = threadIdx.x;
    const int nx = blk.sz[0], ny = blk.sz[1], nz = blk.sz[2];
    const int ex = w.e[0], ey = w.e[1], ez = w.e[2];
    const int P = ex * ey * ez;
    const DivBy dex(ex), dey(ey);
    const uint32_t bflag = blk.bflag;
    const bool lo[3] = {(bflag & 1u) != 0, (bflag & 4u) != 0, (bflag & 16u) != 0};
    const bool hi[3] = {(bflag & 2u) != 0, (bflag & 8u) != 0, (bflag & 32u) != 0};
    const C4AlgPrm aprm{args.prm.l1, args.prm.l2, args.prm.l3, args.prm.l4, args.prm.lf0,
                        args.prm.lf1, args.prm.k1, args.prm.k2, args.prm.p};
    for (int p = tid; p < P; p += kC4Threads) {
        int ti, tj, tk;
        split3(p, dex, dey, ti, tj, tk);
        const int i = w.o[0] + ti + 3, j = w.o[1] + tj + 3, k = w.o[2] + tk + 3;
        const uint64_t gi = blk.offset + (uint64_t)i + (uint64_t)nx * ((uint64_t)j + (uint64_t)ny * k);
        // coordinates and radius with the reference's roundings (rhs.cpp:147-160)
        const double x = __dadd_rn(blk.pmin[0], __dmul_rn((double)i, blk.h[0]));
        const double y = __dadd_rn(blk.pmin[1], __dmul_rn((double)j, blk.h[1]));
        const double z = __dadd_rn(blk.pmin[2], __dmul_rn((double)k, blk.h[2]));
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
        const double rr = __dsqrt_rn(r2);
        double eta = args.prm.eta_const;
        if (rr >= args.prm.eta_r0) {
            const double q = args.prm.eta_r0 / rr;
            eta *= (args.prm.eta_exp == 1.0) ? q : pow(q, args.prm.eta_exp);
        }
        const bool face = bflag != 0 && ((lo[0] && i == 3) || (hi[0] && i == nx - 4) ||
                                         (lo[1] && j == 3) || (hi[1] && j == ny - 4) ||
                                         (lo[2] && k == 3) || (hi[2] && k == nz - 4));
        const double ninv_r = face ? -__ddiv_rn(1.0, rr) : 0.0;
        C4IO io{args.u, args.rhs, S, G::PMAX, p, gi, args.prm.sigma, face, x, y, z, ninv_r};
        dgb_ccz4_algebra(io, aprm, eta);
    }
}

template <int TX, int TY, int TZ, bool MIXED>
__global__ void __launch_bounds__(kC4Threads, kC4MinBlocks) c4_kernel(const C4Args args)
{
    using G = C4Geo<TX, TY, TZ>;
    __shared__ int s_item;
    double *S = args.scratch + (size_t)blockIdx.x * DGB_CCZ4_NUM_SLOTS * G::PMAX;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = (int)atomicAdd(args.queue, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= (int)args.nitems) break;
        const WorkItem w = args.items[it];
        const DevBlock blk = args.blocks[w.blk];
        if (blk.bflag == 0)
            c4_item<TX, TY, TZ, MIXED, false>(args, w, blk, S);
        else
            c4_item<TX, TY, TZ, MIXED, true>(args, w, blk, S);
        c4_points<TX, TY, TZ>(args, w, blk, S);
    }
}

}  // namespace

size_t c4_smem_bytes(int precision)
{
    return precision == DGB_PREC_MIXED ? C4Geo<8, 8, 8>::bytes_mixed : C4Geo<8, 8, 8>::bytes;
}
size_t c4_scratch_per_cta() { return (size_t)DGB_CCZ4_NUM_SLOTS * C4Geo<8, 8, 8>::PMAX; }

cudaError_t c4_configure(int precision)
{
    if (precision == DGB_PREC_MIXED)
        return cudaFuncSetAttribute(c4_kernel<8, 8, 8, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)C4Geo<8, 8, 8>::bytes_mixed);
    return cudaFuncSetAttribute(c4_kernel<8, 8, 8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)C4Geo<8, 8, 8>::bytes);
}

int c4_max_ctas_per_sm(int precision)
{
    int n = 0;
    if (c4_configure(precision) != cudaSuccess) return 0;
    cudaError_t e = precision == DGB_PREC_MIXED
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, c4_kernel<8, 8, 8, true>, kC4Threads,
                                                        C4Geo<8, 8, 8>::bytes_mixed)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, c4_kernel<8, 8, 8, false>, kC4Threads,
                                                        C4Geo<8, 8, 8>::bytes);
    return e == cudaSuccess ? n : 0;
}

cudaError_t c4_launch(int precision, const C4Args &args, int grid, cudaStream_t stream)
{
    if (precision == DGB_PREC_MIXED)
        c4_kernel<8, 8, 8, true><<<grid, kC4Threads, C4Geo<8, 8, 8>::bytes_mixed, stream>>>(args);
    else
        c4_kernel<8, 8, 8, false><<<grid, kC4Threads, C4Geo<8, 8, 8>::bytes, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace dgb
