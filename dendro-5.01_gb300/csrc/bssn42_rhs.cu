// BSSN right-hand side with the BSSN_GR solver's own 4th-order stencil
// binding (BSSN_GR/include/rhs.h:23-37): deriv42 first and second
// derivatives, upwinded deriv42adv advective derivatives and ko_deriv42
// dissipation (BSSN_GR/src/derivs.cpp:11-1410), around the same generated
// system as the 6th-order kernel.  One persistent, work-queued launch over
// all blocks of a plan (8^3 tiles), the structure of rhs_item.cuh:
//
//   the shift components at the tile points are staged once, with the
//   tile's points listed by the sign of each component (a warp then
//   evaluates one upwind form);
//   phase D  for each of the 24 fields: stage tile + 3 in shared memory
//            (cp.async, double buffered) and write to the CTA's workspace
//            slice the first derivatives (of the fields the algebra or the
//            boundary condition reads), for alpha, chi, beta0-2, gt0-5 the
//            second and mixed derivatives (d_y(d_x u), d_z(d_x u), d_z(d_y u)
//            as BSSN_GR/scripts/bssnrhs_derivs.h composes them), the KO sum
//            kx + ky + kz, and the advection sum beta^j ad_j u of the three
//            upwinded derivatives, ((b0 a0 + b1 a1) + b2 a2);
//   phase A  one thread per tile point: the generated algebra
//            (bssn_algebra42.cuh reads the advection sums in place of
//            beta^j d_j u), bssn_bcs on flagged faces, rhs += sigma * KO.
// Every stencil keeps the reference's rounding sequence (stencil42.cuh,
// rhs_item.cuh's ko_at).  FP64 only.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bssn_algebra42.cuh"
#include "dgb_internal.h"
#include "rhs_item.cuh"
#include "stencil42.cuh"

namespace dgb {
namespace {

constexpr int kB4Threads = 256;
#ifndef DGB_B4_MIN_CTAS
#define DGB_B4_MIN_CTAS 2
#endif
constexpr int kB4MinBlocks = DGB_B4_MIN_CTAS;

template <int TX, int TY, int TZ>
struct B4Geo {
    static constexpr int PX = TX + 6, PY = TY + 6, PZ = TZ + 6;
    static constexpr int FBUF = PX * PY * PZ;
    static constexpr int DXB = TX * (TY + 4) * (TZ + 4);  // d_x on the +-2 cross region
    static constexpr int DYB = TX * TY * (TZ + 4);
    static constexpr int PMAX = TX * TY * TZ;
    // doubles: two staged fields, the d_x / d_y boxes, the shift at the tile
    // points, the three upwinded derivatives of the current field; then per
    // direction the tile points ordered by the sign of the shift (uint16)
    static constexpr size_t bytes = (size_t)(2 * FBUF + DXB + DYB + 6 * PMAX) * 8 + 3 * PMAX * 2;
    // DivBy (tile_index.cuh) splits indices q < FBUF by extents < 32 exactly
    static_assert(FBUF < (1 << 13) && TX + 6 < 32 && TY + 6 < 32 && TZ + 6 < 32, "tile too large for DivBy");
};

template <int TX, int TY, int TZ, bool BDY>
__device__ __forceinline__ void b4_item(const RhsArgs &args, const WorkItem &w, const DevBlock &blk,
                                        double *S)
{
    using G = B4Geo<TX, TY, TZ>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *fb0 = reinterpret_cast<double *>(smem_raw);
    double *fb1 = fb0 + G::FBUF;
    double *dxb = fb1 + G::FBUF;
    double *dyb = dxb + G::DXB;
    double *bet = dyb + G::DYB;            // beta0..2 at the tile points
    double *agr = bet + 3 * G::PMAX;       // upwinded d_0, d_1, d_2 of the field
    uint16_t *advl = reinterpret_cast<uint16_t *>(agr + 3 * G::PMAX);
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
    AxisScale ks[3];  // the KO closures' scales (boundary blocks)
    if (BDY) {
        ks[0] = axis_scale(blk.h[0]);
        ks[1] = axis_scale(blk.h[1]);
        ks[2] = axis_scale(blk.h[2]);
    }
    const double kpre[3] = {-1.0 / 64.0 / blk.h[0], -1.0 / 64.0 / blk.h[1], -1.0 / 64.0 / blk.h[2]};
    const int nn[3] = {nx, ny, nz};
    const int st3[3] = {1, sy, sz};

    __shared__ int s_cnt[6];
    if (tid < 6) s_cnt[tid] = 0;
    __syncthreads();
    for (int p = tid; p < P; p += kB4Threads) {
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
    auto tile_pos = [&](int p, int d, int *ti_, int *tj_, int *tk_) {
        int ti, tj, tk;
        split3(p, dex, dey, ti, tj, tk);
        *ti_ = ti; *tj_ = tj; *tk_ = tk;
        return (d == 0 ? w.o[0] + ti : d == 1 ? w.o[1] + tj : w.o[2] + tk) + 3;
    };
    // KO sum at one tile point: ko_deriv42 (BSSN_GR/src/derivs.cpp:914-1410)
    auto ko_sum = [&](const double *c, int ti, int tj, int tk) {
        if (BDY) {
            return ko_at(c, 1, w.o[0] + ti + 3, nx, lo[0], hi[0], ks[0])
                 + ko_at(c, sy, w.o[1] + tj + 3, ny, lo[1], hi[1], ks[1])
                 + ko_at(c, sz, w.o[2] + tk + 3, nz, lo[2], hi[2], ks[2]);
        }
        return ko_64(c, 1, kpre[0]) + ko_64(c, sy, kpre[1]) + ko_64(c, sz, kpre[2]);
    };
    // upwinded derivatives over the tile points ordered by the sign of the
    // shift, then the advection sum per point
    auto advection = [&](const double *F, double *Sa) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (BDY) {
                for (int q = tid; q < P; q += kB4Threads) {
                    const int p = advl[d * G::PMAX + q];
                    int ti, tj, tk;
                    const int pos = tile_pos(p, d, &ti, &tj, &tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    agr[d * G::PMAX + p] = adv42_at(c, st3[d], pos, nn[d], lo[d], hi[d],
                                                    bet[d * G::PMAX + p], ax[d], false);
                }
            } else {
                const int npos = s_cnt[2 * d];
                for (int q = tid; q < npos; q += kB4Threads) {
                    const int p = advl[d * G::PMAX + q];
                    int ti, tj, tk;
                    tile_pos(p, d, &ti, &tj, &tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    agr[d * G::PMAX + p] = adv42_pos(c, st3[d], ax[d].c12);
                }
                for (int q = npos + tid; q < P; q += kB4Threads) {
                    const int p = advl[d * G::PMAX + q];
                    int ti, tj, tk;
                    tile_pos(p, d, &ti, &tj, &tk);
                    const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                    agr[d * G::PMAX + p] = adv42_neg(c, st3[d], ax[d].c12);
                }
            }
        }
        __syncthreads();
        for (int p = tid; p < P; p += kB4Threads) {
            double t = __dmul_rn(bet[p], agr[p]);
            t = __dadd_rn(t, __dmul_rn(bet[G::PMAX + p], agr[G::PMAX + p]));
            Sa[p] = __dadd_rn(t, __dmul_rn(bet[2 * G::PMAX + p], agr[2 * G::PMAX + p]));
        }
    };

    auto issue_load = [&](int v, double *dst) {
        const double *src = args.u[v] + rbase;
        for (int q = tid; q < npad; q += kB4Threads) {
            int i, j, k;
            split3(q, dpx, dpy, i, j, k);
            cp_async8(dst + q, src + i + (uint64_t)nx * (j + (uint64_t)ny * k));
        }
        cp_async_commit();
    };

    issue_load(0, fb0);
    for (int v = 0; v < NV; v++) {
        double *F = (v & 1) ? fb1 : fb0;
        if (v + 1 < NV) {
            issue_load(v + 1, (v & 1) ? fb0 : fb1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const int q2 = c_d2index[v];
        double *Sg = S + (size_t)(3 * v) * G::PMAX;
        double *Sko = S + (size_t)(DGB_NUM_DERIV + v) * G::PMAX;
        double *Sa = S + (size_t)(DGB_B42_ADV0 + v) * G::PMAX;
        // B0-2, At0-5: the algebra reads only their advection sums; their first
        // derivatives feed the boundary condition alone
        const bool want_grad = bflag != 0 || !((v >= 9 && v <= 11) || (v >= 18 && v <= 23));
        if (q2 < 0) {
            for (int p = tid; p < P; p += kB4Threads) {
                int ti, tj, tk;
                split3(p, dex, dey, ti, tj, tk);
                const int pos[3] = {w.o[0] + ti + 3, w.o[1] + tj + 3, w.o[2] + tk + 3};
                const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                if (want_grad) {
#pragma unroll
                    for (int d = 0; d < 3; d++)
                        Sg[d * G::PMAX + p] = d1_42_at(c, st3[d], pos[d], nn[d], lo[d], hi[d], ax[d]);
                }
                Sko[p] = ko_sum(c, ti, tj, tk);
            }
            advection(F, Sa);
        } else {
            double *S2 = S + (size_t)(DGB_NUM_GRAD + 6 * q2) * G::PMAX;
            // (1a) d_x on x in tile and (y in tile +- 2, z in tile) or (y in tile, z halo of 2)
            const int by = ey + 4;
            const DivBy dby(by);
            const int nA = ex * by * ez, nB = ex * ey * 4;
            for (int q = tid; q < nA + nB; q += kB4Threads) {
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
            for (int q = tid; q < nC; q += kB4Threads) {
                int ti, tj, tk;
                split3(q, dex, dey, ti, tj, tk);
                const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 1);
                dyb[q] = d1_42_at(c, sy, w.o[1] + tj + 3, ny, lo[1], hi[1], ax[1]);
            }
            // (1c) pointwise: d_z, xx, yy, zz, KO
            for (int p = tid; p < P; p += kB4Threads) {
                int ti, tj, tk;
                split3(p, dex, dey, ti, tj, tk);
                const int pos[3] = {w.o[0] + ti + 3, w.o[1] + tj + 3, w.o[2] + tk + 3};
                const double *c = F + (ti + 3) + sy * (tj + 3) + sz * (tk + 3);
                Sg[2 * G::PMAX + p] = d1_42_at(c, sz, pos[2], nz, lo[2], hi[2], ax[2]);
                S2[0 * G::PMAX + p] = d2_42_at(c, 1, pos[0], nx, lo[0], hi[0], ax[0]);
                S2[3 * G::PMAX + p] = d2_42_at(c, sy, pos[1], ny, lo[1], hi[1], ax[1]);
                S2[5 * G::PMAX + p] = d2_42_at(c, sz, pos[2], nz, lo[2], hi[2], ax[2]);
                Sko[p] = ko_sum(c, ti, tj, tk);
            }
            advection(F, Sa);  // ends with a barrier: the boxes are complete
            // (2) mixed from the boxes; d_x, d_y at the tile points
            for (int p = tid; p < P; p += kB4Threads) {
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
        __syncthreads();  // F, the boxes and the upwinded derivatives are reused
    }
}

struct B4IO {
    const double *const *uu;
    double *const *rr;
    const double *S;
    int pmax, p;
    uint64_t gi;
    double sigma;
    __device__ __forceinline__ double u(int v) const { return __ldg(uu[v] + gi); }
    __device__ __forceinline__ double d(int s) const { return S[(size_t)s * pmax + p]; }
    __device__ __forceinline__ void out(int v, double x) const
    {
        rr[v][gi] = __dadd_rn(x, __dmul_rn(sigma, S[(size_t)(DGB_NUM_DERIV + v) * pmax + p]));
    }
};

// Phase A (one thread per tile point): the algebra, or bssn_bcs on a flagged
// face (BSSN_GR/src/rhs.cpp:838-982), then + sigma * KO.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void b4_points(const RhsArgs &args, const WorkItem &w, const DevBlock &blk,
                                          const double *S)
{
    using G = B4Geo<TX, TY, TZ>;
    const int tid = threadIdx.x;
    const int nx = blk.sz[0], ny = blk.sz[1], nz = blk.sz[2];
    const int ex = w.e[0], ey = w.e[1], ez = w.e[2];
    const int P = ex * ey * ez;
    const DivBy dex(ex), dey(ey);
    const uint32_t bflag = blk.bflag;
    const bool lo[3] = {(bflag & 1u) != 0, (bflag & 4u) != 0, (bflag & 16u) != 0};
    const bool hi[3] = {(bflag & 2u) != 0, (bflag & 8u) != 0, (bflag & 32u) != 0};
    const AlgPrm aprm{args.prm.l1, args.prm.l2, args.prm.l3, args.prm.l4, args.prm.lf0, args.prm.lf1};
    for (int p = tid; p < P; p += kB4Threads) {
        int ti, tj, tk;
        split3(p, dex, dey, ti, tj, tk);
        const int i = w.o[0] + ti + 3, j = w.o[1] + tj + 3, k = w.o[2] + tk + 3;
        const uint64_t gi = blk.offset + (uint64_t)i + (uint64_t)nx * ((uint64_t)j + (uint64_t)ny * k);
        const double x = __dadd_rn(blk.pmin[0], __dmul_rn((double)i, blk.h[0]));
        const double y = __dadd_rn(blk.pmin[1], __dmul_rn((double)j, blk.h[1]));
        const double z = __dadd_rn(blk.pmin[2], __dmul_rn((double)k, blk.h[2]));
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
        if (bflag != 0 && ((lo[0] && i == 3) || (hi[0] && i == nx - 4) || (lo[1] && j == 3) ||
                           (hi[1] && j == ny - 4) || (lo[2] && k == 3) || (hi[2] && k == nz - 4))) {
            const double ninv_r = -__ddiv_rn(1.0, __dsqrt_rn(r2));
            for (int v = 0; v < NV; v++) {
                const double f = __ldg(args.u[v] + gi);
                const double *g = S + (size_t)(3 * v) * G::PMAX + p;
                double t = __dadd_rn(__dmul_rn(x, g[0]), __dmul_rn(y, g[G::PMAX]));
                t = __dadd_rn(t, __dmul_rn(z, g[2 * G::PMAX]));
                t = __dadd_rn(t, __dmul_rn(c_bc_falloff[v], __dsub_rn(f, c_bc_asym[v])));
                const double ko = S[(size_t)(DGB_NUM_DERIV + v) * G::PMAX + p];
                args.rhs[v][gi] = __dadd_rn(__dmul_rn(ninv_r, t), __dmul_rn(args.prm.sigma, ko));
            }
            continue;
        }
        const double rr = __dsqrt_rn(r2);
        double eta = args.prm.eta_const;
        if (rr >= args.prm.eta_r0) {
            const double q = args.prm.eta_r0 / rr;
            eta *= (args.prm.eta_exp == 1.0) ? q : pow(q, args.prm.eta_exp);
        }
        B4IO io{args.u, args.rhs, S, G::PMAX, p, gi, args.prm.sigma};
        dgb_bssn_algebra_upwind(io, aprm, eta);
    }
}

template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(kB4Threads, kB4MinBlocks) b4_kernel(const RhsArgs args)
{
    using G = B4Geo<TX, TY, TZ>;
    __shared__ int s_item;
    double *S = args.scratch + (size_t)blockIdx.x * DGB_B42_NUM_SLOTS * G::PMAX;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = (int)atomicAdd(args.queue, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= (int)args.nitems) break;
        const WorkItem w = args.items[it];
        const DevBlock blk = args.blocks[w.blk];
        if (blk.bflag == 0)
            b4_item<TX, TY, TZ, false>(args, w, blk, S);
        else
            b4_item<TX, TY, TZ, true>(args, w, blk, S);
        b4_points<TX, TY, TZ>(args, w, blk, S);
    }
}

}  // namespace

size_t b4_smem_bytes() { return B4Geo<8, 8, 8>::bytes; }
size_t b4_scratch_per_cta() { return (size_t)DGB_B42_NUM_SLOTS * B4Geo<8, 8, 8>::PMAX; }

cudaError_t b4_configure()
{
    return cudaFuncSetAttribute(b4_kernel<8, 8, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)B4Geo<8, 8, 8>::bytes);
}

int b4_max_ctas_per_sm()
{
    int n = 0;
    if (b4_configure() != cudaSuccess) return 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, b4_kernel<8, 8, 8>, kB4Threads,
                                                                        B4Geo<8, 8, 8>::bytes);
    return e == cudaSuccess ? n : 0;
}

cudaError_t b4_launch(const RhsArgs &args, int grid, cudaStream_t stream)
{
    b4_kernel<8, 8, 8><<<grid, kB4Threads, B4Geo<8, 8, 8>::bytes, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace dgb
