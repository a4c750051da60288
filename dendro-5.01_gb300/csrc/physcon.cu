// Constraint diagnostics on padded octant blocks: Hamiltonian, momentum and
// Psi4 (physical_constraints, BSSN_GR/src/physcon.cpp:12-96), one persistent,
// work-queued launch over all blocks of a plan, plus the masked L2 norm the
// reference reports for them (computeConstraintL2Norm,
// BSSN_GR/include/grUtils.tcc:40-88).
//
// Work item = a tile of one block's interior (the plan's 8x8x8 schedule).
// Per item:
//   phase D  for each of the 17 fields the diagnostics differentiate (chi,
//            Gt0-2, K, gt0-5, At0-5; BSSN_GR/scripts/constraint_derivs.h):
//            stage tile + 2 on each side in shared memory (cp.async, double
//            buffered), write first derivatives and, for chi and gt0-5, the
//            second and mixed derivatives to the CTA's workspace slice;
//   phase A  one thread per tile point: the Ricci tensor, Hamiltonian,
//            momentum, the Gram-Schmidt tetrad and Psi4
//            (CodeGen/constraints.py:52-172, CodeGen/dendro.py:470-532).
// Stencils are the 4th-order family the reference binds for this call
// (BSSN_GR/include/physcon.h:9-15 -> deriv42_*, BSSN_GR/src/derivs.cpp:11-490)
// with its one-sided closures at domain-boundary faces, evaluated in the
// reference's rounding order; mixed derivatives are d_y(d_x u), d_z(d_x u),
// d_z(d_y u) as the reference composes them.  Everything is FP64.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dgb_internal.h"
#include "exact_mul.cuh"
#include "stencil42.cuh"
#include "tile_index.cuh"

namespace dgb {
namespace {

constexpr int kPcThreads = 256;
#ifndef DGB_PC_MIN_CTAS
#define DGB_PC_MIN_CTAS 2
#endif
// CTAs per SM the register budget is sized for (255 registers at 1, 128 at 2)
constexpr int kPcMinBlocks = DGB_PC_MIN_CTAS;
constexpr int kNumCFields = 17;
constexpr int kGradSlots = 3 * kNumCFields;            // 51
constexpr int kPcSlots = kGradSlots + 7 * 6;           // + chi, gt0-5 second derivatives
// differentiated fields, in slot order, and their VAR index
__constant__ int c_cfield[kNumCFields] = {1, 3, 4, 5, 2, 12, 13, 14, 15, 16, 17,
                                          18, 19, 20, 21, 22, 23};
// slot q -> second-derivative group (0 = chi, 1..6 = gt0..5) or -1
__constant__ int8_t c_cd2[kNumCFields] = {0, -1, -1, -1, -1, 1, 2, 3, 4, 5, 6,
                                          -1, -1, -1, -1, -1, -1};
enum { Q_CHI = 0, Q_GT = 1, Q_K = 4, Q_G = 5, Q_A = 11 };

__host__ __device__ constexpr int sy(int a, int b)
{
    return (a < b ? a : b) == 0 ? (a < b ? b : a) : ((a < b ? a : b) == 1 ? 2 + (a < b ? b : a) : 5);
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ---------------------------------------------------------------- point algebra
struct PcIO {
    const double *const *uu;
    const double *S;
    int pmax, p;
    uint64_t gi;
    __device__ __forceinline__ double u(int v) const { return __ldg(uu[v] + gi); }
    __device__ __forceinline__ double d(int slot) const { return S[(size_t)slot * pmax + p]; }
    __device__ __forceinline__ double grad(int q, int dir) const { return d(3 * q + dir); }
    // second derivative of group r (0 chi, 1..6 gt0..5), pair m = sy(l, m)
    __device__ __forceinline__ double dd(int r, int m) const { return d(kGradSlots + 6 * r + m); }
};

// weight of a symmetric pair in a full (l, m) double sum
__device__ __forceinline__ constexpr double wpair(int m) { return (m == 0 || m == 3 || m == 5) ? 1.0 : 2.0; }

__device__ __forceinline__ void physcon_point(const PcIO &io, double x, double y, double z,
                                              double out[6])
{
    double g[6], A[6], ig[6];
    const double chi = io.u(1), K = io.u(2);
#pragma unroll
    for (int m = 0; m < 6; m++) {
        g[m] = io.u(12 + m);
        A[m] = io.u(18 + m);
    }
    const double det = g[0] * (g[3] * g[5] - g[4] * g[4]) - g[1] * g[1] * g[5]
                     + 2.0 * g[1] * g[2] * g[4] - g[2] * g[2] * g[3];
    ig[0] = (g[3] * g[5] - g[4] * g[4]) / det;
    ig[1] = (g[2] * g[4] - g[1] * g[5]) / det;
    ig[2] = (g[1] * g[4] - g[2] * g[3]) / det;
    ig[3] = (g[0] * g[5] - g[2] * g[2]) / det;
    ig[4] = (g[1] * g[2] - g[0] * g[4]) / det;
    ig[5] = (g[0] * g[3] - g[1] * g[1]) / det;

    // C1[k][(i,j)] = 0.5 (d_j g_ki + d_i g_kj - d_k g_ij), reduced where indices
    // coincide (d_k g_kk / 2, d_i g_ki - d_k g_ii / 2, d_j g_kk / 2); C2 = ig . C1
    double C1[3][6], C2[3][6];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++) {
                double c;
                if (i == j && j == k)
                    c = 0.5 * io.grad(Q_G + sy(k, k), k);
                else if (i == j)
                    c = io.grad(Q_G + sy(k, i), i) - 0.5 * io.grad(Q_G + sy(i, i), k);
                else if (k == i)
                    c = 0.5 * io.grad(Q_G + sy(k, k), j);
                else if (k == j)
                    c = 0.5 * io.grad(Q_G + sy(k, k), i);
                else
                    c = 0.5 * (io.grad(Q_G + sy(k, i), j) + io.grad(Q_G + sy(k, j), i)
                               - io.grad(Q_G + sy(i, j), k));
                C1[k][sy(i, j)] = c;
            }
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int m = 0; m < 6; m++)
            C2[k][m] = ig[sy(k, 0)] * C1[0][m] + ig[sy(k, 1)] * C1[1][m] + ig[sy(k, 2)] * C1[2][m];
    double CalGt[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
#pragma unroll
        for (int m = 0; m < 6; m++) s += wpair(m) * ig[m] * C2[i][m];
        CalGt[i] = s;
    }
    double dchi[3];
#pragma unroll
    for (int d = 0; d < 3; d++) dchi[d] = io.grad(Q_CHI, d);
    const double ichi = 1.0 / chi;
    double trchi = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = 0; l < 3; l++)
            trchi += ig[sy(k, l)] * (io.dd(0, sy(k, l)) - 1.5 * ichi * dchi[k] * dchi[l]);
    const double CalGtdchi = CalGt[0] * dchi[0] + CalGt[1] * dchi[1] + CalGt[2] * dchi[2];

    // Ricci tensor (CodeGen/dendro.py:470-532).  The quadratic term contracts
    // the raised Christoffels C2U[k][i][m] = ig^lm C2^k_li and C1U[k][m][j] =
    // ig^ml C1_klj once instead of ig^lm inside a triple sum per component;
    // C1_ijk + C1_jik = d_k g_ij; on the diagonal the two halves of each
    // symmetrised term are equal and are evaluated once.
    double C2U[3][3][3], C1U[3][3][3];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int m = 0; m < 3; m++) {
                C2U[k][i][m] = ig[sy(0, m)] * C2[k][sy(0, i)] + ig[sy(1, m)] * C2[k][sy(1, i)]
                             + ig[sy(2, m)] * C2[k][sy(2, i)];
                C1U[k][i][m] = ig[sy(i, 0)] * C1[k][sy(0, m)] + ig[sy(i, 1)] * C1[k][sy(1, m)]
                             + ig[sy(i, 2)] * C1[k][sy(2, m)];
            }
    double R[6];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            double t1 = 0.0, c2d = 0.0;
#pragma unroll
            for (int m = 0; m < 6; m++) t1 += wpair(m) * ig[m] * io.dd(1 + sy(i, j), m);
#pragma unroll
            for (int k = 0; k < 3; k++) c2d += C2[k][sy(i, j)] * dchi[k];
            const double xR = 0.5 * ichi * (io.dd(0, sy(i, j)) - c2d) - 0.25 * ichi * ichi * dchi[i] * dchi[j];
            double rt;
            if (i == j) {
                double h2 = 0.0, h3 = 0.0, t4a = 0.0, t4b = 0.0;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    h2 += g[sy(k, i)] * io.grad(Q_GT + k, i);
                    h3 += CalGt[k] * C1[i][sy(i, k)];
                }
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int m = 0; m < 3; m++) {
                        t4a += C2U[k][i][m] * C1[i][sy(k, m)];
                        t4b += C2[k][sy(i, m)] * C1U[k][m][i];
                    }
                rt = -0.5 * t1 + h2 + h3 + (2.0 * t4a + t4b);
            } else {
                double t2 = 0.0, t3 = 0.0, t4 = 0.0;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    t2 += g[sy(k, i)] * io.grad(Q_GT + k, j) + g[sy(k, j)] * io.grad(Q_GT + k, i);
                    t3 += CalGt[k] * io.grad(Q_G + sy(i, j), k);
                }
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int m = 0; m < 3; m++)
                        t4 += C2U[k][i][m] * C1[j][sy(k, m)] + C2U[k][j][m] * C1[i][sy(k, m)]
                            + C2[k][sy(i, m)] * C1U[k][m][j];
                rt = -0.5 * t1 + 0.5 * t2 + 0.5 * t3 + t4;
            }
            R[sy(i, j)] = rt + xR + 0.5 * ichi * g[sy(i, j)] * (trchi - CalGtdchi);
        }

    // Hamiltonian (CodeGen/constraints.py:158)
    double Aup[6];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int l = 0; l < 3; l++) s += ig[sy(i, k)] * ig[sy(j, l)] * A[sy(k, l)];
            Aup[sy(i, j)] = s;
        }
    double chiR = 0.0, sqrA = 0.0;
#pragma unroll
    for (int m = 0; m < 6; m++) {
        chiR += wpair(m) * chi * ig[m] * R[m];
        sqrA += wpair(m) * A[m] * Aup[m];
    }
    out[0] = chiR - sqrA + (2.0 / 3.0) * K * K;

    // momentum (CodeGen/constraints.py:161-170)
#pragma unroll
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double c = 0.0;
#pragma unroll
                for (int m = 0; m < 3; m++) c += C2[m][sy(k, i)] * A[sy(j, m)];
                s += ig[sy(j, k)] * (io.grad(Q_A + sy(i, j), k) - c);
            }
#pragma unroll
        for (int j = 0; j < 3; j++) s -= io.u(3 + j) * A[sy(i, j)];
        double t = 0.0;
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int k = 0; k < 3; k++) t += ig[sy(j, k)] * A[sy(k, i)] * dchi[j];
        s -= 1.5 * t * ichi;
        s -= (2.0 / 3.0) * io.grad(Q_K, i);
        out[1 + i] = s;
    }

    // Psi4 (CodeGen/constraints.py:52-152); zero on the z axis
    // (BSSN_GR/src/physconeqs.cpp:1039-1044)
    if (fabs(x) <= 1e-7 && fabs(y) <= 1e-7) {
        out[4] = 0.0;
        out[5] = 0.0;
        return;
    }
    double gd[6];
#pragma unroll
    for (int m = 0; m < 6; m++) gd[m] = g[m] * ichi;
    auto dot = [&](const double *a, const double *b) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) s += gd[sy(i, j)] * a[i] * b[j];
        return s;
    };
    double rv[3] = {x, y, z}, th[3] = {x * z, y * z, -(x * x + y * y)}, ph[3] = {-y, x, 0.0};
    {
        const double n = sqrt(dot(rv, rv));
#pragma unroll
        for (int i = 0; i < 3; i++) rv[i] /= n;
    }
    {
        const double p1 = dot(th, th), p2 = dot(rv, th);
#pragma unroll
        for (int i = 0; i < 3; i++) th[i] -= p2 * rv[i];
        const double n = sqrt(p1 - p2 * p2);
#pragma unroll
        for (int i = 0; i < 3; i++) th[i] /= n;
    }
    {
        const double p1 = dot(ph, ph), p2 = dot(rv, ph), p3 = dot(th, ph);
#pragma unroll
        for (int i = 0; i < 3; i++) ph[i] -= p2 * rv[i] + p3 * th[i];
        const double n = sqrt(p1 - p2 * p2 - p3 * p3);
#pragma unroll
        for (int i = 0; i < 3; i++) ph[i] /= n;
    }
    const double invsqrt2 = 0.7071067811865475244;
    double mre[3], mim[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        mre[i] = th[i] * invsqrt2;
        mim[i] = ph[i] * invsqrt2;
    }
    double Av[3];
#pragma unroll
    for (int i = 0; i < 3; i++) Av[i] = A[sy(i, 0)] * rv[0] + A[sy(i, 1)] * rv[1] + A[sy(i, 2)] * rv[2];
    double p3r = 0.0, p3i = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            if (i == j) continue;  // MR, NR are antisymmetric
            double uu = 0.0, vv = 0.0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double c = io.grad(Q_A + sy(k, i), j);
#pragma unroll
                for (int m = 0; m < 3; m++) c += C2[m][sy(k, i)] * A[sy(m, j)];
                uu += mre[k] * c;
                vv += mim[k] * c;
            }
            const double MR = mre[i] * rv[j] - mre[j] * rv[i];
            const double NR = mim[i] * rv[j] - mim[j] * rv[i];
            p3r += MR * uu - NR * vv;
            p3i += NR * uu + MR * vv;
        }
    p3r *= ichi;
    p3i *= ichi;
    double rdchi = 0.0, mredchi = 0.0, mimdchi = 0.0, mreA = 0.0, mimA = 0.0, Ar = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        rdchi += rv[i] * dchi[i];
        mredchi += mre[i] * dchi[i];
        mimdchi += mim[i] * dchi[i];
        mreA += mre[i] * Av[i];
        mimA += mim[i] * Av[i];
        Ar += Av[i] * rv[i];
    }
    const double Atemp = ichi * ichi * (Ar + K * chi / 3.0 + 0.5 * rdchi);
    double p1r = 0.0, p1i = 0.0, p2r = 0.0, p2i = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            const double w = (i == j) ? 1.0 : 2.0;
            const double MM = mre[i] * mre[j] - mim[i] * mim[j];
            const double NN = mre[i] * mim[j] + mre[j] * mim[i];
            p1r += w * R[sy(i, j)] * MM;
            p1i += w * R[sy(i, j)] * NN;
            p2r += w * A[sy(i, j)] * MM;
            p2i += w * A[sy(i, j)] * NN;
        }
    p2r *= Atemp;
    p2i *= Atemp;
    const double p4r = ichi * ichi * (mreA * (mreA + 0.5 * mredchi) - mimA * (mimA + 0.5 * mimdchi));
    const double p4i = ichi * ichi * (mreA * (mimA - 0.5 * mimdchi) + mimA * (mreA - 0.5 * mredchi));
    out[4] = p1r + p2r - p3r - p4r;
    out[5] = -(p1i + p2i - p3i - p4i);
}

// ---------------------------------------------------------------- kernel
template <int TX, int TY, int TZ>
struct PcGeo {
    static constexpr int PX = TX + 4, PY = TY + 4, PZ = TZ + 4;
    static constexpr int FBUF = PX * PY * PZ;
    static constexpr int DXB = TX * PY * PZ;
    static constexpr int DYB = TX * TY * PZ;
    static constexpr int PMAX = TX * TY * TZ;
    static constexpr size_t bytes = (size_t)(2 * FBUF + DXB + DYB) * 8;
    // DivBy (tile_index.cuh) splits indices q < FBUF by extents < 32 exactly
    static_assert(FBUF < (1 << 13) && TX + 6 < 32 && TY + 6 < 32 && TZ + 6 < 32, "tile too large for DivBy");
};

// Phase D of a work item.  BDY: the block touches a domain face.  Interior
// blocks are compiled with the closure tests constant-false, so the
// one-sided stencils are not issued under a false predicate on every point.
template <int TX, int TY, int TZ, bool BDY>
__device__ __forceinline__ void physcon_item(const PcArgs &args, const WorkItem &w, const DevBlock &blk,
                                             double *S)
{
    using G = PcGeo<TX, TY, TZ>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *fb0 = reinterpret_cast<double *>(smem_raw);
    double *fb1 = fb0 + G::FBUF;
    double *dxb = fb1 + G::FBUF;
    double *dyb = dxb + G::DXB;
    const int tid = threadIdx.x;
    const int nx = blk.sz[0], ny = blk.sz[1], nz = blk.sz[2];
    const int ex = w.e[0], ey = w.e[1], ez = w.e[2];
    const int px = ex + 4, py = ey + 4, pz = ez + 4;
    const int npad = px * py * pz;
    const DivBy dpx(px), dpy(py);
    const int P = ex * ey * ez;
    const DivBy dex(ex), dey(ey);
    const int sy_ = px, sz_ = px * py;
    // staged region starts 2 points before the tile's first interior point
    const uint64_t rbase = blk.offset + (uint64_t)(w.o[0] + 1)
                         + (uint64_t)nx * ((uint64_t)(w.o[1] + 1) + (uint64_t)ny * (w.o[2] + 1));
    const uint32_t bflag = BDY ? blk.bflag : 0u;
    const bool lo[3] = {(bflag & 1u) != 0, (bflag & 4u) != 0, (bflag & 16u) != 0};
    const bool hi[3] = {(bflag & 2u) != 0, (bflag & 8u) != 0, (bflag & 32u) != 0};
    const Ax4 ax[3] = {ax4(blk.h[0]), ax4(blk.h[1]), ax4(blk.h[2])};

    auto issue_load = [&](int q, double *dst) {
        const double *src = args.u[c_cfield[q]] + rbase;
        for (int e = tid; e < npad; e += kPcThreads) {
            int i, j, k;
            split3(e, dpx, dpy, i, j, k);
            cp_async8(dst + e, src + i + (uint64_t)nx * (j + (uint64_t)ny * k));
        }
        cp_async_commit();
    };

    issue_load(0, fb0);
    for (int q = 0; q < kNumCFields; q++) {
        double *F = (q & 1) ? fb1 : fb0;
        if (q + 1 < kNumCFields) {
            issue_load(q + 1, (q & 1) ? fb0 : fb1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        double *Sg = S + (size_t)(3 * q) * G::PMAX;
        const int r2 = c_cd2[q];
        if (r2 < 0) {
            for (int p = tid; p < P; p += kPcThreads) {
                int ti, tj, tk;
                split3(p, dex, dey, ti, tj, tk);
                const double *c = F + (ti + 2) + sy_ * (tj + 2) + sz_ * (tk + 2);
                Sg[p] = d1_42_at(c, 1, w.o[0] + ti + 3, nx, lo[0], hi[0], ax[0]);
                Sg[G::PMAX + p] = d1_42_at(c, sy_, w.o[1] + tj + 3, ny, lo[1], hi[1], ax[1]);
                Sg[2 * G::PMAX + p] = d1_42_at(c, sz_, w.o[2] + tk + 3, nz, lo[2], hi[2], ax[2]);
            }
        } else {
            double *S2 = S + (size_t)(kGradSlots + 6 * r2) * G::PMAX;
            // d_x on x in tile and (y in tile +- 2, z in tile) or (y in tile, z in the z halo)
            const int by = ey + 4;
            const DivBy dby(by);
            const int nA = ex * by * ez, nB = ex * ey * 4;
            for (int e = tid; e < nA + nB; e += kPcThreads) {
                int ti, tj, tk;
                if (e < nA) {
                    split3(e, dex, dby, ti, tj, tk);
                    tk += 2;
                } else {
                    const int e3 = e - nA;
                    int kk;  // 0..3
                    split3(e3, dex, dey, ti, tj, kk);
                    tj += 2;
                    tk = kk < 2 ? kk : ez + kk;
                }
                const double *c = F + (ti + 2) + sy_ * tj + sz_ * tk;
                dxb[ti + ex * (tj + by * tk)] = d1_42_at(c, 1, w.o[0] + ti + 3, nx, lo[0], hi[0], ax[0]);
            }
            // d_y on x, y in tile, z in tile +- 2
            const int nC = ex * ey * pz;
            for (int e = tid; e < nC; e += kPcThreads) {
                int ti, tj, tk;
                split3(e, dex, dey, ti, tj, tk);
                const double *c = F + (ti + 2) + sy_ * (tj + 2) + sz_ * tk;
                dyb[e] = d1_42_at(c, sy_, w.o[1] + tj + 3, ny, lo[1], hi[1], ax[1]);
            }
            for (int p = tid; p < P; p += kPcThreads) {
                int ti, tj, tk;
                split3(p, dex, dey, ti, tj, tk);
                const int pi = w.o[0] + ti + 3, pj = w.o[1] + tj + 3, pk = w.o[2] + tk + 3;
                const double *c = F + (ti + 2) + sy_ * (tj + 2) + sz_ * (tk + 2);
                Sg[2 * G::PMAX + p] = d1_42_at(c, sz_, pk, nz, lo[2], hi[2], ax[2]);
                S2[0 * G::PMAX + p] = d2_42_at(c, 1, pi, nx, lo[0], hi[0], ax[0]);
                S2[3 * G::PMAX + p] = d2_42_at(c, sy_, pj, ny, lo[1], hi[1], ax[1]);
                S2[5 * G::PMAX + p] = d2_42_at(c, sz_, pk, nz, lo[2], hi[2], ax[2]);
            }
            __syncthreads();
            for (int p = tid; p < P; p += kPcThreads) {
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
// boundary blocks.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void physcon_points(const PcArgs &args, const WorkItem &w,
                                               const DevBlock &blk, const double *S)
{
    using G = PcGeo<TX, TY, TZ>;
    const int tid = threadIdx.x;
    const int nx = blk.sz[0], ny = blk.sz[1];
    const int ex = w.e[0], ey = w.e[1], ez = w.e[2];
    const int P = ex * ey * ez;
    const DivBy dex(ex), dey(ey);
    for (int p = tid; p < P; p += kPcThreads) {
        int ti, tj, tk;
        split3(p, dex, dey, ti, tj, tk);
        const int i = w.o[0] + ti + 3, j = w.o[1] + tj + 3, k = w.o[2] + tk + 3;
        const uint64_t gi = blk.offset + (uint64_t)i + (uint64_t)nx * ((uint64_t)j + (uint64_t)ny * k);
        // x = pmin + i h with the reference's two roundings (physcon.cpp:64-69)
        const double x = __dadd_rn(blk.pmin[0], __dmul_rn((double)i, blk.h[0]));
        const double y = __dadd_rn(blk.pmin[1], __dmul_rn((double)j, blk.h[1]));
        const double z = __dadd_rn(blk.pmin[2], __dmul_rn((double)k, blk.h[2]));
        PcIO io{args.u, S, G::PMAX, p, gi};
        double out[6];
        physcon_point(io, x, y, z, out);
#pragma unroll
        for (int c = 0; c < 6; c++) args.cons[c][gi] = out[c];
    }
}

template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(kPcThreads, kPcMinBlocks) physcon_kernel(const PcArgs args)
{
    using G = PcGeo<TX, TY, TZ>;
    __shared__ int s_item;
    double *S = args.scratch + (size_t)blockIdx.x * kPcSlots * G::PMAX;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = (int)atomicAdd(args.queue, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= (int)args.nitems) break;
        const WorkItem w = args.items[it];
        const DevBlock blk = args.blocks[w.blk];
        if (blk.bflag == 0)
            physcon_item<TX, TY, TZ, false>(args, w, blk, S);
        else
            physcon_item<TX, TY, TZ, true>(args, w, blk, S);
        physcon_points<TX, TY, TZ>(args, w, blk, S);
    }
}

// ---------------------------------------------------------------- masked L2 norm
// Per CTA: sum of squares of each field over the nodes whose mask value is
// >= threshold, and the count; fixed partition and fixed reduction order,
// so the result is reproducible run to run.
constexpr int kNormThreads = 256;
constexpr int kNormCtas = 1024;

__global__ void __launch_bounds__(kNormThreads) l2_partial_kernel(const NormArgs a)
{
    __shared__ double sh[kNormThreads / 32][DGB_NUM_CONSTRAINTS + 1];
    double acc[DGB_NUM_CONSTRAINTS + 1];
#pragma unroll
    for (int v = 0; v <= DGB_NUM_CONSTRAINTS; v++) acc[v] = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * kNormThreads;
    for (uint64_t n = (uint64_t)blockIdx.x * kNormThreads + threadIdx.x; n < a.ndof; n += stride) {
        if (a.mask && a.mask[n] < a.threshold) continue;  // as the reference: NaN counts
#pragma unroll
        for (int v = 0; v < DGB_NUM_CONSTRAINTS; v++)
            if (v < a.nvars) {
                const double c = a.f[v][n];
                acc[v] += c * c;
            }
        acc[DGB_NUM_CONSTRAINTS] += 1.0;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v <= DGB_NUM_CONSTRAINTS; v++) {
        double s = acc[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sh[warp][v] = s;
    }
    __syncthreads();
    if (threadIdx.x <= DGB_NUM_CONSTRAINTS) {
        double s = 0.0;
        for (int q = 0; q < kNormThreads / 32; q++) s += sh[q][threadIdx.x];
        a.partial[(size_t)blockIdx.x * (DGB_NUM_CONSTRAINTS + 1) + threadIdx.x] = s;
    }
}

__global__ void __launch_bounds__(32) l2_final_kernel(const double *partial, int nparts, int nvars,
                                                      double *out)
{
    __shared__ double tot[DGB_NUM_CONSTRAINTS + 1];
    const int v = threadIdx.x;
    if (v <= DGB_NUM_CONSTRAINTS) {
        double s = 0.0;
        for (int q = 0; q < nparts; q++) s += partial[(size_t)q * (DGB_NUM_CONSTRAINTS + 1) + v];
        tot[v] = s;
    }
    __syncthreads();
    const double cnt = tot[DGB_NUM_CONSTRAINTS];
    if (v < nvars) out[v] = cnt > 0.0 ? sqrt(tot[v] / cnt) : 0.0;
    if (v == DGB_NUM_CONSTRAINTS) out[DGB_NUM_CONSTRAINTS] = cnt;
}

}  // namespace

size_t physcon_smem_bytes() { return PcGeo<8, 8, 8>::bytes; }
size_t physcon_scratch_per_cta() { return (size_t)kPcSlots * PcGeo<8, 8, 8>::PMAX; }
int physcon_threads() { return kPcThreads; }

cudaError_t physcon_configure()
{
    return cudaFuncSetAttribute(physcon_kernel<8, 8, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)PcGeo<8, 8, 8>::bytes);
}

int physcon_max_ctas_per_sm()
{
    int n = 0;
    if (physcon_configure() != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, physcon_kernel<8, 8, 8>, kPcThreads,
                                                      PcGeo<8, 8, 8>::bytes) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t physcon_launch(const PcArgs &args, int grid, cudaStream_t stream)
{
    physcon_kernel<8, 8, 8><<<grid, kPcThreads, PcGeo<8, 8, 8>::bytes, stream>>>(args);
    return cudaGetLastError();
}

int norm_partials() { return kNormCtas; }

cudaError_t l2_norm_launch(const NormArgs &a, double *out_dev, cudaStream_t stream)
{
    l2_partial_kernel<<<kNormCtas, kNormThreads, 0, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    l2_final_kernel<<<1, 32, 0, stream>>>(a.partial, kNormCtas, a.nvars, out_dev);
    return cudaGetLastError();
}

}  // namespace dgb
