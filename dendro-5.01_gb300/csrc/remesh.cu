// Wavelet refinement indicator on the unzipped blocks: Mesh::isReMeshUnzip
// (include/mesh.tcc:2035-2197) with WaveletEl::compute_wavelets_3D
// (src/waveletRefEl.cpp:92-271), element order 6.
//
// Per leaf (one warp), per refinement variable until the running maximum
// passes the leaf's tolerance:
//   interior leaf   the degree-6 interpolant through the 7^3 even points of the
//                   leaf's 13^3 padded patch, evaluated at the 4^3 points with
//                   odd patch indices 3, 5, 7, 9 (separable: x, then y, then z);
//   boundary leaf   the degree-3 interpolant through the leaf's nodes 3, 5, 7, 9,
//                   evaluated at 4, 6, 8 (3^3 points);
//   wavelet         |u - Pu| / max(1, |u|) at those points, RMS over 64 slots
//                   (a boundary leaf's unused 37 slots are zero).
// The reference interpolates all eight children of the parent element and
// reads the odd points from them; the children's other points are never
// read, so this kernel evaluates only the 64 (27) points, with the same
// weights and summation order per point: the Lagrange weight of parent node a
// at the target (one correctly rounded quotient of two exact integers), one
// fused multiply-add chain over a ascending.  The RMS is summed sequentially
// in slot order as normL2 (include/mathUtils.tcc:51-65) does.  Results are
// therefore bit-identical to the oracle's full eight-child restatement.
//
// Memory: a leaf reads 407 (91) values per variable out of its patch; patches
// of neighbouring leaves overlap, so most reads hit L2.  The kernel is bound by
// the FP64 pipe (372 seven-term chains per interior leaf and variable).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>

#include "../../include/dendro_gb300.h"
#include "dgb_internal.h"

namespace dgb {
namespace {

constexpr int kWvWarps = 4;
constexpr int kPatch = 13;

struct WvArgs {
    const double *u[DGB_WAVELET_MAX_VARS];
    int nvars;
    uint64_t nleaves;
    uint64_t unzip_len;
    const uint64_t *base;
    const uint32_t *side;
    const uint8_t *bdy;
    const double *tol;
    double coarse_fac;
    double *wmax;
    uint8_t *flags;
    unsigned long long *changed;
    double wi[4][7];  // interior: weights of the 7 parents at patch index 3, 5, 7, 9
    double wb[3][4];  // boundary: weights of the 4 parents at patch index 4, 6, 8
};

struct WvSmem {
    double par[343];  // parents (interior 7^3, boundary 4^3)
    double odd[64];   // the field at the wavelet points
    double x[196];    // after the x pass
    double y[112];    // after the y pass
    double wc[64];    // wavelets
};

// Lagrange weight of node a of nn uniform nodes at x = tx / 2 (node units).
double lagrange_w(int nn, int tx, int a)
{
    int64_t num = 1, den = 1;
    for (int b = 0; b < nn; b++) {
        if (b == a) continue;
        num *= (int64_t)(tx - 2 * b);
        den *= (int64_t)(2 * a - 2 * b);
    }
    return (double)num / (double)den;
}

template <int N>
__device__ __forceinline__ double chain(const double *w, const double *x, int stride)
{
    double t = __dmul_rn(w[0], x[0]);
#pragma unroll
    for (int a = 1; a < N; a++) t = __fma_rn(w[a], x[a * stride], t);
    return t;
}

// |u - Pu| / max(1, |u|); the division by 1 is skipped (exact either way)
__device__ __forceinline__ double rel_wavelet(double diff, double u)
{
    const double au = fabs(u);
    return 1.0 < au ? __ddiv_rn(fabs(diff), au) : fabs(diff);
}

__global__ void __launch_bounds__(kWvWarps * 32) wavelet_kernel(const WvArgs a)
{
    __shared__ WvSmem smem[kWvWarps];
    const int lane = threadIdx.x & 31;
    WvSmem &s = smem[threadIdx.x >> 5];
    unsigned long long nchanged = 0;
    const uint64_t stride = (uint64_t)gridDim.x * kWvWarps;
    for (uint64_t e = (uint64_t)blockIdx.x * kWvWarps + (threadIdx.x >> 5); e < a.nleaves;
         e += stride) {
        const uint64_t base = a.base[e];
        const uint64_t n = a.side[e];
        const bool bdy = a.bdy[e] != 0;
        const double tol = a.tol[e];
        // the whole patch must lie inside the unzipped vector
        if (n < kPatch || n > (1u << 20) ||
            base + (kPatch - 1) * (1 + n + n * n) >= a.unzip_len) {
            if (lane == 0) {
                a.wmax[e] = __longlong_as_double(0x7ff8000000000000ll);
                a.flags[e] = DGB_OCT_INVALID;
            }
            continue;
        }
        double wm = 0.0;
        for (int v = 0; v < a.nvars; v++) {
            const double *u = a.u[v] + base;
            int nw;
            if (!bdy) {
                for (int t = lane; t < 343; t += 32) {
                    const int i = t % 7, j = (t / 7) % 7, k = t / 49;
                    s.par[t] = __ldg(u + 2 * i + n * (2 * j + n * 2 * k));
                }
                for (int t = lane; t < 64; t += 32) {
                    const int i = t & 3, j = (t >> 2) & 3, k = t >> 4;
                    s.odd[t] = __ldg(u + (3 + 2 * i) + n * ((3 + 2 * j) + n * (3 + 2 * k)));
                }
                __syncwarp();
                for (int t = lane; t < 196; t += 32)  // x[(k*7+j)*4+i]
                    s.x[t] = chain<7>(a.wi[t & 3], s.par + (t >> 2) * 7, 1);
                __syncwarp();
                for (int t = lane; t < 112; t += 32) {  // y[(k*4+jj)*4+i]
                    const int i = t & 3, jj = (t >> 2) & 3, k = t >> 4;
                    s.y[t] = chain<7>(a.wi[jj], s.x + k * 28 + i, 4);
                }
                __syncwarp();
                for (int t = lane; t < 64; t += 32) {  // z[(kk*4+jj)*4+i]
                    const int i = t & 3, jj = (t >> 2) & 3, kk = t >> 4;
                    const double z = chain<7>(a.wi[kk], s.y + jj * 4 + i, 16);
                    s.wc[t] = rel_wavelet(__dsub_rn(z, s.odd[t]), s.odd[t]);
                }
                nw = 64;
            } else {
                for (int t = lane; t < 64; t += 32) {
                    const int i = t & 3, j = (t >> 2) & 3, k = t >> 4;
                    s.par[t] = __ldg(u + (3 + 2 * i) + n * ((3 + 2 * j) + n * (3 + 2 * k)));
                }
                if (lane < 27) {
                    const int i = lane % 3, j = (lane / 3) % 3, k = lane / 9;
                    s.odd[lane] = __ldg(u + (4 + 2 * i) + n * ((4 + 2 * j) + n * (4 + 2 * k)));
                }
                __syncwarp();
                for (int t = lane; t < 48; t += 32)  // x[(k*4+j)*3+i]
                    s.x[t] = chain<4>(a.wb[t % 3], s.par + (t / 3) * 4, 1);
                __syncwarp();
                for (int t = lane; t < 36; t += 32) {  // y[(k*3+jj)*3+i]
                    const int i = t % 3, jj = (t / 3) % 3, k = t / 9;
                    s.y[t] = chain<4>(a.wb[jj], s.x + k * 12 + i, 3);
                }
                __syncwarp();
                if (lane < 27) {  // z[(kk*3+jj)*3+i]
                    const int i = lane % 3, jj = (lane / 3) % 3, kk = lane / 9;
                    const double z = chain<4>(a.wb[kk], s.y + jj * 3 + i, 9);
                    s.wc[lane] = rel_wavelet(__dsub_rn(s.odd[lane], z), s.odd[lane]);
                }
                nw = 27;
            }
            __syncwarp();
            double l = 0.0;
            if (lane == 0) {
                double acc = 0.0;
                for (int t = 0; t < nw; t++) acc = __dadd_rn(acc, __dmul_rn(s.wc[t], s.wc[t]));
                l = __ddiv_rn(__dsqrt_rn(acc), 8.0);  // sqrt(64 slots)
            }
            l = __shfl_sync(0xffffffffu, l, 0);
            __syncwarp();
            if (wm < l) wm = l;
            if (wm > tol) break;
        }
        if (lane == 0) {
            uint8_t f = DGB_OCT_NO_CHANGE;
            if (wm > tol)
                f = DGB_OCT_SPLIT;
            else if (wm < __dmul_rn(a.coarse_fac, tol))
                f = DGB_OCT_COARSE;
            a.wmax[e] = wm;
            a.flags[e] = f;
            nchanged += f != DGB_OCT_NO_CHANGE;
        }
    }
    if (lane == 0 && a.changed && nchanged) atomicAdd(a.changed, nchanged);
}

int wavelet_grid(uint64_t nleaves)
{
    static int cap = 0;
    if (!cap) {
        int dev = 0, sms = 0, occ = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, wavelet_kernel, kWvWarps * 32, 0);
        cap = std::max(1, sms) * std::max(1, occ);
    }
    const uint64_t need = (nleaves + kWvWarps - 1) / kWvWarps;
    return (int)std::min<uint64_t>(need, (uint64_t)cap);
}

}  // namespace
}  // namespace dgb

using namespace dgb;

extern "C" dgb_status dgb_remesh_wavelets(const double *const *unzipped, const uint32_t *var_ids,
                                          int nvars, uint64_t unzip_len, uint64_t nleaves,
                                          const uint64_t *patch_base, const uint32_t *block_side,
                                          const uint8_t *boundary, const double *tol,
                                          double coarse_fac, double *wmax, uint8_t *flags,
                                          unsigned long long *changed, void *stream)
{
    if (!unzipped || !var_ids || nvars < 1 || nvars > DGB_WAVELET_MAX_VARS) {
        set_error("dgb_remesh_wavelets: bad variable list");
        return DGB_ERR_INVALID;
    }
    if (nleaves && (!patch_base || !block_side || !boundary || !tol || !wmax || !flags)) {
        set_error("dgb_remesh_wavelets: null leaf array");
        return DGB_ERR_INVALID;
    }
    WvArgs a{};
    for (int v = 0; v < nvars; v++) {
        a.u[v] = unzipped[var_ids[v]];
        if (!a.u[v]) {
            set_error("dgb_remesh_wavelets: null field pointer");
            return DGB_ERR_INVALID;
        }
    }
    a.nvars = nvars;
    a.nleaves = nleaves;
    a.unzip_len = unzip_len;
    a.base = patch_base;
    a.side = block_side;
    a.bdy = boundary;
    a.tol = tol;
    a.coarse_fac = coarse_fac;
    a.wmax = wmax;
    a.flags = flags;
    a.changed = changed;
    for (int i = 0; i < 4; i++)
        for (int b = 0; b < 7; b++) a.wi[i][b] = lagrange_w(7, 3 + 2 * i, b);
    for (int i = 0; i < 3; i++)
        for (int b = 0; b < 4; b++) a.wb[i][b] = lagrange_w(4, 1 + 2 * i, b);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (changed) e = cudaMemsetAsync(changed, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess && nleaves) {
        wavelet_kernel<<<wavelet_grid(nleaves), kWvWarps * 32, 0, st>>>(a);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        set_error(std::string("dgb_remesh_wavelets: ") + cudaGetErrorString(e));
        return DGB_ERR_CUDA;
    }
    return DGB_OK;
}
