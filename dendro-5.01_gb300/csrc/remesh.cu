// Wavelet refinement indicator on the unzipped blocks: Mesh::isReMeshUnzip
// (include/mesh.tcc:2035-2197) with WaveletEl::compute_wavelets_3D
// (src/waveletRefEl.cpp:92-271), element order 6.
//
// Per leaf, per refinement variable until the running maximum passes the
// leaf's tolerance:
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
// Schedule: persistent CTAs of 4 warps; each warp owns an equal contiguous
// range of leaves and works through it in batches of 16: all 32 lanes
// interpolate one leaf at a time (squared wavelets to shared memory), then
// lane b sums leaf b's 64 squares, so the 16 sequential sums of a batch run
// side by side.  Memory: a leaf reads 407 (91) values per variable out of its
// patch; neighbouring patches overlap, so most reads hit L2.  The kernel is
// bound by the FP64 pipe (372 seven-term chains per interior leaf and
// variable, about 100 warp instructions of which 91 are the chains).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>

#include "../../include/dendro_gb300.h"
#include "dgb_internal.h"

namespace dgb {
namespace {

constexpr int kWvWarps = 4;
constexpr int kBatch = 16;  // leaves per warp whose RMS sums run side by side
constexpr int kPatch = 13;
constexpr int kWcStride = 65;  // padded row: lanes reading row b hit distinct banks

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
};

// Interpolation weights (constants of the method, set once per process):
// interior, the 7 parents at patch index 3, 5, 7, 9; boundary, the 4 parents
// at patch index 4, 6, 8.
__constant__ double c_wi[4][7];
__constant__ double c_wb[3][4];

struct WvSmem {
    double par[343];                 // parents (interior 7^3, boundary 4^3)
    double x[196];                   // after the x pass
    double y[112];                   // after the y pass
    double sq[kBatch][kWcStride];    // squared wavelets of the batch's leaves
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
// (|u - Pu| / max(1, |u|))^2 on the lanes of `mask`.  The division by
// max(1, |u|) = 1 is exact, so it is only carried out when some lane has
// |u| > 1 (the refinement fields are mostly of magnitude <= 1).
__device__ __forceinline__ double rel_wavelet_sq(double diff, double u, unsigned mask)
{
    const double au = fabs(u);
    double w = fabs(diff);
    const bool big = 1.0 < au;
    if (__any_sync(mask, big)) {
        const double q = __ddiv_rn(w, au);
        if (big) w = q;
    }
    return __dmul_rn(w, w);
}

// Squared wavelets of one leaf's patch (u at its first point) into row[0..63]
// (interior) or row[0..26] (boundary), slot order of compute_wavelets_3D.
__device__ __forceinline__ void leaf_wavelets(WvSmem &s, const double *u, uint64_t n, bool bdy,
                                              double *row, int lane)
{
    if (!bdy) {
        double odd[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int t = lane + 32 * q;
            const int i = t & 3, j = (t >> 2) & 3, k = t >> 4;
            odd[q] = __ldg(u + (3 + 2 * i) + n * ((3 + 2 * j) + n * (3 + 2 * k)));
        }
        for (int t = lane; t < 343; t += 32) {
            const int i = t % 7, j = (t / 7) % 7, k = t / 49;
            s.par[t] = __ldg(u + 2 * i + n * (2 * j + n * 2 * k));
        }
        __syncwarp();
        for (int t = lane; t < 196; t += 32)  // x[(k*7+j)*4+i]
            s.x[t] = chain<7>(c_wi[t & 3], s.par + (t >> 2) * 7, 1);
        __syncwarp();
        for (int t = lane; t < 112; t += 32) {  // y[(k*4+jj)*4+i]
            const int i = t & 3, jj = (t >> 2) & 3, k = t >> 4;
            s.y[t] = chain<7>(c_wi[jj], s.x + k * 28 + i, 4);
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 2; q++) {  // z[(kk*4+jj)*4+i]
            const int t = lane + 32 * q;
            const int i = t & 3, jj = (t >> 2) & 3, kk = t >> 4;
            const double z = chain<7>(c_wi[kk], s.y + jj * 4 + i, 16);
            row[t] = rel_wavelet_sq(__dsub_rn(z, odd[q]), odd[q], 0xffffffffu);
        }
    } else {
        const int i3 = lane % 3, j3 = (lane / 3) % 3, k3 = lane / 9;
        const double odd =
            lane < 27 ? __ldg(u + (4 + 2 * i3) + n * ((4 + 2 * j3) + n * (4 + 2 * k3))) : 0.0;
        for (int t = lane; t < 64; t += 32) {  // parents at 3, 5, 7, 9
            const int i = t & 3, j = (t >> 2) & 3, k = t >> 4;
            s.par[t] = __ldg(u + (3 + 2 * i) + n * ((3 + 2 * j) + n * (3 + 2 * k)));
        }
        __syncwarp();
        for (int t = lane; t < 48; t += 32)  // x[(k*4+j)*3+i]
            s.x[t] = chain<4>(c_wb[t % 3], s.par + (t / 3) * 4, 1);
        __syncwarp();
        for (int t = lane; t < 36; t += 32) {  // y[(k*3+jj)*3+i]
            const int i = t % 3, jj = (t / 3) % 3, k = t / 9;
            s.y[t] = chain<4>(c_wb[jj], s.x + k * 12 + i, 3);
        }
        __syncwarp();
        if (lane < 27) {  // z[(kk*3+jj)*3+i]
            const double z = chain<4>(c_wb[k3], s.y + j3 * 3 + i3, 9);
            row[lane] = rel_wavelet_sq(__dsub_rn(odd, z), odd, 0x07ffffffu);
        }
    }
    __syncwarp();  // par / x / y are reused by the next leaf
}

// One warp per batch of kBatch leaves.  Per refinement variable, the warp
// computes the wavelets of every leaf of the batch still below its
// tolerance (all lanes on one leaf at a time), then lane b sums leaf b's 64
// squares in slot order: the sequential sums of 16 leaves run side by side.
__global__ void __launch_bounds__(kWvWarps * 32, 4) wavelet_kernel(const WvArgs a)
{
    extern __shared__ __align__(16) unsigned char wv_smem[];
    const int lane = threadIdx.x & 31;
    WvSmem &s = reinterpret_cast<WvSmem *>(wv_smem)[threadIdx.x >> 5];
    unsigned long long nchanged = 0;
    // warp w owns leaves [w L / W, (w + 1) L / W): equal shares, no tail wave
    const uint64_t nw = (uint64_t)gridDim.x * kWvWarps;
    const uint64_t w = (uint64_t)blockIdx.x * kWvWarps + (threadIdx.x >> 5);
    const uint64_t lo = w * a.nleaves / nw, hi = (w + 1) * a.nleaves / nw;
    for (uint64_t b0 = lo; b0 < hi; b0 += kBatch) {
        const uint64_t e = b0 + lane;
        bool mine = lane < kBatch && e < hi;
        uint64_t base = 0, n = 0;
        bool bdy = false;
        double tol = 0.0;
        if (mine) {
            base = a.base[e];
            n = a.side[e];
            bdy = a.bdy[e] != 0;
            tol = a.tol[e];
            // the whole patch must lie inside the unzipped vector
            if (n < kPatch || n > (1u << 20) ||
                base + (kPatch - 1) * (1 + n + n * n) >= a.unzip_len) {
                a.wmax[e] = __longlong_as_double(0x7ff8000000000000ll);
                a.flags[e] = DGB_OCT_INVALID;
                mine = false;
            }
        }
        unsigned active = __ballot_sync(0xffffffffu, mine);
        const unsigned valid = active;
        double wm = 0.0;
        for (int v = 0; v < a.nvars && active; v++) {
            for (unsigned m = active; m; m &= m - 1) {
                const int b = __ffs(m) - 1;
                const uint64_t bb = __shfl_sync(0xffffffffu, base, b);
                const uint64_t nb = __shfl_sync(0xffffffffu, n, b);
                const bool db = __shfl_sync(0xffffffffu, (int)bdy, b) != 0;
                leaf_wavelets(s, a.u[v] + bb, nb, db, s.sq[b], lane);
            }
            if ((active >> lane) & 1u) {
                const double *row = s.sq[lane];
                const int nw = bdy ? 27 : 64;
                double acc = 0.0;
                for (int t = 0; t < nw; t++) acc = __dadd_rn(acc, row[t]);
                const double l = __ddiv_rn(__dsqrt_rn(acc), 8.0);  // sqrt(64 slots)
                if (wm < l) wm = l;
            }
            active = __ballot_sync(0xffffffffu, ((active >> lane) & 1u) && !(wm > tol));
            __syncwarp();  // the rows are rewritten for the next variable
        }
        if ((valid >> lane) & 1u) {
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
    // warp total, one atomic per warp
    for (int o = 16; o; o >>= 1) nchanged += __shfl_xor_sync(0xffffffffu, nchanged, o);
    if (lane == 0 && a.changed && nchanged) atomicAdd(a.changed, nchanged);
}

constexpr size_t kWvSmemBytes = kWvWarps * sizeof(WvSmem);

int g_wavelet_cap = 0;  // CTAs resident on the device at once

cudaError_t wavelet_configure()
{
    if (g_wavelet_cap) return cudaSuccess;
    double wi[4][7], wb[3][4];
    for (int i = 0; i < 4; i++)
        for (int b = 0; b < 7; b++) wi[i][b] = lagrange_w(7, 3 + 2 * i, b);
    for (int i = 0; i < 3; i++)
        for (int b = 0; b < 4; b++) wb[i][b] = lagrange_w(4, 1 + 2 * i, b);
    cudaError_t e = cudaMemcpyToSymbol(c_wi, wi, sizeof(wi));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_wb, wb, sizeof(wb));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(wavelet_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kWvSmemBytes);
    int dev = 0, sms = 0, occ = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, wavelet_kernel, kWvWarps * 32,
                                                          kWvSmemBytes);
    if (e == cudaSuccess) g_wavelet_cap = std::max(1, sms) * std::max(1, occ);
    return e;
}

// Persistent: as many CTAs as fit on the device at once.
int wavelet_grid(uint64_t nleaves)
{
    const uint64_t per_cta = (uint64_t)kWvWarps * kBatch;
    return (int)std::min<uint64_t>((nleaves + per_cta - 1) / per_cta, (uint64_t)g_wavelet_cap);
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
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = wavelet_configure();
    if (e == cudaSuccess && changed)
        e = cudaMemsetAsync(changed, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess && nleaves) {
        wavelet_kernel<<<wavelet_grid(nleaves), kWvWarps * 32, kWvSmemBytes, st>>>(a);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        set_error(std::string("dgb_remesh_wavelets: ") + cudaGetErrorString(e));
        return DGB_ERR_CUDA;
    }
    return DGB_OK;
}
