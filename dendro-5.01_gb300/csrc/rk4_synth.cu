// RK4 stage update with the per-node BSSN constraint closure, and the
// device side of the synthetic fill.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dgb_internal.h"
#include "synth.cuh"

namespace dgb {
namespace {

struct Rk4Args {
    double *dst[NV];
    const double *prev[NV];
    const double *k[4 * NV];
    uint64_t n;
    double dt, chi_floor;
    int stage;
    unsigned int *status;
};

// RK4 tableau, BSSN_GR/include/rkBSSN.h:55-58.
__constant__ double c_rk4_c[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
__constant__ double c_rk4_u[4] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0};

// Stage sums as in RK_BSSN::performSingleIteration
// (BSSN_GR/src/rkBSSN.cpp:895-905, 996-1011), then enforce_bssn_constraints
// (BSSN_GR/src/bssn_constraints.cpp:12-172): gt /= det^(1/3), At trace
// removed with the rescaled metric, chi and alpha floored at chi_floor.
// det <= 0 (where the reference exits) raises bit 0 of *status.
__global__ void __launch_bounds__(256) rk4_kernel(const Rk4Args a)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t node = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; node < a.n; node += stride) {
        double x[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) {
            double s = a.prev[v][node];
            if (a.stage < 3) {
                s += c_rk4_u[a.stage + 1] * a.dt * a.k[a.stage * NV + v][node];
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++) s += c_rk4_c[q] * a.dt * a.k[q * NV + v][node];
            }
            x[v] = s;
        }
        // gt = x[12..17] (00,01,02,11,12,22), At = x[18..23]
        double g00 = x[12], g01 = x[13], g02 = x[14], g11 = x[15], g12 = x[16], g22 = x[17];
        double det = g00 * (g11 * g22 - g12 * g12) - g01 * g01 * g22 + 2.0 * g01 * g02 * g12
                   - g02 * g02 * g11;
        if (!(det > 0.0)) atomicOr(a.status, 1u);
        // det^(-1/3): the reference's 1 / pow(det, 1/3) as one reciprocal cube
        // root (within an ulp of it; the pow costs several times the rest of the node)
        const double sc = det < 0.0 ? __longlong_as_double(0x7ff8000000000000ll)  // as pow's NaN
                                    : rcbrt(det);
        g00 *= sc; g01 *= sc; g02 *= sc; g11 *= sc; g12 *= sc; g22 *= sc;
        det = g00 * (g11 * g22 - g12 * g12) - g01 * g01 * g22 + 2.0 * g01 * g02 * g12
            - g02 * g02 * g11;
        const double idet = 1.0 / det;
        const double u00 = idet * (g11 * g22 - g12 * g12);
        const double u01 = idet * (-g01 * g22 + g02 * g12);
        const double u02 = idet * (g01 * g12 - g02 * g11);
        const double u11 = idet * (g00 * g22 - g02 * g02);
        const double u12 = idet * (-g00 * g12 + g01 * g02);
        const double u22 = idet * (g00 * g11 - g01 * g01);
        const double tr3 = (1.0 / 3.0) * (x[18] * u00 + x[21] * u11 + x[23] * u22
                                          + 2.0 * (x[19] * u01 + x[20] * u02 + x[22] * u12));
        x[18] -= tr3 * g00; x[19] -= tr3 * g01; x[20] -= tr3 * g02;
        x[21] -= tr3 * g11; x[22] -= tr3 * g12; x[23] -= tr3 * g22;
        x[12] = g00; x[13] = g01; x[14] = g02; x[15] = g11; x[16] = g12; x[17] = g22;
        if (x[1] < a.chi_floor) x[1] = a.chi_floor;
        x[0] = (x[0] < a.chi_floor) ? a.chi_floor : x[0];
#pragma unroll
        for (int v = 0; v < NV; v++) a.dst[v][node] = x[v];
    }
}

struct SynthArgs {
    double *u[NV + 1];  // the 24 BSSN fields, or theta_z4 of the CCZ4 set at index 24
    int v0, v1;         // variables [v0, v1) are filled
    const DevBlock *blocks;
    uint32_t nblk;
    uint64_t seed;
    double noise;
};

// One CTA per block (grid-stride over blocks); same arithmetic as the host fill.
__global__ void __launch_bounds__(256) synth_kernel(const SynthArgs a)
{
    for (uint32_t b = blockIdx.x; b < a.nblk; b += gridDim.x) {
        const DevBlock d = a.blocks[b];
        const uint64_t n = (uint64_t)d.sz[0] * d.sz[1] * d.sz[2];
        for (int v = a.v0; v < a.v1; v++) {
            const uint64_t key = dgb_noise_key(a.seed, b, (uint32_t)v);
            double *dst = a.u[v] + d.offset;
            for (uint64_t p = threadIdx.x; p < n; p += blockDim.x) {
                const int i = (int)(p % d.sz[0]);
                const uint64_t r = p / d.sz[0];
                const int j = (int)(r % d.sz[1]);
                const int k = (int)(r / d.sz[1]);
                dst[p] = dgb_synth_value(v, key, p, i, j, k, d.pmin, d.h, a.noise);
            }
        }
    }
}

}  // namespace

cudaError_t rk4_launch(int stage, double *const *dst, const double *const *prev,
                       const double *const *k, uint64_t nnodes, double dt, double chi_floor,
                       unsigned int *status, cudaStream_t stream)
{
    Rk4Args a;
    for (int v = 0; v < NV; v++) {
        a.dst[v] = dst[v];
        a.prev[v] = prev[v];
    }
    for (int q = 0; q < 4 * NV; q++) a.k[q] = (q / NV <= stage) ? k[q] : nullptr;
    a.n = nnodes;
    a.dt = dt;
    a.chi_floor = chi_floor;
    a.stage = stage;
    a.status = status;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    uint64_t blocks = (nnodes + 255) / 256;
    const uint64_t cap = (uint64_t)nsm * 8;
    if (blocks > cap) blocks = cap;
    rk4_kernel<<<(unsigned)blocks, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t synth_fill_launch(const DevBlock *blocks, uint32_t nblk, const uint64_t *,
                              uint64_t, double *const *u, int v0, int v1, uint64_t seed,
                              double noise, cudaStream_t stream)
{
    SynthArgs a;
    for (int v = 0; v <= NV; v++) a.u[v] = (v >= v0 && v < v1) ? u[v - v0] : nullptr;
    a.v0 = v0;
    a.v1 = v1;
    a.blocks = blocks;
    a.nblk = nblk;
    a.seed = seed;
    a.noise = noise;
    const unsigned grid = nblk < 65535u ? nblk : 65535u;
    synth_kernel<<<grid, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace dgb
