// BSSN right-hand side of one block with no allocation at all.
//
// Some callers cannot call cudaMalloc where they need the right-hand side:
// a solver that has reserved nearly all device memory for its own pool (the
// unzipped and zipped state of a large mesh) and forbids further
// allocations, a host runtime that owns the device allocator and does not
// allow direct cudaMalloc, or a time-step loop that must not pay the
// device-wide synchronisation of cudaMalloc/cudaFree.  For them this file
// keeps the derivative workspace of the RHS kernel in a fixed array compiled
// into the library; the caller passes only the field arrays (inputs) and the
// right-hand-side arrays (outputs), both in device memory.
//
// The kernel is the per-tile RHS of rhs_item.cuh (the same code the
// plan-based, persistent launch runs) with one CTA per 6^3 tile and each CTA
// on its own slice of the fixed workspace, so a block may need at most
// DGB_NOALLOC_MAX_TILES tiles; larger blocks are rejected.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "rhs_item.cuh"

namespace dgb {
namespace {

constexpr int kNaT = 6;  // tile side
using NaGeo = Geo<kNaT, kNaT, kNaT>;
constexpr size_t kNaSlice = (size_t)DGB_NUM_SLOTS * NaGeo::PMAX;  // doubles per CTA

// The fixed workspace: DGB_NOALLOC_MAX_TILES slices of 162 x 216 doubles
// (64 MiB in all).  Every device that loads the library holds it until the
// process exits.  Every call shares it and it keeps the last call's contents;
// nothing in it needs to start at zero (each CTA writes every slot of its
// slice before reading it), and two calls that overlap on the GPU race on it.
static __device__ __align__(256) double g_noalloc_ws[(size_t)DGB_NOALLOC_MAX_TILES * kNaSlice];

constexpr int kMaxDevices = 64;
std::mutex g_ws_mutex;
double *g_ws_ptr[kMaxDevices] = {};

// Device address of the workspace on the current device, looked up once per
// device (the array's name is only a host-side stand-in in host code) and
// kept for the life of the process: after cudaDeviceReset the kept address
// belongs to a destroyed context, so the entry must not be used after one.
dgb_status workspace_on_current_device(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error("dgb_bssnrhs_block_noalloc: no current CUDA device");
        return DGB_ERR_NOT_INIT;
    }
    std::lock_guard<std::mutex> lock(g_ws_mutex);
    if (!g_ws_ptr[dev]) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_noalloc_ws);
        if (e != cudaSuccess || !p) {
            set_error(std::string("dgb_bssnrhs_block_noalloc: cudaGetSymbolAddress: ") +
                      cudaGetErrorString(e));
            return DGB_ERR_CUDA;
        }
        g_ws_ptr[dev] = p;
    }
    *out = g_ws_ptr[dev];
    return DGB_OK;
}

struct NaTiles {
    int n[3], base[3], rem[3];  // tiles per axis; extents base+1 for the first rem tiles
};

__global__ void __launch_bounds__(kThreads, kMinBlocks)
rhs_noalloc_kernel(const RhsArgs args, const DevBlock blk, const NaTiles t, double *ws)
{
    int it = blockIdx.x;
    WorkItem w;
    w.blk = 0;
    for (int a = 0; a < 3; a++) {
        const int q = it % t.n[a];
        it /= t.n[a];
        w.o[a] = (uint16_t)(q * t.base[a] + (q < t.rem[a] ? q : t.rem[a]));
        w.e[a] = (uint16_t)(t.base[a] + (q < t.rem[a] ? 1 : 0));
    }
    const AlgPrm aprm{args.prm.l1, args.prm.l2, args.prm.l3, args.prm.l4, args.prm.lf0,
                      args.prm.lf1};
    rhs_item<kNaT, kNaT, kNaT, false>(args, w, blk, ws + (size_t)blockIdx.x * kNaSlice, aprm);
}

}  // namespace
}  // namespace dgb

using namespace dgb;

extern "C" dgb_status dgb_bssnrhs_block_noalloc(double *const *rhs, const double *const *u,
                                                uint64_t offset, const double *ptmin,
                                                const double *ptmax, const uint32_t *sz,
                                                uint32_t bflag, const dgb_bssn_params *prm,
                                                void *stream)
{
    if (!rhs || !u || !ptmin || !ptmax || !sz || !prm) {
        set_error("dgb_bssnrhs_block_noalloc: null argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV; v++)
        if (!rhs[v] || !u[v]) {
            set_error("dgb_bssnrhs_block_noalloc: null field pointer");
            return DGB_ERR_INVALID;
        }
    if (bflag > 63u) {
        set_error("dgb_bssnrhs_block_noalloc: bflag has bits beyond the six faces");
        return DGB_ERR_INVALID;
    }
    if (prm->fd_order != 0 && prm->fd_order != 6) {
        set_error("dgb_bssnrhs_block_noalloc: the 6th-order binding only (fd_order 6 or 0)");
        return DGB_ERR_UNSUPPORTED;
    }
    if (prm->gauge != DGB_GAUGE_ETA_CONST) {
        set_error("dgb_bssnrhs_block_noalloc: only the constant-eta standard gauge is built");
        return DGB_ERR_UNSUPPORTED;
    }
    NaTiles t;
    DevBlock blk;
    long long ntiles = 1;
    for (int a = 0; a < 3; a++) {
        if (sz[a] < 7 || sz[a] > 4096) {
            set_error("dgb_bssnrhs_block_noalloc: each block side must be in [7, 4096]");
            return DGB_ERR_INVALID;
        }
        if (bflag != 0 && sz[a] < 13) {
            // the one-sided closures read interior points 3..8 from each flagged
            // face; with 13 or more points per side the 6^3 cut below gives tiles
            // of at least 3 points, whose 3-point halo holds those taps
            set_error("dgb_bssnrhs_block_noalloc: domain-boundary blocks need at least 13 "
                      "points per side");
            return DGB_ERR_INVALID;
        }
        const int m = (int)sz[a] - 6;
        t.n[a] = (m + kNaT - 1) / kNaT;
        t.base[a] = m / t.n[a];
        t.rem[a] = m % t.n[a];
        ntiles *= t.n[a];
        blk.sz[a] = sz[a];
        blk.pmin[a] = ptmin[a];
        blk.h[a] = (ptmax[a] - ptmin[a]) / (double)(sz[a] - 1);
        if (!(blk.h[a] > 0.0)) {
            set_error("dgb_bssnrhs_block_noalloc: ptmax must exceed ptmin");
            return DGB_ERR_INVALID;
        }
    }
    if (ntiles > DGB_NOALLOC_MAX_TILES) {
        set_error("dgb_bssnrhs_block_noalloc: the block needs " + std::to_string(ntiles) +
                  " tiles of 6^3 interior points but the fixed workspace holds " +
                  std::to_string(DGB_NOALLOC_MAX_TILES) +
                  " (largest cubic block: 42^3 padded points); use dgb_bssn_rhs for larger blocks");
        return DGB_ERR_INVALID;
    }
    blk.offset = offset;
    blk.bflag = bflag;
    double *ws = nullptr;
    dgb_status s = workspace_on_current_device(&ws);
    if (s != DGB_OK) return s;
    RhsArgs a{};
    for (int v = 0; v < NV; v++) {
        a.u[v] = u[v];
        a.rhs[v] = rhs[v];
    }
    a.blocks = nullptr;
    a.items = nullptr;
    a.nitems = (uint32_t)ntiles;
    a.queue = nullptr;
    a.scratch = ws;
    a.prm.l1 = prm->lambda[0]; a.prm.l2 = prm->lambda[1];
    a.prm.l3 = prm->lambda[2]; a.prm.l4 = prm->lambda[3];
    a.prm.lf0 = prm->lambda_f[0]; a.prm.lf1 = prm->lambda_f[1];
    a.prm.eta_const = prm->eta_const; a.prm.eta_r0 = prm->eta_r0;
    a.prm.eta_exp = prm->eta_damping_exp; a.prm.sigma = prm->ko_sigma;
    const size_t smem = Smem<kNaT, kNaT, kNaT, false>::bytes;  // below the 48 KB default
    rhs_noalloc_kernel<<<(unsigned)ntiles, kThreads, smem, (cudaStream_t)stream>>>(a, blk, t, ws);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("dgb_bssnrhs_block_noalloc: launch: ") + cudaGetErrorString(e));
        return DGB_ERR_CUDA;
    }
    return DGB_OK;
}
