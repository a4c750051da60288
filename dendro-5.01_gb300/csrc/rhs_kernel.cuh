// The persistent, work-queued RHS kernel and its launch helpers, templated
// on the tile shape, the precision and the gather (fused unzip) mode.
#pragma once
#include "rhs_item.cuh"

namespace dgb {
namespace {

template <int TX, int TY, int TZ, bool MIXED, bool GATHER>
__global__ void __launch_bounds__(kThreads, kMinBlocks) rhs_kernel(const RhsArgs args)
{
    using G = Geo<TX, TY, TZ>;
    __shared__ int s_item;
    const int tid = threadIdx.x;
    double *S = args.scratch + (size_t)blockIdx.x * DGB_NUM_SLOTS * G::PMAX;
    const AlgPrm aprm{args.prm.l1, args.prm.l2, args.prm.l3, args.prm.l4, args.prm.lf0,
                      args.prm.lf1};

    for (;;) {
        __syncthreads();  // previous item fully consumed s_item / shared buffers
        if (tid == 0) s_item = (int)atomicAdd(args.queue, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= (int)args.nitems) break;
        const WorkItem w = args.items[it];
        const DevBlock blk = args.blocks[w.blk];
        rhs_item<TX, TY, TZ, MIXED, GATHER>(args, w, blk, S, aprm);
    }
}

template <int TX, int TY, int TZ, bool MIXED, bool GATHER>
cudaError_t launch_variant(const RhsArgs &args, int grid, cudaStream_t stream)
{
    const size_t smem = Smem<TX, TY, TZ, MIXED, GATHER>::bytes;
    rhs_kernel<TX, TY, TZ, MIXED, GATHER><<<grid, kThreads, smem, stream>>>(args);
    return cudaGetLastError();
}

template <int TX, int TY, int TZ, bool MIXED, bool GATHER>
cudaError_t configure_variant()
{
    const size_t smem = Smem<TX, TY, TZ, MIXED, GATHER>::bytes;
    return cudaFuncSetAttribute(rhs_kernel<TX, TY, TZ, MIXED, GATHER>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int TX, int TY, int TZ, bool MIXED, bool GATHER>
int occupancy_variant()
{
    int n = 0;
    const size_t smem = Smem<TX, TY, TZ, MIXED, GATHER>::bytes;
    if (configure_variant<TX, TY, TZ, MIXED, GATHER>() != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rhs_kernel<TX, TY, TZ, MIXED, GATHER>,
                                                      kThreads, smem) != cudaSuccess)
        return 0;
    return n;
}

// dispatch over the compiled tile shapes (kTileShapes order)
template <bool GATHER>
cudaError_t launch_any(int variant, bool mixed, const RhsArgs &a, int grid, cudaStream_t st)
{
    switch (variant) {
    case 0: return mixed ? launch_variant<8, 8, 8, true, GATHER>(a, grid, st) : launch_variant<8, 8, 8, false, GATHER>(a, grid, st);
    case 1: return mixed ? launch_variant<7, 7, 7, true, GATHER>(a, grid, st) : launch_variant<7, 7, 7, false, GATHER>(a, grid, st);
    case 2: return mixed ? launch_variant<8, 8, 4, true, GATHER>(a, grid, st) : launch_variant<8, 8, 4, false, GATHER>(a, grid, st);
    case 3: return mixed ? launch_variant<16, 8, 4, true, GATHER>(a, grid, st) : launch_variant<16, 8, 4, false, GATHER>(a, grid, st);
    case 4: return mixed ? launch_variant<6, 6, 6, true, GATHER>(a, grid, st) : launch_variant<6, 6, 6, false, GATHER>(a, grid, st);
    case 5: return mixed ? launch_variant<8, 8, 16, true, GATHER>(a, grid, st) : launch_variant<8, 8, 16, false, GATHER>(a, grid, st);
    case 6: return mixed ? launch_variant<7, 13, 13, true, GATHER>(a, grid, st) : launch_variant<7, 13, 13, false, GATHER>(a, grid, st);
    case 7: return mixed ? launch_variant<7, 7, 13, true, GATHER>(a, grid, st) : launch_variant<7, 7, 13, false, GATHER>(a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

template <bool GATHER>
cudaError_t configure_any(int variant, bool mixed)
{
    switch (variant) {
    case 0: return mixed ? configure_variant<8, 8, 8, true, GATHER>() : configure_variant<8, 8, 8, false, GATHER>();
    case 1: return mixed ? configure_variant<7, 7, 7, true, GATHER>() : configure_variant<7, 7, 7, false, GATHER>();
    case 2: return mixed ? configure_variant<8, 8, 4, true, GATHER>() : configure_variant<8, 8, 4, false, GATHER>();
    case 3: return mixed ? configure_variant<16, 8, 4, true, GATHER>() : configure_variant<16, 8, 4, false, GATHER>();
    case 4: return mixed ? configure_variant<6, 6, 6, true, GATHER>() : configure_variant<6, 6, 6, false, GATHER>();
    case 5: return mixed ? configure_variant<8, 8, 16, true, GATHER>() : configure_variant<8, 8, 16, false, GATHER>();
    case 6: return mixed ? configure_variant<7, 13, 13, true, GATHER>() : configure_variant<7, 13, 13, false, GATHER>();
    case 7: return mixed ? configure_variant<7, 7, 13, true, GATHER>() : configure_variant<7, 7, 13, false, GATHER>();
    default: return cudaErrorInvalidValue;
    }
}

template <bool GATHER>
int occupancy_any(int variant, bool mixed)
{
    switch (variant) {
    case 0: return mixed ? occupancy_variant<8, 8, 8, true, GATHER>() : occupancy_variant<8, 8, 8, false, GATHER>();
    case 1: return mixed ? occupancy_variant<7, 7, 7, true, GATHER>() : occupancy_variant<7, 7, 7, false, GATHER>();
    case 2: return mixed ? occupancy_variant<8, 8, 4, true, GATHER>() : occupancy_variant<8, 8, 4, false, GATHER>();
    case 3: return mixed ? occupancy_variant<16, 8, 4, true, GATHER>() : occupancy_variant<16, 8, 4, false, GATHER>();
    case 4: return mixed ? occupancy_variant<6, 6, 6, true, GATHER>() : occupancy_variant<6, 6, 6, false, GATHER>();
    case 5: return mixed ? occupancy_variant<8, 8, 16, true, GATHER>() : occupancy_variant<8, 8, 16, false, GATHER>();
    case 6: return mixed ? occupancy_variant<7, 13, 13, true, GATHER>() : occupancy_variant<7, 13, 13, false, GATHER>();
    case 7: return mixed ? occupancy_variant<7, 7, 13, true, GATHER>() : occupancy_variant<7, 7, 13, false, GATHER>();
    default: return 0;
    }
}

}  // namespace
}  // namespace dgb
