// Persistent, work-queued launch of the BSSN right-hand side over all blocks
// of a plan; the per-tile work is rhs_item (rhs_item.cuh).
#include "rhs_item.cuh"

namespace dgb {

const TileShape kTileShapes[] = {{8, 8, 8}, {7, 7, 7}, {8, 8, 4}, {16, 8, 4}, {6, 6, 6}};
const int kNumTileShapes = sizeof(kTileShapes) / sizeof(kTileShapes[0]);

namespace {

template <int TX, int TY, int TZ, bool MIXED>
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
        rhs_item<TX, TY, TZ, MIXED>(args, w, blk, S, aprm);
    }
}

template <int TX, int TY, int TZ, bool MIXED>
cudaError_t launch_variant(const RhsArgs &args, int grid, cudaStream_t stream)
{
    const size_t smem = Smem<TX, TY, TZ, MIXED>::bytes;
    rhs_kernel<TX, TY, TZ, MIXED><<<grid, kThreads, smem, stream>>>(args);
    return cudaGetLastError();
}

template <int TX, int TY, int TZ, bool MIXED>
cudaError_t configure_variant()
{
    const size_t smem = Smem<TX, TY, TZ, MIXED>::bytes;
    return cudaFuncSetAttribute(rhs_kernel<TX, TY, TZ, MIXED>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int TX, int TY, int TZ, bool MIXED>
int occupancy_variant()
{
    int n = 0;
    const size_t smem = Smem<TX, TY, TZ, MIXED>::bytes;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rhs_kernel<TX, TY, TZ, MIXED>, kThreads,
                                                      smem) != cudaSuccess)
        return 0;
    return n;
}

#define DGB_DISPATCH(VARIANT, MIXEDV, CALL)                                     \
    switch (VARIANT) {                                                          \
    case 0: return MIXEDV ? CALL<8, 8, 8, true>() : CALL<8, 8, 8, false>();     \
    case 1: return MIXEDV ? CALL<7, 7, 7, true>() : CALL<7, 7, 7, false>();     \
    case 2: return MIXEDV ? CALL<8, 8, 4, true>() : CALL<8, 8, 4, false>();     \
    case 3: return MIXEDV ? CALL<16, 8, 4, true>() : CALL<16, 8, 4, false>();   \
    case 4: return MIXEDV ? CALL<6, 6, 6, true>() : CALL<6, 6, 6, false>();     \
    default: break;                                                             \
    }

}  // namespace

size_t rhs_smem_bytes(int variant, int precision)
{
    const TileShape t = kTileShapes[variant];
    const size_t fb = (size_t)(t.tx + 6) * (t.ty + 6) * (t.tz + 6);
    const size_t bx = (size_t)t.tx * (t.ty + 6) * (t.tz + 6) + (size_t)t.tx * t.ty * (t.tz + 6);
    return precision == DGB_PREC_MIXED ? 2 * fb * 8 + 2 * fb * 4 + 2 * bx * 4 : 2 * fb * 8 + bx * 8;
}

int rhs_threads(int) { return kThreads; }

size_t rhs_scratch_per_cta(int variant)
{
    const TileShape t = kTileShapes[variant];
    return (size_t)DGB_NUM_SLOTS * t.tx * t.ty * t.tz;
}

cudaError_t rhs_launch(int variant, int precision, const RhsArgs &args, int grid,
                       cudaStream_t stream)
{
    const bool mixed = precision == DGB_PREC_MIXED;
    switch (variant) {
    case 0: return mixed ? launch_variant<8, 8, 8, true>(args, grid, stream) : launch_variant<8, 8, 8, false>(args, grid, stream);
    case 1: return mixed ? launch_variant<7, 7, 7, true>(args, grid, stream) : launch_variant<7, 7, 7, false>(args, grid, stream);
    case 2: return mixed ? launch_variant<8, 8, 4, true>(args, grid, stream) : launch_variant<8, 8, 4, false>(args, grid, stream);
    case 3: return mixed ? launch_variant<16, 8, 4, true>(args, grid, stream) : launch_variant<16, 8, 4, false>(args, grid, stream);
    case 4: return mixed ? launch_variant<6, 6, 6, true>(args, grid, stream) : launch_variant<6, 6, 6, false>(args, grid, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t rhs_configure(int variant, int precision)
{
    const bool mixed = precision == DGB_PREC_MIXED;
    DGB_DISPATCH(variant, mixed, configure_variant)
    return cudaErrorInvalidValue;
}

int rhs_max_ctas_per_sm(int variant, int precision)
{
    const bool mixed = precision == DGB_PREC_MIXED;
    if (rhs_configure(variant, precision) != cudaSuccess) return 0;
    DGB_DISPATCH(variant, mixed, occupancy_variant)
    return 0;
}

}  // namespace dgb
