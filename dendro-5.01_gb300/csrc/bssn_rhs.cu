// Persistent, work-queued launch of the BSSN right-hand side over all blocks
// of a plan (unzipped fields); the per-tile work is rhs_item (rhs_item.cuh).
#include "rhs_kernel.cuh"

namespace dgb {

// 8x8x16 (variant 5): the deep tile halves the z halo and the mixed-derivative
// boxes' z extension per interior point; at 100 KB of shared memory it still
// fits 2 CTAs per SM in FP64 (not in mixed precision, nor with the gather
// indices of the fused stepper); 2 % faster than 8^3 on the uneven batch.
// 7x13x13 (variant 6, 107 KB in FP64) covers the 13^3 and 25^3 interiors of the
// octree's 19^3 and 31^3 blocks in 2 and 16 tiles instead of 4 and 32; it is
// the FP64 default (the autotuner's choice for every block class of the uneven
// batch and of the octree, 1 % faster than 8x8x16 on the former, 6 % on the
// latter's RK4 step; a 9x9x13 variant was never chosen and was dropped).
// 7x7x13 (variant 7) is the deep tile that fits 2 CTAs per SM in mixed
// precision (96 KB; the autotuner's choice on the octree).
const TileShape kTileShapes[] = {{8, 8, 8},  {7, 7, 7},   {8, 8, 4}, {16, 8, 4},
                                 {6, 6, 6},  {8, 8, 16},  {7, 13, 13}, {7, 7, 13}};
const int kNumTileShapes = sizeof(kTileShapes) / sizeof(kTileShapes[0]);
static_assert(sizeof(kTileShapes) / sizeof(kTileShapes[0]) <= kMaxTileShapes, "too many tile shapes");
const int kDefaultVariantFp64 = 6;

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
    return launch_any<false>(variant, precision == DGB_PREC_MIXED, args, grid, stream);
}

cudaError_t rhs_configure(int variant, int precision)
{
    return configure_any<false>(variant, precision == DGB_PREC_MIXED);
}

int rhs_max_ctas_per_sm(int variant, int precision)
{
    return occupancy_any<false>(variant, precision == DGB_PREC_MIXED);
}

}  // namespace dgb
