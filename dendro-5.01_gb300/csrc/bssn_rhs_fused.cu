// The RHS kernels in gather mode for the fused unzip -> RHS step: tiles are
// staged from the zipped state (and the buffer of interpolated padded
// points) through per-point gather indices, and each RHS value goes
// straight to the zipped node its padded point owns.  No unzipped field
// set exists in this mode.
#include "rhs_kernel.cuh"

namespace dgb {

cudaError_t rhs_launch_gather(int variant, int precision, const RhsArgs &args, int grid,
                              cudaStream_t stream)
{
    const bool mixed = precision == DGB_PREC_MIXED;
    const cudaError_t e = configure_any<true>(variant, mixed);
    if (e != cudaSuccess) return e;
    return launch_any<true>(variant, mixed, args, grid, stream);
}

int rhs_max_ctas_per_sm_gather(int variant, int precision)
{
    return occupancy_any<true>(variant, precision == DGB_PREC_MIXED);
}

}  // namespace dgb
