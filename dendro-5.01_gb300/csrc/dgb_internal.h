// Internal declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/dendro_gb300.h"

namespace dgb {

constexpr int NV = DGB_NUM_VARS;

// Per-block data the kernels read (built once per plan).
struct DevBlock {
    uint64_t offset;
    uint32_t sz[3];
    uint32_t bflag;  // domain-boundary faces, bit 2a / 2a+1 = low / high side of axis a
    double pmin[3];
    double h[3];
};

// One unit of the persistent work queue: a rectangular tile of a block's
// interior.  o = tile origin in interior coordinates (padded index - 3),
// e = tile extents.
struct WorkItem {
    uint32_t blk;
    uint16_t o[3];
    uint16_t e[3];
};

// Runtime constants of the RHS (bssn:: globals).
struct RhsParams {
    double l1, l2, l3, l4, lf0, lf1;
    double eta_const, eta_r0, eta_exp, sigma;
};

struct RhsArgs {
    const double *u[NV];
    double *rhs[NV];
    const DevBlock *blocks;
    const WorkItem *items;
    uint32_t nitems;
    unsigned int *queue;   // work-queue head, zeroed before each launch
    double *scratch;       // per-CTA derivative workspace
    RhsParams prm;
    // gather mode (fused unzip) only: u = zipped fields, rhs = zipped outputs;
    // padded point gi reads u[v][gmap[gi]] when gmap[gi] < ndof, else
    // ib[v][gmap[gi] - ndof] (interpolated points); its RHS goes to
    // rhs[v][zmap[gi]] unless zmap[gi] = 0xFFFFFFFF (not the node's owner)
    const double *ib[NV];
    const uint32_t *gmap;
    const uint32_t *zmap;
    uint32_t ndof;
};

// Tile schedule: one compiled kernel variant per max tile shape.
struct TileShape {
    int tx, ty, tz;
};

// Compiled variants (index into kTileShapes).
extern const TileShape kTileShapes[];
extern const int kNumTileShapes;
constexpr int kMaxTileShapes = 10;  // capacity of the per-variant caches
extern const int kDefaultVariantFp64;  // the plan's FP64 variant unless set or tuned

size_t rhs_smem_bytes(int variant, int precision);
int rhs_threads(int variant);
size_t rhs_scratch_per_cta(int variant);  // doubles
cudaError_t rhs_launch(int variant, int precision, const RhsArgs &args, int grid,
                       cudaStream_t stream);
cudaError_t rhs_configure(int variant, int precision);
// the gather-mode (fused unzip) kernels, same variants
cudaError_t rhs_launch_gather(int variant, int precision, const RhsArgs &args, int grid,
                              cudaStream_t stream);
int rhs_max_ctas_per_sm_gather(int variant, int precision);
// the gather-mode RHS over a plan (dgb_api.cu)
// changes whenever a work-item buffer of the plan is freed (see dgb_rk4_step)
uint64_t plan_items_gen(const dgb_plan *p);
dgb_status run_rhs_gather(dgb_plan *p, double *const *k, const double *const *z,
                          const double *const *ib, const uint32_t *gmap, const uint32_t *zmap,
                          uint32_t ndof, int precision, cudaStream_t st);
int rhs_max_ctas_per_sm(int variant, int precision);

cudaError_t rk4_launch(int stage, double *const *dst, const double *const *prev,
                       const double *const *k, uint64_t nnodes, double dt, double chi_floor,
                       unsigned int *status, cudaStream_t stream);

// fills variables [v0, v1) (v1 <= 25; index 24 = theta_z4 of the CCZ4 set);
// u[q] is the array of variable v0 + q
cudaError_t synth_fill_launch(const DevBlock *blocks, uint32_t nblk, const uint64_t *first_pt,
                              uint64_t total, double *const *u, int v0, int v1, uint64_t seed,
                              double noise, cudaStream_t stream);

// CCZ4 right-hand side (ccz4_rhs.cu): 25 variables, CCZ4_GR/include/grUtils.h:46.
constexpr int NV4 = 25;
struct C4Params {
    double l1, l2, l3, l4, lf0, lf1, k1, k2, p;
    double eta_const, eta_r0, eta_exp, sigma;
};
struct C4Args {
    const double *u[NV4];
    double *rhs[NV4];
    const DevBlock *blocks;
    const WorkItem *items;   // the 8x8x8 schedule (tile variant 0)
    uint32_t nitems;
    unsigned int *queue;
    double *scratch;
    C4Params prm;
};
// BSSN right-hand side with the BSSN_GR 4th-order binding (bssn42_rhs.cu);
// the RhsArgs fields of the 6th-order kernel, 8x8x8 schedule, FP64.
size_t b4_smem_bytes();
size_t b4_scratch_per_cta();  // doubles
cudaError_t b4_configure();
int b4_max_ctas_per_sm();
cudaError_t b4_launch(const RhsArgs &args, int grid, cudaStream_t stream);

size_t c4_smem_bytes(int precision);
size_t c4_scratch_per_cta();  // doubles
cudaError_t c4_configure(int precision);
int c4_max_ctas_per_sm(int precision);
cudaError_t c4_launch(int precision, const C4Args &args, int grid, cudaStream_t stream);

// Constraint diagnostics (physcon.cu).
struct PcArgs {
    const double *u[NV];
    double *cons[DGB_NUM_CONSTRAINTS];
    const DevBlock *blocks;
    const WorkItem *items;   // the 8x8x8 schedule (tile variant 0)
    uint32_t nitems;
    unsigned int *queue;
    double *scratch;
};
size_t physcon_smem_bytes();
size_t physcon_scratch_per_cta();  // doubles
int physcon_threads();
cudaError_t physcon_configure();
int physcon_max_ctas_per_sm();
cudaError_t physcon_launch(const PcArgs &args, int grid, cudaStream_t stream);

struct NormArgs {
    const double *f[DGB_NUM_CONSTRAINTS];
    int nvars;
    const double *mask;      // may be null: every node counts
    double threshold;
    uint64_t ndof;
    double *partial;         // norm_partials() x (DGB_NUM_CONSTRAINTS + 1) doubles
};
int norm_partials();
cudaError_t l2_norm_launch(const NormArgs &a, double *out_dev, cudaStream_t stream);

void set_error(const std::string &msg);

}  // namespace dgb
