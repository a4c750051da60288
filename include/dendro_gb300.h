/*
 * dendro_gb300.h — C ABI of the GB300 (sm_103a) BSSN per-step hot path.
 *
 * Plain pointers and sizes only.  Every entry point returns a dgb_status and
 * never aborts; dgb_last_error() gives the message of the last failure on
 * the calling thread.  A plan is not thread-safe; distinct plans on distinct
 * streams are independent.
 *
 * Field layout (identical to the reference's unzipped vectors): 24 separate
 * arrays, one per evolved variable in the order of bssn::VAR
 * (BSSN_GR/include/grDef.h:31): alpha, chi, K, Gt0..2, beta0..2, B0..2,
 * gt00,01,02,11,12,22, At00,01,02,11,12,22.  Block b occupies
 * [offset_b, offset_b + sz0*sz1*sz2) of each array, x fastest
 * (IDX(i,j,k) = i + sz0*(j + sz1*k), BSSN_GR/include/rhs.h:21).
 */
#ifndef DENDRO_GB300_H
#define DENDRO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGB_NUM_VARS 24
/* constraint diagnostics, bssn::VAR_CONSTRAINT order (BSSN_GR/include/grDef.h):
 * ham, mom0, mom1, mom2, psi4_real, psi4_img */
#define DGB_NUM_CONSTRAINTS 6

typedef enum {
    DGB_OK = 0,
    DGB_ERR_INVALID = 1,     /* bad argument, size or block descriptor */
    DGB_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    DGB_ERR_ALLOC = 3,       /* device or pinned allocation failed */
    DGB_ERR_NOT_INIT = 4,    /* dgb_init not called / no device */
    DGB_ERR_TIMEOUT = 5,     /* reserved: no entry of this build waits on the device with a
                                bound, so none returns it */
    DGB_ERR_NONFINITE = 6,   /* NaN/Inf found by a checking entry point */
    DGB_ERR_CONSTRAINT = 7,  /* det(gt) <= 0 in the RK constraint step */
    DGB_ERR_UNSUPPORTED = 8  /* valid request this build does not implement */
} dgb_status;

enum { DGB_PREC_FP64 = 0, DGB_PREC_MIXED = 1 };

/* One padded octant block; what bssnRHS derives per block from ot::Block
 * (BSSN_GR/src/rhs.cpp:45-62): getOffset(), getAllocationSz{X,Y,Z}(),
 * getBlkNodeFlag(), ptmin = corner - 3dx, ptmax = corner + 3dx. */
typedef struct {
    uint64_t offset;
    uint32_t sz[3];
    uint32_t bflag;
    double ptmin[3];
    double ptmax[3];
} dgb_block_desc;

/* The bssn:: globals the RHS and the RK update read
 * (BSSN_GR/include/parameters.h; defaults BSSN_GR/src/parameters.cpp). */
typedef struct {
    double lambda[4];        /* BSSN_LAMBDA (integers in the reference) */
    double lambda_f[2];      /* BSSN_LAMBDA_F */
    double eta_const;        /* ETA_CONST */
    double eta_r0;           /* ETA_R0 */
    double eta_damping_exp;  /* ETA_DAMPING_EXP */
    double ko_sigma;         /* KO_DISS_SIGMA */
    double chi_floor;        /* CHI_FLOOR */
    /* Finite-difference binding of the right-hand side: 6 (or 0) = the
     * QuadGrav 6th-order one (QuadGrav/include/derivs.h:80-97: deriv64,
     * centred advective derivative, ko_deriv42); 4 = the BSSN_GR solver's own
     * (BSSN_GR/include/rhs.h:23-37: deriv42, upwinded deriv42adv, ko_deriv42),
     * FP64 only and not in the fused-unzip stepper. */
    int fd_order;
    /* Gauge / eta variant of the generated equations (BSSN_GR/src/rhs.cpp:
     * 226-246): DGB_GAUGE_ETA_CONST (0, the default build's
     * bssneqs_eta_const_standard_gauge.cpp) is the one built; the others
     * (USE_ETA_FUNC, USE_ROCHESTER_GAUGE builds) are refused with
     * DGB_ERR_UNSUPPORTED at dgb_plan_create. */
    int gauge;
} dgb_bssn_params;
#define DGB_GAUGE_ETA_CONST 0           /* standard gauge, constant eta */
#define DGB_GAUGE_ETA_FUNC 1            /* standard gauge, eta function (USE_ETA_FUNC) */
#define DGB_GAUGE_ROCHESTER_ETA_CONST 2 /* USE_ROCHESTER_GAUGE */
#define DGB_GAUGE_ROCHESTER_ETA_FUNC 3  /* USE_ROCHESTER_GAUGE + USE_ETA_FUNC */

typedef struct dgb_plan dgb_plan;

/* Library / device set-up.  Replaces the CUDA context set-up the reference
 * does inside cuda::computeRHS (BSSN_GR/cuda_gr/src/rhs_cuda.cu:12-133). */
dgb_status dgb_init(int device);
const char *dgb_last_error(void);
int dgb_version(void);

/* Block list -> device plan (descriptors, work items, tile schedule,
 * workspace).  Replaces the per-call block partitioning and workspace
 * allocation of cuda::computeRHS (rhs_cuda.cu:35-133). */
dgb_status dgb_plan_create(const dgb_block_desc *blocks, size_t nblk,
                           const dgb_bssn_params *prm, dgb_plan **plan);
dgb_status dgb_plan_destroy(dgb_plan *plan);
/* Number of padded points sum_b sz0*sz1*sz2 (length of each field array). */
uint64_t dgb_plan_unzipped_size(const dgb_plan *plan);
uint64_t dgb_plan_interior_points(const dgb_plan *plan);

/* bssnRHS over all blocks of the plan, DEVICE pointers, on `stream`
 * (a cudaStream_t, 0 = legacy default).  Replaces
 * void bssnRHS(double**, const double**, const ot::Block*, unsigned)
 * (BSSN_GR/include/rhs.h:45, BSSN_GR/src/rhs.cpp:9-76).  Writes only the
 * interior points of each block of rhs[v]; padding is left untouched.
 * precision: DGB_PREC_FP64 (drop-in) or DGB_PREC_MIXED (FP32 stencils/KO). */
dgb_status dgb_bssn_rhs(dgb_plan *plan, double *const *rhs, const double *const *u,
                        int precision, void *stream);

/* Same call with HOST arrays (the reference's calling convention): copies the
 * fields in, computes, writes the interior of rhs back, synchronously; the
 * padding of rhs is left untouched.  Fields that lie in memory from
 * dgb_host_alloc may be uploaded straight from the caller's arrays; others go
 * through the library's pinned staging.  When the upload goes through the
 * staging and rhs lies in dgb_host_alloc memory, the kernel stores the
 * interior points into rhs over the host link as it runs; otherwise they are
 * downloaded and written back by host threads (except the last chunk's, which
 * the kernel stores when rhs lies in dgb_host_alloc memory).  The first call
 * builds the plan's pipeline: device slots for three chunks of fields each
 * way and a second derivative workspace for overlapping chunk kernels. */
dgb_status dgb_bssn_rhs_host(dgb_plan *plan, double *const *rhs, const double *const *u,
                             int precision);

/* Page-locked host memory for the caller's unzipped field arrays (the
 * reference allocates them with new[] in Mesh::createUnZippedVector,
 * include/mesh.tcc:245-262).  The host-array entries (dgb_bssn_rhs_host,
 * dgb_ccz4_rhs_host, dgb_physical_constraints_host) may upload input fields
 * that lie entirely inside one such allocation without the host-side staging
 * copy, and store into outputs that do (see dgb_bssn_rhs_host).  Thread-safe. */
dgb_status dgb_host_alloc(size_t bytes, void **ptr);
dgb_status dgb_host_free(void *ptr);

/* One block, host arrays: replaces bssnrhs(double**, const double**,
 * const unsigned& offset, const double* ptmin, const double* ptmax,
 * const unsigned* sz, const unsigned& bflag) (BSSN_GR/include/rhs.h:47-50,
 * BSSN_GR/src/rhs.cpp:86-392). */
dgb_status dgb_bssnrhs_block_host(double *const *rhs, const double *const *u,
                                  uint64_t offset, const double *ptmin, const double *ptmax,
                                  const uint32_t *sz, uint32_t bflag,
                                  const dgb_bssn_params *prm, int precision);

/* One block, DEVICE arrays, and no allocation of any kind.  No counterpart
 * in the reference (it allocates 210 scratch arrays per block call,
 * BSSN_GR/scripts/bssnrhs_memalloc.h); it exists for callers that cannot
 * call cudaMalloc where they need the right-hand side: a solver whose
 * device memory is fully reserved by its own pool, a host runtime that owns
 * the device allocator, or a time-step loop that must not pay the
 * device-wide synchronisation of cudaMalloc/cudaFree.  The derivative
 * workspace is a fixed array inside the library (DGB_NOALLOC_MAX_TILES
 * slices, 64 MiB, held on every device that loads the library until exit),
 * so a block may span at most DGB_NOALLOC_MAX_TILES tiles of 6^3 interior
 * points (a cube of at most 42^3 padded points); larger blocks are rejected
 * with DGB_ERR_INVALID.  Interior and domain-boundary blocks (bflag != 0:
 * at least 13 points per side, bflag <= 63).  FP64 and the 6th-order
 * binding only (fd_order 4 and the other gauges are refused with
 * DGB_ERR_UNSUPPORTED); same results as dgb_bssn_rhs.  The first call on a
 * device looks up the workspace's device address and keeps it for the life
 * of the process; make that first call before any stream capture, and do
 * not call this entry after cudaDeviceReset on that device (the kept address
 * belongs to the context the reset destroyed).  All calls share the
 * workspace: calls that overlap on the GPU (other streams, other threads)
 * race on it.  The launch is asynchronous on `stream`. */
#define DGB_NOALLOC_MAX_TILES 239
dgb_status dgb_bssnrhs_block_noalloc(double *const *rhs, const double *const *u,
                                     uint64_t offset, const double *ptmin, const double *ptmax,
                                     const uint32_t *sz, uint32_t bflag,
                                     const dgb_bssn_params *prm, void *stream);

/* Autotuner: for every compiled kernel variant (maximum tile) and every
 * block-size class of the plan (sizes, and whether the block touches a domain
 * face), times each candidate tile cap on the caller's device buffers; keeps
 * the variant whose per-class best caps give the shortest total, and those
 * caps.  Optional; the chosen schedule is used by every BSSN RHS entry of the
 * plan until the next autotune or dgb_plan_set_tile_variant. */
dgb_status dgb_plan_autotune(dgb_plan *plan, double *const *rhs, const double *const *u,
                             int precision, void *stream);
/* The per-class tile caps the autotuner chose: count classes; when rows is not
 * NULL, up to cap rows of 7 values (sx, sy, sz, touches-a-face, cap_x, cap_y,
 * cap_z). */
dgb_status dgb_plan_class_tiles(const dgb_plan *plan, int precision, uint32_t *rows, size_t cap,
                                size_t *count);
/* Current maximum tile extents (out: tx,ty,tz) of the schedule chosen for
 * `precision`; every block is cut into the fewest tiles within them. */
dgb_status dgb_plan_tile(const dgb_plan *plan, int precision, uint32_t *tile3);
/* Compiled tile schedules: count, and explicit choice (bypasses autotune and
 * clears its per-class caps). */
int dgb_num_tile_variants(void);
dgb_status dgb_plan_set_tile_variant(dgb_plan *plan, int precision, int variant);

/* The ccz4:: globals ccz4rhs reads (CCZ4_GR/include/parameters.h):
 * CCZ4_LAMBDA, CCZ4_LAMBDA_F, CCZ4_KAPPA, P_EXPO, ETA_*, KO_DISS_SIGMA. */
typedef struct {
    double lambda[4];
    double lambda_f[2];
    double kappa[2];
    double p_expo;
    double eta_const;
    double eta_r0;
    double eta_damping_exp;
    double ko_sigma;
} dgb_ccz4_params;
#define DGB_CCZ4_NUM_VARS 25

/* CCZ4 right-hand side over every block of a plan, device pointers:
 * replaces the per-block loop over ccz4rhs (CCZ4_GR/src/rhs.cpp:12-298,
 * called from CCZ4_GR/src/rk4CCZ4.cpp:498/584).  rhs and u are 25 arrays in
 * CCZ4 variable order (alpha, psi, K, Gh0-2, beta0-2, B0-2, gt0-5, At0-5,
 * theta_z4, CCZ4_GR/include/grUtils.h:46); interior points are written,
 * padding untouched.  The CCZ4 solver's 4th-order stencils (upwind advective
 * derivatives, its KO form), ccz4_bcs on flagged faces, KO on every variable
 * but theta_z4.  DGB_PREC_MIXED: FP32 (compensated) stencils on interior
 * blocks, FP64 everywhere else.  The plan's block list is used; its BSSN
 * parameters are not.  Asynchronous on
 * `stream`; calls on one plan must be ordered on one stream. */
dgb_status dgb_ccz4_rhs(dgb_plan *plan, const dgb_ccz4_params *prm, double *const *rhs,
                        const double *const *u, int precision, void *stream);
/* Same call with HOST arrays (the reference's calling convention, 25 fields
 * each way): the chunked pipeline of dgb_bssn_rhs_host (host gather, upload,
 * kernel, download and scatter of the interior points overlapped);
 * synchronous; the padding of rhs is left untouched. */
dgb_status dgb_ccz4_rhs_host(dgb_plan *plan, const dgb_ccz4_params *prm, double *const *rhs,
                             const double *const *u, int precision);

/* Constraint diagnostics over every block of a plan, device pointers:
 * replaces the per-block loop over physical_constraints (BSSN_GR/src/physcon.cpp:12-96,
 * called from BSSN_GR/src/bssnCtx.cpp:332-355 and rkBSSN.cpp:1659).
 * cons[0..5] = ham, mom0, mom1, mom2, psi4_real, psi4_img are written at each
 * block's interior points (padding untouched) from the 24 unzipped fields
 * u; 4th-order stencils with one-sided closures on flagged faces, FP64.
 * Asynchronous on `stream`; shares the plan's work queue and workspace with
 * dgb_bssn_rhs, so calls on one plan must be ordered on one stream. */
dgb_status dgb_physical_constraints(dgb_plan *plan, double *const *cons, const double *const *u,
                                    void *stream);
/* Same call with HOST arrays (24 fields in, 6 out), through the chunked
 * pipeline of the host-array RHS entries; synchronous; only interior points
 * of the outputs are written. */
dgb_status dgb_physical_constraints_host(dgb_plan *plan, double *const *cons,
                                         const double *const *u);
/* Masked RMS of nvars (<= DGB_NUM_CONSTRAINTS) zipped device vectors of
 * ndof values: sqrt(sum c^2 / count) over the nodes whose mask value is not
 * below threshold (mask may be NULL: every node counts).  Replaces
 * computeConstraintL2Norm (BSSN_GR/include/grUtils.tcc:40-88) on one rank.
 * Deterministic reduction order; synchronises `stream`; out is host memory. */
dgb_status dgb_constraint_l2(const double *const *fields, int nvars, const double *mask,
                             double threshold, uint64_t ndof, double *out, void *stream);

/* RK4 stage update on zipped (CG) vectors with the per-node constraint
 * closure, device pointers.  stage 0..2: dst = prev + U[s+1] dt k[s];
 * stage 3: dst = prev + sum_s C[s] dt k[s]; then enforce_bssn_constraints.
 * k is 4 x 24 pointers (only k[0..stage] are read).  Replaces the node loops
 * of RK_BSSN::performSingleIteration (BSSN_GR/src/rkBSSN.cpp:895-905,
 * 996-1011) and enforce_bssn_constraints (BSSN_GR/src/bssn_constraints.cpp). */
dgb_status dgb_rk4_stage(int stage, double *const *dst, const double *const *prev,
                         const double *const *k, uint64_t nnodes, double dt,
                         double chi_floor, void *stream);

/* Seeded synthetic Brill-Lindquist + U(-1,1)*noise fields at every padded
 * point of every block (host or device memory).  Host and device fill give
 * identical bits. */
dgb_status dgb_synth_fill_host(const dgb_block_desc *blocks, size_t nblk,
                               double *const *u, uint64_t seed, double noise, int nthreads);
dgb_status dgb_synth_fill_device(dgb_plan *plan, double *const *u, uint64_t seed,
                                 double noise, void *stream);
/* One variable of the synthetic set, var in [0, 24]: the 24 BSSN fields,
 * or 24 = theta_z4 of the CCZ4 set (value 0 + noise).  The CCZ4 state is
 * the 24 BSSN fields (psi takes chi's values, Gh takes Gt's) plus var 24. */
dgb_status dgb_synth_fill_var_host(const dgb_block_desc *blocks, size_t nblk, int var,
                                   double *dst, uint64_t seed, double noise, int nthreads);
dgb_status dgb_synth_fill_var_device(dgb_plan *plan, int var, double *dst, uint64_t seed,
                                     double noise, void *stream);
/* Synthetic block lists.  which = 1: 512 uniform 13^3 blocks, dx = 0.05,
 * tiled 8x8x8 over [-1.2,1.2]^3; which = 2: 20,000 blocks, 70/20/8/2 % of
 * 13^3/19^3/31^3/61^3, levels 4-10 on [-32,32]^3.  Pass blocks == NULL to
 * get the count. */
dgb_status dgb_synth_blocks(int which, uint64_t seed, dgb_block_desc *blocks, size_t *nblk);

/* ------------------------------------------------------------------------
 * Octree mesh, unzip / zip and the full RK4 step
 * ------------------------------------------------------------------------ */

/* Synthetic 2:1-balanced octree on a cubic domain, refined to max_level
 * within fine_radius of each puncture and one level coarser per doubling of
 * the distance, down to min_level.  Host-side; replaces the mesh the
 * reference builds in ot::Mesh (src/mesh.cpp:283).  With max_block_refine =
 * -1 the leaves are ordered, grouped into blocks and numbered as the
 * reference's mesh does: elements in its Hilbert order, blocks of
 * octree2BlockDecomposition (src/octUtils.cpp:556-741) in the same order with
 * the same offsets and face flags (src/mesh.cpp:8640-8790), the CG vector in
 * the order of Mesh::buildE2NMap (src/mesh.cpp:3895-3960), zip from each
 * node's owning element.  max_block_refine = 0..3 instead groups maximal
 * aligned cubes of up to 2^max_block_refine leaves per side (not the
 * reference's blocks; same element order and CG numbering rule). */
typedef struct {
    double domain_min[3], domain_max[3];
    int max_level, min_level, ele_order; /* ele_order must be 6 */
    int num_punctures;
    double puncture[4][3];
    double fine_radius;
    int max_block_refine; /* -1 (the reference's blocks) or 0..3 */
    /* The reference's octree depth (m_uiMaxDepth, BSSN_MAXDEPTH in its
     * parameter files): its block decomposition depends on it (volumes of
     * 2^32 octree units or more are never one block); max_level + 3..30 (the
     * reference needs leaves of at least 8 octree units, where the 7 nodes of
     * an order-6 element fall on distinct integer positions), or 0 for
     * max_level + 4. */
    int octree_depth;
} dgb_mesh_params;
typedef struct dgb_mesh dgb_mesh;
dgb_status dgb_mesh_create(const dgb_mesh_params *prm, dgb_mesh **mesh);
dgb_status dgb_mesh_destroy(dgb_mesh *mesh);
/* sizes[0..6]: leaves, independent nodes (zipped length), blocks, padded
 * points (unzipped length), interpolation rows, source elements, source
 * levels. */
dgb_status dgb_mesh_sizes(const dgb_mesh *mesh, uint64_t *sizes);
dgb_status dgb_mesh_blocks(const dgb_mesh *mesh, dgb_block_desc *blocks);
dgb_status dgb_mesh_dof_coords(const dgb_mesh *mesh, double *xyz);
dgb_status dgb_mesh_leaf_levels(const dgb_mesh *mesh, uint8_t *level, uint32_t *anchor);
/* The element order's space-filling curve: per state s (nstates of them),
 * order[8s + i] = the child (x | y << 1 | z << 2) visited i-th and
 * next[8s + c] = child c's state; state 0 at the root.  Any pointer may be
 * NULL.  The reference holds the same curve as tables (src/hcurvedata.cpp). */
dgb_status dgb_mesh_hilbert_tables(uint8_t *order, uint8_t *next, int *nstates);
/* The mesh's unzip / zip operators in the form dgb_unzip_plan_create takes
 * (array lengths from dgb_mesh_sizes; src_refs holds 343 per source). */
dgb_status dgb_mesh_unzip_operator(const dgb_mesh *mesh, uint32_t *copy_src, uint64_t *interp_dst,
                                   uint64_t *interp_ref, uint64_t *src_refs, uint64_t *level_ptr,
                                   uint64_t *zip_src);
/* Per leaf of the mesh (dgb_mesh_sizes()[0] entries each; any pointer may be
 * NULL): patch_base = first point of the leaf's 13^3 padded patch in the
 * unzipped vector (its 7^3 nodes and 3 padding points per side,
 * Mesh::getUnzipElementalNodalValues, include/mesh.tcc:9136-9176);
 * block_side = side of its block's padded grid; boundary = 1 when the leaf
 * touches the domain boundary (Mesh::isBoundaryOctant, include/mesh.h:1482-1486);
 * corner = its minimum corner (3 per leaf) and hx = its node spacing, domain
 * units: the arguments isReMeshUnzip passes its wavelet_tol callback
 * (include/mesh.tcc:2090-2099). */
dgb_status dgb_mesh_leaf_patches(const dgb_mesh *mesh, uint64_t *patch_base, uint32_t *block_side,
                                 uint8_t *boundary, double *corner, double *hx);

/* ---- wavelet refinement indicator (Mesh::isReMeshUnzip) ---------------- */
/* Refinement flags (OCT_NO_CHANGE, OCT_SPLIT, OCT_COARSE, include/mesh.h:108-110) */
#define DGB_OCT_NO_CHANGE 0u
#define DGB_OCT_SPLIT 1u
#define DGB_OCT_COARSE 2u
#define DGB_OCT_INVALID 255u /* leaf patch outside the unzipped vector */
#define DGB_WAVELET_MAX_VARS 32

/* Wavelet tolerance per leaf from its corner (host arrays): the radial ramp
 * of bssn::computeWTol (BSSN_GR/src/grUtils.cpp:1869-1891),
 * min(tol_max, max(tol_min, (tol_max - tol_min) / (r1 - r0) * (r - r0) + tol_min))
 * with r = |corner| in domain coordinates when use_function, else tol_min. */
dgb_status dgb_wavelet_tol_radial(const double *corner, uint64_t nleaves, double tol_min,
                                  double tol_max, double r0, double r1, int use_function,
                                  double *tol);

/* Replaces the indicator of Mesh::isReMeshUnzip (include/mesh.tcc:2035-2197;
 * wavelets of WaveletEl::compute_wavelets_3D, src/waveletRefEl.cpp:92-271),
 * element order 6.  unzipped: host array of device pointers (all fields of
 * unzip_len points), var_ids: host array of nvars (1..DGB_WAVELET_MAX_VARS)
 * refinement variables.  Per leaf (device arrays of nleaves, as
 * dgb_mesh_leaf_patches gives them, tol from the wavelet_tol callback):
 * wmax = the largest RMS wavelet over the variables, stopping at the first
 * variable that passes tol (eleWMax); flags = DGB_OCT_SPLIT if wmax > tol,
 * DGB_OCT_COARSE if wmax < coarse_fac * tol, else DGB_OCT_NO_CHANGE;
 * DGB_OCT_INVALID (wmax NaN) for a leaf whose patch does not fit.  changed
 * (device, may be NULL): number of leaves flagged split or coarse, the
 * reference's isMeshLocalChanged.  Asynchronous on stream. */
dgb_status dgb_remesh_wavelets(const double *const *unzipped, const uint32_t *var_ids, int nvars,
                               uint64_t unzip_len, uint64_t nleaves, const uint64_t *patch_base,
                               const uint32_t *block_side, const uint8_t *boundary,
                               const double *tol, double coarse_fac, double *wmax, uint8_t *flags,
                               unsigned long long *changed, void *stream);

/* Device unzip / zip for any mesh, from its operator.  A node reference is
 * a 64-bit word: bit 63 clear = the zipped node in the low 32 bits; bit 63
 * set = the degree-6 Lagrange interpolant of source element (bits 12..42)
 * at local position codes (bits 0..11, 4 bits per axis x,y,z, code = 2*xi,
 * xi in [0,6] in node spacings).  Source elements are elements whose 343
 * nodal values (src_refs, x fastest) some reference interpolates from, the
 * way Mesh::getElementNodalValues (include/mesh.tcc:2467) rebuilds hanging
 * nodes; they are grouped by refinement level, coarsest first
 * (level_ptr[l]..level_ptr[l+1]), and a reference may only name a source of
 * an earlier group.  Padded point p copies zipped node copy_src[p]
 * (0xFFFFFFFF: not a copy), or, for the rows interp_dst[r], takes
 * interp_ref[r]; zipped node d reads padded point zip_src[d].  A maintainer
 * builds the operator once per mesh from ot::Mesh's maps: its element-to-node
 * map and hanging-node parents (include/mesh.h:1152-1161) and its block list. */
typedef struct dgb_unzip_plan dgb_unzip_plan;
dgb_status dgb_unzip_plan_create(uint64_t ndof, uint64_t unzipped_size, const uint32_t *copy_src,
                                 uint64_t ninterp, const uint64_t *interp_dst,
                                 const uint64_t *interp_ref, uint64_t nsrc,
                                 const uint64_t *src_refs, uint64_t nlevels,
                                 const uint64_t *level_ptr, const uint64_t *zip_src,
                                 dgb_unzip_plan **plan);
dgb_status dgb_unzip_plan_destroy(dgb_unzip_plan *plan);
/* Replaces ot::Mesh::unzip(const T* in, T* out, unsigned dof) for nvars
 * fields (include/mesh.h:1697, include/mesh.tcc:7436-8690), device arrays. */
dgb_status dgb_unzip(dgb_unzip_plan *plan, const double *const *zipped, double *const *unzipped,
                     int nvars, void *stream);
/* Replaces ot::Mesh::zip(const T* unzipped, T* zipped) (include/mesh.h:1740,
 * include/mesh.tcc:3775-3822), device arrays. */
dgb_status dgb_zip(dgb_unzip_plan *plan, const double *const *unzipped, double *const *zipped,
                   int nvars, void *stream);

/* Full RK4 step on the zipped state (24 device arrays of the plan's ndof),
 * in place: for each stage, unzip -> bssnRHS (+KO, boundary conditions) ->
 * zip -> stage update with the constraint closure; the four stages of one
 * step are one CUDA graph, captured on the first call and replayed.
 * Replaces RK_BSSN::performSingleIteration's RK4 branch
 * (BSSN_GR/src/rkBSSN.cpp:603-1012).  The stepper owns its stage buffers and,
 * unless fused (DGB_STEP_FUSED_UNZIP below), the unzipped field set. */
typedef struct dgb_stepper dgb_stepper;
dgb_status dgb_stepper_create(dgb_plan *rhs_plan, dgb_unzip_plan *uz, int precision,
                              dgb_stepper **stepper);
/* flags: DGB_STEP_FUSED_UNZIP = the fused unzip -> RHS step: no unzipped
 * field set is held; the RHS kernel stages its tiles from the zipped state
 * (and a compact buffer of the interpolated padded points) through a gather
 * index per padded point and writes each value to the zipped node its
 * padded point owns.  Same results as the unfused stepper, bit for bit; 8
 * bytes per padded point of maps instead of 2 x 24 x 8 bytes of fields. */
#define DGB_STEP_FUSED_UNZIP 1u
dgb_status dgb_stepper_create_ex(dgb_plan *rhs_plan, dgb_unzip_plan *uz, int precision,
                                 unsigned flags, dgb_stepper **stepper);
/* Device memory the stepper itself holds (bytes). */
dgb_status dgb_stepper_device_bytes(const dgb_stepper *stepper, uint64_t *bytes);
dgb_status dgb_stepper_destroy(dgb_stepper *stepper);
dgb_status dgb_rk4_step(dgb_stepper *stepper, double *const *state, double dt, double chi_floor,
                        int nsteps, void *stream);

/* Seeded Brill-Lindquist + noise at arbitrary points (zipped vectors);
 * noise keyed by (seed, point index, variable). */
dgb_status dgb_synth_fill_points_host(const double *xyz, uint64_t n, double *const *u,
                                      uint64_t seed, double noise, int nthreads);

/* Measured FP64 FMA throughput of the current device (GFLOP/s, 2 per FMA)
 * and the probe kernel's time: the roofline denominator of the FP64-bound
 * RHS.  No reference counterpart (measurement support). */
dgb_status dgb_measure_fp64_peak(double *gflops, double *ms);

/* Self-test of the integer-pipe exact tap products used by the FP64
 * stencils: mismatches against the IEEE multiply over n pseudo-random
 * doubles (host when on_device == 0, else the current device).  No
 * reference counterpart (test support). */
dgb_status dgb_selftest_exact_mul(int on_device, uint64_t n, uint64_t seed,
                                  uint64_t *mismatches);

#ifdef __cplusplus
}
#endif
#endif /* DENDRO_GB300_H */
