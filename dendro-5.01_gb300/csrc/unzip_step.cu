// Device unzip / zip from a mesh operator, and the full RK4 step as one CUDA
// graph per step.
//
// unzip (per call, for nvars fields):
//   1. source elements, one launch per refinement level, coarsest first: the
//      343 nodal values of every element something interpolates from, each a
//      zipped-node copy or (a hanging node) an interpolation from a coarser
//      source element;
//   2. copies: one thread per padded point, all fields per thread;
//   3. interpolated padded points: one thread per row, the separable degree-6
//      Lagrange sum over one source element (1, 7, 49 or 343 terms).
// zip: one gather per independent node.  All HBM/L2-bound; the RK4 step
// around them is  for s in 0..3: unzip(prev or im) -> bssnRHS -> zip ->
// stage update  (BSSN_GR/src/rkBSSN.cpp:803-1012), captured once and replayed.
//
// Fused mode (DGB_STEP_FUSED_UNZIP): no unzipped field set.  Per stage only
// the source elements (1) and the interpolated points (3, into a compact
// buffer, one row per interpolated padded point) are materialised; the RHS
// kernel stages its tiles from the zipped state and that buffer through a
// per-padded-point gather index and writes each RHS value straight to the
// zipped node its padded point owns (the zip), so steps 2 and the zip
// disappear, and with them 2 x 24 x 8 bytes per padded point of device memory.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "dgb_internal.h"

namespace dgb {
namespace {

constexpr uint32_t kSentinel = 0xFFFFFFFFu;
constexpr uint64_t kInterp = 1ull << 63;
constexpr int kNpe = 343;

struct FieldPtrs {
    const double *in[NV];
    double *out[NV];
    int nvars;
};

// 1-D Lagrange weights at xi = code/2 for the odd codes 1, 3, ..., 11
struct LagTable {
    double w[6][7];
};

__device__ __forceinline__ int axis_terms(uint32_t code, const LagTable &T, double *w, int *idx)
{
    if ((code & 1u) == 0) {
        w[0] = 1.0;
        idx[0] = (int)(code >> 1);
        return 1;
    }
    const int r = (int)(code >> 1);
#pragma unroll
    for (int i = 0; i < 7; i++) {
        w[i] = T.w[r][i];
        idx[i] = i;
    }
    return 7;
}

// Value of reference ref for field v (zipped array z, source table dg).
__device__ __forceinline__ double ref_value(uint64_t ref, const double *__restrict__ z,
                                            const double *__restrict__ dg, const LagTable &T)
{
    if (!(ref & kInterp)) return __ldg(z + (uint32_t)ref);
    const uint64_t src = (ref >> 12) & 0x7FFFFFFFull;
    double wx[7], wy[7], wz[7];
    int ix[7], iy[7], iz[7];
    const int nx = axis_terms((uint32_t)(ref & 0xF), T, wx, ix);
    const int ny = axis_terms((uint32_t)((ref >> 4) & 0xF), T, wy, iy);
    const int nz = axis_terms((uint32_t)((ref >> 8) & 0xF), T, wz, iz);
    const double *e = dg + src * kNpe;
    double acc = 0.0;
    for (int c = 0; c < nz; c++) {
        double accy = 0.0;
        for (int b = 0; b < ny; b++) {
            const double *row = e + 7 * (iy[b] + 7 * iz[c]);
            double accx = 0.0;
            for (int a = 0; a < nx; a++) accx = fma(wx[a], row[ix[a]], accx);
            accy = fma(wy[b], accx, accy);
        }
        acc = fma(wz[c], accy, acc);
    }
    return acc;
}

struct DgArgs {
    const double *z[NV];
    double *dg[NV];
    int nvars;
    const uint64_t *refs;
    uint64_t first, count;  // source range of this level
    LagTable T;
};

__global__ void __launch_bounds__(256) dg_fill_kernel(const DgArgs a)
{
    const uint64_t n = a.count * kNpe;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += stride) {
        const uint64_t slot = a.first * kNpe + t;
        const uint64_t ref = __ldg(a.refs + slot);
        for (int v = 0; v < a.nvars; v++) a.dg[v][slot] = ref_value(ref, a.z[v], a.dg[v], a.T);
    }
}

__global__ void __launch_bounds__(256) unzip_copy_kernel(const FieldPtrs f, const uint32_t *__restrict__ src,
                                                         uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += stride) {
        const uint32_t s = __ldg(src + p);
        if (s == kSentinel) continue;
        // all loads before the stores: 24 independent reads in flight per
        // thread (out and in are not known not to alias)
        double val[NV];
#pragma unroll
        for (int v = 0; v < NV; v++)
            if (v < f.nvars) val[v] = __ldg(f.in[v] + s);
#pragma unroll
        for (int v = 0; v < NV; v++)
            if (v < f.nvars) f.out[v][p] = val[v];
    }
}

// Interpolated padded points grouped by source element: one CTA refines a
// source element onto its 13^3 half-lattice (codes 0..12 per axis) with three
// separable passes in shared memory (x, then y, then z: the same operations
// in the same order as ref_value, so the values are bit-identical), then
// scatters the rows of that source.
struct GroupArgs {
    FieldPtrs f;
    const double *dg[NV];
    const uint64_t *gptr;   // nsrc + 1
    const uint64_t *gdst;   // destinations grouped by source
    const uint16_t *gcode;  // cx + 13 * (cy + 13 * cz)
    uint64_t nsrc;
    LagTable T;
    bool compact;           // write row r to out[v][r] (fused mode) instead of out[v][gdst[r]]
};

__device__ __forceinline__ double pass1(const double *in, int code, int stride, const LagTable &T)
{
    if ((code & 1) == 0) return in[(code >> 1) * stride];
    const double *w = T.w[code >> 1];
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < 7; a++) acc = fma(w[a], in[a * stride], acc);
    return acc;
}

__global__ void __launch_bounds__(256) unzip_group_kernel(const GroupArgs a)
{
    __shared__ double e[kNpe];            // [k][j][i]
    __shared__ double A[7 * 7 * 13];      // [k][j][cx]
    __shared__ double B[7 * 13 * 13];     // [k][cy][cx]
    __shared__ double Cc[13 * 13 * 13];   // [cz][cy][cx]
    for (uint64_t s = blockIdx.x; s < a.nsrc; s += gridDim.x) {
        const uint64_t r0 = a.gptr[s], r1 = a.gptr[s + 1];
        if (r0 == r1) continue;
        for (int v = 0; v < a.f.nvars; v++) {
            __syncthreads();
            for (int t = threadIdx.x; t < kNpe; t += blockDim.x) e[t] = a.dg[v][s * kNpe + t];
            __syncthreads();
            for (int t = threadIdx.x; t < 7 * 7 * 13; t += blockDim.x) {
                const int cx = t % 13, jk = t / 13;
                A[t] = pass1(e + 7 * jk, cx, 1, a.T);
            }
            __syncthreads();
            for (int t = threadIdx.x; t < 7 * 13 * 13; t += blockDim.x) {
                const int cx = t % 13, cy = (t / 13) % 13, k = t / 169;
                B[t] = pass1(A + (k * 7) * 13 + cx, cy, 13, a.T);
            }
            __syncthreads();
            for (int t = threadIdx.x; t < 13 * 13 * 13; t += blockDim.x) {
                const int cxy = t % 169, cz = t / 169;
                Cc[t] = pass1(B + cxy, cz, 169, a.T);
            }
            __syncthreads();
            for (uint64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
                a.f.out[v][a.compact ? r : a.gdst[r]] = Cc[a.gcode[r]];
        }
    }
}

__global__ void __launch_bounds__(256) zip_kernel(const FieldPtrs f, const uint64_t *__restrict__ src,
                                                  uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t d = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; d < n; d += stride) {
        const uint64_t s = __ldg(src + d);
        double val[NV];
#pragma unroll
        for (int v = 0; v < NV; v++)
            if (v < f.nvars) val[v] = __ldg(f.in[v] + s);
#pragma unroll
        for (int v = 0; v < NV; v++)
            if (v < f.nvars) f.out[v][d] = val[v];
    }
}

// Fused mode's maps.  gmap[p]: the zipped node a padded point copies, or
// ndof + r for the r-th interpolated row (grouped order), or ndof + ninterp
// (a zero row) for points beyond the domain faces; zmap[p]: the zipped node
// whose value is read from padded point p by the zip, or kSentinel.
__global__ void gmap_copy_kernel(uint32_t *gmap, const uint32_t *__restrict__ copy, uint64_t n,
                                 uint32_t outside)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += stride) {
        const uint32_t c = copy[p];
        gmap[p] = c == kSentinel ? outside : c;
    }
}

__global__ void gmap_interp_kernel(uint32_t *gmap, const uint64_t *__restrict__ gdst, uint64_t n,
                                   uint32_t ndof)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += stride)
        gmap[gdst[r]] = ndof + (uint32_t)r;
}

__global__ void zmap_kernel(uint32_t *zmap, const uint64_t *__restrict__ zip, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t d = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; d < n; d += stride)
        zmap[zip[d]] = (uint32_t)d;
}

unsigned grid_for(uint64_t n, int threads)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    uint64_t g = (n + threads - 1) / threads;
    const uint64_t cap = (uint64_t)nsm * 16;
    if (g > cap) g = cap;
    if (g == 0) g = 1;
    return (unsigned)g;
}

// Uniform-node Lagrange basis on 0..6 (the reference's interpolation matrices
// come from a Vandermonde solve on the same nodes, FEM/src/refel.cpp:84-170).
LagTable lagrange_table()
{
    LagTable T;
    for (int r = 0; r < 6; r++) {
        const double xi = r + 0.5;
        for (int i = 0; i < 7; i++) {
            double num = 1.0, den = 1.0;
            for (int m = 0; m < 7; m++) {
                if (m == i) continue;
                num *= (xi - m);
                den *= (double)(i - m);
            }
            T.w[r][i] = num / den;
        }
    }
    return T;
}

}  // namespace
}  // namespace dgb

using namespace dgb;

struct dgb_unzip_plan {
    uint64_t ndof = 0, nunz = 0, ninterp = 0, nsrc = 0;
    std::vector<uint64_t> level_ptr;
    uint32_t *d_copy = nullptr;
    uint64_t *d_srefs = nullptr, *d_zip = nullptr;
    uint64_t *d_gptr = nullptr, *d_gdst = nullptr;  // interpolated rows grouped by source
    uint16_t *d_gcode = nullptr;
    double *d_dg = nullptr;  // nsrc * 343 * 24 source nodal values
    LagTable T;
};

struct dgb_stepper {
    dgb_plan *plan = nullptr;
    dgb_unzip_plan *uz = nullptr;
    int precision = 0;
    bool fused = false;
    double *d_U = nullptr, *d_R = nullptr, *d_k = nullptr, *d_im = nullptr;
    uint32_t *d_gmap = nullptr, *d_zmap = nullptr;  // fused mode
    double *d_ib = nullptr;                         // fused mode: NV x (ninterp + 1)
    uint64_t device_bytes = 0;
    unsigned int *d_status = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t exec = nullptr;
    const double *key_state[NV] = {};
    double key_dt = 0.0, key_floor = 0.0;
    uint64_t key_items = 0;  // plan_items_gen of the plan(s) at capture
};

namespace {

#define DGB_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                   \
            return DGB_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

// step 1: the source elements' nodal values, coarsest level first
dgb_status fill_sources(dgb_unzip_plan *p, const double *const *zipped, int nvars, cudaStream_t st)
{
    if (!p->nsrc) return DGB_OK;
    DgArgs a;
    for (int v = 0; v < NV; v++) {
        a.z[v] = v < nvars ? zipped[v] : nullptr;
        a.dg[v] = p->d_dg + (size_t)v * p->nsrc * kNpe;
    }
    a.nvars = nvars;
    a.refs = p->d_srefs;
    a.T = p->T;
    for (size_t l = 0; l + 1 < p->level_ptr.size(); l++) {
        a.first = p->level_ptr[l];
        a.count = p->level_ptr[l + 1] - p->level_ptr[l];
        if (!a.count) continue;
        dg_fill_kernel<<<grid_for(a.count * kNpe, 256), 256, 0, st>>>(a);
        DGB_CUDA(cudaGetLastError());
    }
    return DGB_OK;
}

// step 3: the interpolated padded points, to their padded positions or (compact)
// to rows 0..ninterp-1 of out in grouped order
dgb_status interp_rows(dgb_unzip_plan *p, double *const *out, int nvars, bool compact,
                       cudaStream_t st)
{
    if (!p->ninterp) return DGB_OK;
    GroupArgs a;
    a.f.nvars = nvars;
    for (int v = 0; v < NV; v++) {
        a.f.in[v] = nullptr;
        a.f.out[v] = v < nvars ? out[v] : nullptr;
        a.dg[v] = p->d_dg + (size_t)v * p->nsrc * kNpe;
    }
    a.gptr = p->d_gptr;
    a.gdst = p->d_gdst;
    a.gcode = p->d_gcode;
    a.nsrc = p->nsrc;
    a.T = p->T;
    a.compact = compact;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t grid = p->nsrc < (uint64_t)nsm * 8 ? p->nsrc : (uint64_t)nsm * 8;
    unzip_group_kernel<<<(unsigned)grid, 256, 0, st>>>(a);
    DGB_CUDA(cudaGetLastError());
    return DGB_OK;
}

dgb_status do_unzip(dgb_unzip_plan *p, const double *const *zipped, double *const *unzipped,
                    int nvars, cudaStream_t st)
{
    dgb_status r = fill_sources(p, zipped, nvars, st);
    if (r != DGB_OK) return r;
    FieldPtrs f;
    f.nvars = nvars;
    for (int v = 0; v < NV; v++) {
        f.in[v] = v < nvars ? zipped[v] : nullptr;
        f.out[v] = v < nvars ? unzipped[v] : nullptr;
    }
    if (p->nunz) {
        unzip_copy_kernel<<<grid_for(p->nunz, 256), 256, 0, st>>>(f, p->d_copy, p->nunz);
        DGB_CUDA(cudaGetLastError());
    }
    return interp_rows(p, unzipped, nvars, false, st);
}

dgb_status do_zip(dgb_unzip_plan *p, const double *const *unzipped, double *const *zipped,
                  int nvars, cudaStream_t st)
{
    FieldPtrs f;
    f.nvars = nvars;
    for (int v = 0; v < NV; v++) {
        f.in[v] = v < nvars ? unzipped[v] : nullptr;
        f.out[v] = v < nvars ? zipped[v] : nullptr;
    }
    if (p->ndof) {
        zip_kernel<<<grid_for(p->ndof, 256), 256, 0, st>>>(f, p->d_zip, p->ndof);
        DGB_CUDA(cudaGetLastError());
    }
    return DGB_OK;
}

// The four stages of one RK4 step on stream st.
dgb_status enqueue_step(dgb_stepper *s, double *const *state, double dt, double chi_floor,
                        cudaStream_t st)
{
    const uint64_t nu = s->uz->nunz, nd = s->uz->ndof;
    double *U[NV], *R[NV], *IM[NV];
    const double *K[4 * NV];
    for (int v = 0; v < NV; v++) {
        U[v] = s->d_U ? s->d_U + (size_t)v * nu : nullptr;
        R[v] = s->d_R ? s->d_R + (size_t)v * nu : nullptr;
        IM[v] = s->d_im + (size_t)v * nd;
        for (int q = 0; q < 4; q++) K[q * NV + v] = s->d_k + ((size_t)q * NV + v) * nd;
    }
    double *IB[NV];
    const uint64_t nib = s->uz->ninterp + 1;
    for (int v = 0; v < NV; v++) IB[v] = s->d_ib ? s->d_ib + (size_t)v * nib : nullptr;
    for (int stage = 0; stage < 4; stage++) {
        const double *const *src = stage == 0 ? (const double *const *)state : (const double *const *)IM;
        double *KS[NV];
        for (int v = 0; v < NV; v++) KS[v] = (double *)K[stage * NV + v];
        if (s->fused) {
            dgb_status r = fill_sources(s->uz, src, NV, st);
            if (r == DGB_OK) r = interp_rows(s->uz, IB, NV, true, st);
            if (r == DGB_OK)
                r = run_rhs_gather(s->plan, KS, src, (const double *const *)IB, s->d_gmap,
                                   s->d_zmap, (uint32_t)nd, s->precision, st);
            if (r != DGB_OK) return r;
        } else {
            dgb_status r = do_unzip(s->uz, src, U, NV, st);
            if (r != DGB_OK) return r;
            r = dgb_bssn_rhs(s->plan, R, U, s->precision, st);
            if (r != DGB_OK) return r;
            r = do_zip(s->uz, R, KS, NV, st);
            if (r != DGB_OK) return r;
        }
        DGB_CUDA(rk4_launch(stage, stage < 3 ? IM : state, (const double *const *)state, K, nd, dt,
                            chi_floor, s->d_status, st));
    }
    return DGB_OK;
}

bool ref_ok(uint64_t ref, uint64_t ndof, uint64_t src_limit)
{
    if (!(ref & kInterp)) return ref < ndof;
    if (((ref >> 12) & 0x7FFFFFFFull) >= src_limit) return false;
    if (ref & 0x7FFFF80000000000ull) return false;  // bits 43..62 unused
    for (int a = 0; a < 3; a++)
        if (((ref >> (4 * a)) & 0xF) > 12) return false;
    return true;
}

}  // namespace

extern "C" {

dgb_status dgb_unzip_plan_create(uint64_t ndof, uint64_t unzipped_size, const uint32_t *copy_src,
                                 uint64_t ninterp, const uint64_t *interp_dst,
                                 const uint64_t *interp_ref, uint64_t nsrc,
                                 const uint64_t *src_refs, uint64_t nlevels,
                                 const uint64_t *level_ptr, const uint64_t *zip_src,
                                 dgb_unzip_plan **out)
{
    if (!out || (unzipped_size && !copy_src) || (ndof && !zip_src) ||
        (ninterp && (!interp_dst || !interp_ref)) || (nsrc && (!src_refs || !level_ptr))) {
        set_error("dgb_unzip_plan_create: null argument");
        return DGB_ERR_INVALID;
    }
    if (ndof >= kSentinel || nsrc >= (1ull << 31)) {
        set_error("dgb_unzip_plan_create: operator too large for its encoding");
        return DGB_ERR_INVALID;
    }
    // validate the operator so the kernels cannot read or write out of range,
    // and sources are only read after they are filled
    for (uint64_t p = 0; p < unzipped_size; p++)
        if (copy_src[p] != kSentinel && copy_src[p] >= ndof) {
            set_error("dgb_unzip_plan_create: copy source out of range");
            return DGB_ERR_INVALID;
        }
    if (nsrc && (level_ptr[0] != 0 || level_ptr[nlevels] != nsrc)) {
        set_error("dgb_unzip_plan_create: level_ptr must span the sources");
        return DGB_ERR_INVALID;
    }
    for (uint64_t l = 0; nsrc && l < nlevels; l++) {
        if (level_ptr[l + 1] < level_ptr[l]) return DGB_ERR_INVALID;
        for (uint64_t t = level_ptr[l] * kNpe; t < level_ptr[l + 1] * kNpe; t++)
            if (!ref_ok(src_refs[t], ndof, level_ptr[l])) {
                set_error("dgb_unzip_plan_create: a source element reads an unfilled source");
                return DGB_ERR_INVALID;
            }
    }
    for (uint64_t r = 0; r < ninterp; r++)
        if (interp_dst[r] >= unzipped_size || !ref_ok(interp_ref[r], ndof, nsrc)) {
            set_error("dgb_unzip_plan_create: bad interpolation row");
            return DGB_ERR_INVALID;
        }
    for (uint64_t d = 0; d < ndof; d++)
        if (zip_src[d] >= unzipped_size) {
            set_error("dgb_unzip_plan_create: zip source out of range");
            return DGB_ERR_INVALID;
        }
    dgb_unzip_plan *p = new dgb_unzip_plan();
    p->ndof = ndof;
    p->nunz = unzipped_size;
    p->ninterp = ninterp;
    p->nsrc = nsrc;
    if (nsrc) p->level_ptr.assign(level_ptr, level_ptr + nlevels + 1);
    p->T = lagrange_table();
    cudaError_t e = cudaSuccess;
    auto up = [&](void **dst, const void *src, size_t bytes) {
        if (e != cudaSuccess || bytes == 0) return;
        e = cudaMalloc(dst, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    };
    up((void **)&p->d_copy, copy_src, unzipped_size * 4);
    up((void **)&p->d_zip, zip_src, ndof * 8);
    up((void **)&p->d_srefs, src_refs, nsrc * kNpe * 8);
    if (e == cudaSuccess && nsrc) e = cudaMalloc(&p->d_dg, nsrc * kNpe * NV * sizeof(double));
    if (ninterp) {
        // group the interpolated rows by source element (counting sort)
        std::vector<uint64_t> gptr(nsrc + 1, 0), gdst(ninterp);
        std::vector<uint16_t> gcode(ninterp);
        for (uint64_t r = 0; r < ninterp; r++) gptr[((interp_ref[r] >> 12) & 0x7FFFFFFFull) + 1]++;
        for (uint64_t s = 0; s < nsrc; s++) gptr[s + 1] += gptr[s];
        std::vector<uint64_t> fill(gptr.begin(), gptr.end() - 1);
        for (uint64_t r = 0; r < ninterp; r++) {
            const uint64_t ref = interp_ref[r];
            const uint64_t s = (ref >> 12) & 0x7FFFFFFFull;
            const uint64_t q = fill[s]++;
            gdst[q] = interp_dst[r];
            gcode[q] = (uint16_t)((ref & 0xF) + 13 * (((ref >> 4) & 0xF) + 13 * ((ref >> 8) & 0xF)));
        }
        up((void **)&p->d_gptr, gptr.data(), gptr.size() * 8);
        up((void **)&p->d_gdst, gdst.data(), gdst.size() * 8);
        up((void **)&p->d_gcode, gcode.data(), gcode.size() * 2);
    }
    if (e != cudaSuccess) {
        set_error(std::string("dgb_unzip_plan_create: ") + cudaGetErrorString(e));
        dgb_unzip_plan_destroy(p);
        return DGB_ERR_ALLOC;
    }
    *out = p;
    return DGB_OK;
}

dgb_status dgb_unzip_plan_destroy(dgb_unzip_plan *p)
{
    if (!p) return DGB_OK;
    cudaFree(p->d_copy);
    cudaFree(p->d_zip);
    cudaFree(p->d_srefs);
    cudaFree(p->d_dg);
    cudaFree(p->d_gptr);
    cudaFree(p->d_gdst);
    cudaFree(p->d_gcode);
    delete p;
    return DGB_OK;
}

dgb_status dgb_unzip(dgb_unzip_plan *p, const double *const *zipped, double *const *unzipped,
                     int nvars, void *stream)
{
    if (!p || !zipped || !unzipped || nvars < 1 || nvars > NV) {
        set_error("dgb_unzip: bad argument");
        return DGB_ERR_INVALID;
    }
    return do_unzip(p, zipped, unzipped, nvars, (cudaStream_t)stream);
}

dgb_status dgb_zip(dgb_unzip_plan *p, const double *const *unzipped, double *const *zipped,
                   int nvars, void *stream)
{
    if (!p || !zipped || !unzipped || nvars < 1 || nvars > NV) {
        set_error("dgb_zip: bad argument");
        return DGB_ERR_INVALID;
    }
    return do_zip(p, unzipped, zipped, nvars, (cudaStream_t)stream);
}

dgb_status dgb_stepper_destroy(dgb_stepper *s)
{
    if (!s) return DGB_OK;
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->ev_in) cudaEventDestroy(s->ev_in);
    if (s->ev_out) cudaEventDestroy(s->ev_out);
    if (s->st) cudaStreamDestroy(s->st);
    cudaFree(s->d_U);
    cudaFree(s->d_R);
    cudaFree(s->d_k);
    cudaFree(s->d_im);
    cudaFree(s->d_gmap);
    cudaFree(s->d_zmap);
    cudaFree(s->d_ib);
    cudaFree(s->d_status);
    delete s;
    return DGB_OK;
}

dgb_status dgb_stepper_create_ex(dgb_plan *rhs_plan, dgb_unzip_plan *uz, int precision,
                                 unsigned flags, dgb_stepper **out)
{
    if (!rhs_plan || !uz || !out) {
        set_error("dgb_stepper_create: null argument");
        return DGB_ERR_INVALID;
    }
    if (flags & ~(unsigned)DGB_STEP_FUSED_UNZIP) {
        set_error("dgb_stepper_create: unknown flags");
        return DGB_ERR_INVALID;
    }
    if (dgb_plan_unzipped_size(rhs_plan) != uz->nunz) {
        set_error("dgb_stepper_create: the RHS plan and the unzip plan disagree on the unzipped size");
        return DGB_ERR_INVALID;
    }
    const bool fused = (flags & DGB_STEP_FUSED_UNZIP) != 0;
    const size_t nu = uz->nunz, nd = uz->ndof, nib = uz->ninterp + 1;
    if (fused && nd + nib >= kSentinel) {
        set_error("dgb_stepper_create: too many nodes for 32-bit gather indices");
        return DGB_ERR_INVALID;
    }
    dgb_stepper *s = new dgb_stepper();
    s->plan = rhs_plan;
    s->uz = uz;
    s->precision = precision;
    s->fused = fused;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e != cudaSuccess) return;
        e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) s->device_bytes += bytes;
    };
    if (!fused) {
        alloc((void **)&s->d_U, (size_t)NV * nu * 8);
        alloc((void **)&s->d_R, (size_t)NV * nu * 8);
    } else {
        alloc((void **)&s->d_gmap, nu * 4);
        alloc((void **)&s->d_zmap, nu * 4);
        alloc((void **)&s->d_ib, (size_t)NV * nib * 8);
    }
    alloc((void **)&s->d_k, (size_t)4 * NV * nd * 8);
    alloc((void **)&s->d_im, (size_t)NV * nd * 8);
    alloc((void **)&s->d_status, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_out, cudaEventDisableTiming);
    // padding beyond domain faces is never written by unzip: keep it finite
    // (fused mode: the zero row the gather index of such points names)
    if (e == cudaSuccess && !fused) e = cudaMemsetAsync(s->d_U, 0, (size_t)NV * nu * 8, s->st);
    if (e == cudaSuccess && !fused) e = cudaMemsetAsync(s->d_R, 0, (size_t)NV * nu * 8, s->st);
    if (e == cudaSuccess && fused) e = cudaMemsetAsync(s->d_ib, 0, (size_t)NV * nib * 8, s->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_im, 0, (size_t)NV * nd * 8, s->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_status, 0, sizeof(unsigned int), s->st);
    if (e == cudaSuccess && fused) {
        if (nu) {
            gmap_copy_kernel<<<grid_for(nu, 256), 256, 0, s->st>>>(s->d_gmap, uz->d_copy, nu,
                                                                  (uint32_t)(nd + uz->ninterp));
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && uz->ninterp) {
            gmap_interp_kernel<<<grid_for(uz->ninterp, 256), 256, 0, s->st>>>(
                s->d_gmap, uz->d_gdst, uz->ninterp, (uint32_t)nd);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && nu) e = cudaMemsetAsync(s->d_zmap, 0xFF, nu * 4, s->st);
        if (e == cudaSuccess && nd) {
            zmap_kernel<<<grid_for(nd, 256), 256, 0, s->st>>>(s->d_zmap, uz->d_zip, nd);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        set_error(std::string("dgb_stepper_create: ") + cudaGetErrorString(e));
        dgb_stepper_destroy(s);
        return DGB_ERR_ALLOC;
    }
    // one RHS outside any capture: builds the plan's work items and kernel attributes
    double *U[NV], *R[NV];
    dgb_status r;
    if (!fused) {
        for (int v = 0; v < NV; v++) {
            U[v] = s->d_U + (size_t)v * nu;
            R[v] = s->d_R + (size_t)v * nu;
        }
        r = dgb_bssn_rhs(rhs_plan, R, U, precision, s->st);
    } else {
        const double *Z[NV], *IB[NV];
        for (int v = 0; v < NV; v++) {
            Z[v] = s->d_im + (size_t)v * nd;
            R[v] = s->d_k + (size_t)v * nd;
            IB[v] = s->d_ib + (size_t)v * nib;
        }
        r = run_rhs_gather(rhs_plan, R, Z, IB, s->d_gmap, s->d_zmap, (uint32_t)nd, precision, s->st);
    }
    if (r == DGB_OK && cudaStreamSynchronize(s->st) != cudaSuccess) r = DGB_ERR_CUDA;
    if (r != DGB_OK) {
        dgb_stepper_destroy(s);
        return r;
    }
    *out = s;
    return DGB_OK;
}

dgb_status dgb_stepper_create(dgb_plan *rhs_plan, dgb_unzip_plan *uz, int precision,
                              dgb_stepper **out)
{
    return dgb_stepper_create_ex(rhs_plan, uz, precision, 0u, out);
}

dgb_status dgb_stepper_device_bytes(const dgb_stepper *s, uint64_t *bytes)
{
    if (!s || !bytes) return DGB_ERR_INVALID;
    *bytes = s->device_bytes;
    return DGB_OK;
}

dgb_status dgb_rk4_step(dgb_stepper *s, double *const *state, double dt, double chi_floor,
                        int nsteps, void *stream)
{
    if (!s || !state || nsteps < 0) {
        set_error("dgb_rk4_step: bad argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV; v++)
        if (!state[v]) return DGB_ERR_INVALID;
    // the graph holds the plans' work-item addresses: capture again when one was freed
    const uint64_t items = plan_items_gen(s->plan);
    bool same = s->exec && s->key_dt == dt && s->key_floor == chi_floor && s->key_items == items;
    for (int v = 0; same && v < NV; v++) same = s->key_state[v] == state[v];
    if (!same) {
        if (s->exec) {
            cudaGraphExecDestroy(s->exec);
            s->exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        DGB_CUDA(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
        dgb_status r = enqueue_step(s, state, dt, chi_floor, s->st);
        const cudaError_t ec = cudaStreamEndCapture(s->st, &g);
        if (r != DGB_OK) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        if (ec != cudaSuccess) {
            set_error(std::string("dgb_rk4_step: capture: ") + cudaGetErrorString(ec));
            return DGB_ERR_CUDA;
        }
        const cudaError_t ei = cudaGraphInstantiate(&s->exec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            s->exec = nullptr;
            set_error(std::string("dgb_rk4_step: instantiate: ") + cudaGetErrorString(ei));
            return DGB_ERR_CUDA;
        }
        for (int v = 0; v < NV; v++) s->key_state[v] = state[v];
        s->key_dt = dt;
        s->key_floor = chi_floor;
        s->key_items = items;
    }
    cudaStream_t caller = (cudaStream_t)stream;
    DGB_CUDA(cudaEventRecord(s->ev_in, caller));
    DGB_CUDA(cudaStreamWaitEvent(s->st, s->ev_in, 0));
    for (int k = 0; k < nsteps; k++) DGB_CUDA(cudaGraphLaunch(s->exec, s->st));
    DGB_CUDA(cudaEventRecord(s->ev_out, s->st));
    DGB_CUDA(cudaStreamWaitEvent(caller, s->ev_out, 0));
    unsigned int h = 0;
    DGB_CUDA(cudaMemcpyAsync(&h, s->d_status, sizeof h, cudaMemcpyDeviceToHost, s->st));
    DGB_CUDA(cudaStreamSynchronize(s->st));
    if (h & 1u) {
        cudaMemsetAsync(s->d_status, 0, sizeof(unsigned int), s->st);
        set_error("dgb_rk4_step: det(gt) <= 0 at some node (the reference exits here)");
        return DGB_ERR_CONSTRAINT;
    }
    return DGB_OK;
}

}  // extern "C"
