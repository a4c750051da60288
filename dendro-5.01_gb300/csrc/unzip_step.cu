// Device unzip / zip from a generic mesh operator, and the full RK4 step as
// one CUDA graph per step.
//
// unzip: a copy pass (one thread per padded point, all fields per thread, the
// zipped index read once) and an interpolation pass (one thread per
// interpolation row: hanging nodes and padding next to coarser leaves,
// 2..343 terms).  zip: one gather per independent node.  All three are
// HBM-bound; the RK4 step around them is
//   for s in 0..3: unzip(prev or im) -> bssnRHS -> zip -> stage update
// (BSSN_GR/src/rkBSSN.cpp:803-1012), captured once and replayed.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>

#include "dgb_internal.h"

namespace dgb {
namespace {

constexpr uint32_t kSentinel = 0xFFFFFFFFu;

struct FieldPtrs {
    const double *in[NV];
    double *out[NV];
    int nvars;
};

__global__ void __launch_bounds__(256) unzip_copy_kernel(const FieldPtrs f, const uint32_t *__restrict__ src,
                                                         uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += stride) {
        const uint32_t s = __ldg(src + p);
        if (s == kSentinel) continue;
        for (int v = 0; v < f.nvars; v++) f.out[v][p] = __ldg(f.in[v] + s);
    }
}

__global__ void __launch_bounds__(128) unzip_interp_kernel(const FieldPtrs f, const uint64_t *__restrict__ dst,
                                                           const uint64_t *__restrict__ ptr,
                                                           const uint32_t *__restrict__ col,
                                                           const double *__restrict__ w, uint64_t nrows)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < nrows; r += stride) {
        const uint64_t b = ptr[r], e = ptr[r + 1], d = dst[r];
        double acc[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) acc[v] = 0.0;
        for (uint64_t t = b; t < e; t++) {
            const uint32_t c = __ldg(col + t);
            const double wt = __ldg(w + t);
#pragma unroll
            for (int v = 0; v < NV; v++)
                if (v < f.nvars) acc[v] = fma(wt, __ldg(f.in[v] + c), acc[v]);
        }
#pragma unroll
        for (int v = 0; v < NV; v++)
            if (v < f.nvars) f.out[v][d] = acc[v];
    }
}

__global__ void __launch_bounds__(256) zip_kernel(const FieldPtrs f, const uint64_t *__restrict__ src,
                                                  uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t d = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; d < n; d += stride) {
        const uint64_t s = __ldg(src + d);
        for (int v = 0; v < f.nvars; v++) f.out[v][d] = __ldg(f.in[v] + s);
    }
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

}  // namespace
}  // namespace dgb

using namespace dgb;

struct dgb_unzip_plan {
    uint64_t ndof = 0, nunz = 0, ninterp = 0, nnz = 0;
    uint32_t *d_copy = nullptr;
    uint64_t *d_idst = nullptr, *d_iptr = nullptr, *d_zip = nullptr;
    uint32_t *d_icol = nullptr;
    double *d_iw = nullptr;
};

struct dgb_stepper {
    dgb_plan *plan = nullptr;
    dgb_unzip_plan *uz = nullptr;
    int precision = 0;
    double *d_U = nullptr, *d_R = nullptr, *d_k = nullptr, *d_im = nullptr;
    unsigned int *d_status = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t exec = nullptr;
    const double *key_state[NV] = {};
    double key_dt = 0.0, key_floor = 0.0;
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

dgb_status do_unzip(dgb_unzip_plan *p, const double *const *zipped, double *const *unzipped,
                    int nvars, cudaStream_t st)
{
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
    if (p->ninterp) {
        unzip_interp_kernel<<<grid_for(p->ninterp, 128), 128, 0, st>>>(f, p->d_idst, p->d_iptr, p->d_icol,
                                                                      p->d_iw, p->ninterp);
        DGB_CUDA(cudaGetLastError());
    }
    return DGB_OK;
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
        U[v] = s->d_U + (size_t)v * nu;
        R[v] = s->d_R + (size_t)v * nu;
        IM[v] = s->d_im + (size_t)v * nd;
        for (int q = 0; q < 4; q++) K[q * NV + v] = s->d_k + ((size_t)q * NV + v) * nd;
    }
    for (int stage = 0; stage < 4; stage++) {
        const double *const *src = stage == 0 ? (const double *const *)state : (const double *const *)IM;
        dgb_status r = do_unzip(s->uz, src, U, NV, st);
        if (r != DGB_OK) return r;
        r = dgb_bssn_rhs(s->plan, R, U, s->precision, st);
        if (r != DGB_OK) return r;
        double *KS[NV];
        for (int v = 0; v < NV; v++) KS[v] = (double *)K[stage * NV + v];
        r = do_zip(s->uz, R, KS, NV, st);
        if (r != DGB_OK) return r;
        DGB_CUDA(rk4_launch(stage, stage < 3 ? IM : state, (const double *const *)state, K, nd, dt,
                            chi_floor, s->d_status, st));
    }
    return DGB_OK;
}

}  // namespace

extern "C" {

dgb_status dgb_unzip_plan_create(uint64_t ndof, uint64_t unzipped_size, const uint32_t *copy_src,
                                 uint64_t ninterp, const uint64_t *interp_dst,
                                 const uint64_t *interp_ptr, const uint32_t *interp_col,
                                 const double *interp_w, const uint64_t *zip_src,
                                 dgb_unzip_plan **out)
{
    if (!out || (unzipped_size && !copy_src) || (ndof && !zip_src) ||
        (ninterp && (!interp_dst || !interp_ptr || !interp_col || !interp_w))) {
        set_error("dgb_unzip_plan_create: null argument");
        return DGB_ERR_INVALID;
    }
    if (ndof >= kSentinel) {
        set_error("dgb_unzip_plan_create: more than 2^32-1 zipped nodes");
        return DGB_ERR_INVALID;
    }
    // validate the operator so the kernels cannot read or write out of range
    for (uint64_t p = 0; p < unzipped_size; p++)
        if (copy_src[p] != kSentinel && copy_src[p] >= ndof) {
            set_error("dgb_unzip_plan_create: copy source out of range");
            return DGB_ERR_INVALID;
        }
    const uint64_t nnz = ninterp ? interp_ptr[ninterp] : 0;
    if (ninterp && interp_ptr[0] != 0) return DGB_ERR_INVALID;
    for (uint64_t r = 0; r < ninterp; r++) {
        if (interp_dst[r] >= unzipped_size || interp_ptr[r + 1] < interp_ptr[r]) {
            set_error("dgb_unzip_plan_create: bad interpolation row");
            return DGB_ERR_INVALID;
        }
    }
    for (uint64_t t = 0; t < nnz; t++)
        if (interp_col[t] >= ndof) {
            set_error("dgb_unzip_plan_create: interpolation column out of range");
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
    p->nnz = nnz;
    cudaError_t e = cudaSuccess;
    auto up = [&](void **dst, const void *src, size_t bytes) {
        if (e != cudaSuccess || bytes == 0) return;
        e = cudaMalloc(dst, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    };
    up((void **)&p->d_copy, copy_src, unzipped_size * 4);
    up((void **)&p->d_zip, zip_src, ndof * 8);
    up((void **)&p->d_idst, interp_dst, ninterp * 8);
    up((void **)&p->d_iptr, interp_ptr, ninterp ? (ninterp + 1) * 8 : 0);
    up((void **)&p->d_icol, interp_col, nnz * 4);
    up((void **)&p->d_iw, interp_w, nnz * 8);
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
    cudaFree(p->d_idst);
    cudaFree(p->d_iptr);
    cudaFree(p->d_icol);
    cudaFree(p->d_iw);
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
    cudaFree(s->d_status);
    delete s;
    return DGB_OK;
}

dgb_status dgb_stepper_create(dgb_plan *rhs_plan, dgb_unzip_plan *uz, int precision,
                              dgb_stepper **out)
{
    if (!rhs_plan || !uz || !out) {
        set_error("dgb_stepper_create: null argument");
        return DGB_ERR_INVALID;
    }
    if (dgb_plan_unzipped_size(rhs_plan) != uz->nunz) {
        set_error("dgb_stepper_create: the RHS plan and the unzip plan disagree on the unzipped size");
        return DGB_ERR_INVALID;
    }
    dgb_stepper *s = new dgb_stepper();
    s->plan = rhs_plan;
    s->uz = uz;
    s->precision = precision;
    const size_t nu = uz->nunz, nd = uz->ndof;
    cudaError_t e = cudaMalloc(&s->d_U, (size_t)NV * nu * 8);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_R, (size_t)NV * nu * 8);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_k, (size_t)4 * NV * nd * 8);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_im, (size_t)NV * nd * 8);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_status, sizeof(unsigned int));
    // padding beyond domain faces is never written by unzip: keep it finite
    if (e == cudaSuccess) e = cudaMemset(s->d_U, 0, (size_t)NV * nu * 8);
    if (e == cudaSuccess) e = cudaMemset(s->d_R, 0, (size_t)NV * nu * 8);
    if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_out, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        set_error(std::string("dgb_stepper_create: ") + cudaGetErrorString(e));
        dgb_stepper_destroy(s);
        return DGB_ERR_ALLOC;
    }
    // one RHS outside any capture: builds the plan's work items and kernel attributes
    double *U[NV], *R[NV];
    for (int v = 0; v < NV; v++) {
        U[v] = s->d_U + (size_t)v * nu;
        R[v] = s->d_R + (size_t)v * nu;
    }
    dgb_status r = dgb_bssn_rhs(rhs_plan, R, U, precision, s->st);
    if (r == DGB_OK && cudaStreamSynchronize(s->st) != cudaSuccess) r = DGB_ERR_CUDA;
    if (r != DGB_OK) {
        dgb_stepper_destroy(s);
        return r;
    }
    *out = s;
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
    bool same = s->exec && s->key_dt == dt && s->key_floor == chi_floor;
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
