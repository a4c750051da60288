// C ABI of the library: device set-up, plans, the RHS entry points (device
// and host arrays), the RK4 stage update and the synthetic fill.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "dgb_internal.h"
#include "host_rows.h"
#include "synth.cuh"

namespace dgb {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }

static int g_device = -1;
static int g_nsm = 0;

#define DGB_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                   \
            return DGB_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

}  // namespace dgb

using namespace dgb;

struct dgb_plan {
    int device = -1;
    int nsm = 0;
    std::vector<dgb_block_desc> blocks;
    dgb_bssn_params prm{};
    uint64_t unzipped = 0, interior = 0;
    DevBlock *d_blocks = nullptr;
    uint64_t *d_first = nullptr;  // first padded point of each block (synthetic fill)
    // work items per tile variant (built lazily)
    std::vector<WorkItem *> d_items;
    std::vector<uint32_t> nitems;
    int variant[2] = {0, 0};  // chosen tile variant per precision
    // per precision: tile caps per block-size class picked by the autotuner
    // (class key: sizes and whether the block touches a domain face); blocks of
    // classes without an entry take the variant's full tile
    std::map<uint64_t, TileShape> caps[2];
    uint64_t caps_gen[2] = {0, 0};
    struct ItemCache {
        int variant = -1;
        uint64_t gen = ~0ull;
        WorkItem *d = nullptr;
        uint32_t n = 0;
    } rhs_items[2][kMaxTileShapes];  // the BSSN RHS's capped work items per precision and variant
    // bumped whenever a work-item buffer is freed: a captured RK4 graph that
    // may hold the old buffer's address is captured again
    uint64_t items_gen = 0;
    unsigned int *d_queue = nullptr;
    double *d_scratch = nullptr;
    size_t scratch_doubles = 0;
    int occupancy[8][2] = {};  // resident CTAs per SM per (variant, precision)
    int occupancy_g[8][2] = {};  // the same for the gather-mode kernels (0 = not yet known)
    int pc_occupancy = 0;      // constraint kernel, resident CTAs per SM (0 = not yet known)
    // CCZ4 kernel: its own workspace (241 slots per point), allocated at first use
    int c4_occupancy[2] = {0, 0};  // per precision
    int b4_occupancy = 0;          // the 4th-order BSSN kernel (same workspace buffer)
    double *d_scratch4 = nullptr;
    size_t scratch4_doubles = 0;
    // host-array entry point: chunked pipeline, built at first use
    struct HostPipe *pipe = nullptr;
    bool borrowed_scratch = false;  // a chunk sub-plan using its parent's workspace
};

void destroy_pipe(struct HostPipe *h);

namespace dgb {
void host_gather(double *dst, size_t slot_pts, const double *const *u, int nv, uint64_t start,
                 uint64_t span);
void host_scatter_rows(double *const *rhs, const double *src, size_t islot, int nv,
                       const IRow *rows, size_t nrows, uint64_t start);
}  // namespace dgb

// The host-array entry point as a pipeline over chunks of blocks (contiguous
// in the caller's unzipped arrays): host threads copy chunk a's fields into
// pinned staging while the GPU uploads chunk a-1... in order per chunk
//   gather (host) -> H2D -> RHS -> pack the interior rows (device) -> D2H
//   -> scatter of the interior rows (host)
// with three device slots, two pinned staging buffers each way and separate
// upload / compute / download streams, so transfers overlap the kernel.
// Input fields in dgb_host_alloc memory skip the gather: the upload reads
// the caller's page-locked arrays directly.
// Only interior points are written back, so the caller's rhs padding is
// untouched without uploading rhs.
struct HostPipe {
    // slots hold up to NV4 (CCZ4) fields; BSSN uses the first NV
    size_t slot_pts = 0;
    std::vector<uint64_t> start, span;
    std::vector<std::vector<uint32_t>> members;
    std::vector<dgb_plan *> sub;
    double *d_slots = nullptr;          // 3 u slots, then 3 rhs slots, NV4 * slot_pts each
    // the right-hand side's interior points of a chunk, packed row by row on the
    // device before the download: only interior values cross the link and
    // land in host memory
    std::vector<IRow> rows;             // all chunks, in chunk order
    std::vector<size_t> row_ptr;        // chunk c: rows[row_ptr[c] .. row_ptr[c+1])
    std::vector<uint64_t> ispan;        // packed interior points per chunk
    size_t islot = 0;
    IRow *d_rows = nullptr;
    double *d_packed = nullptr;         // 3 packed slots, NV4 * islot each
    double *h_in[2] = {nullptr, nullptr}, *h_out[2] = {nullptr, nullptr};  // pinned
    // upload mode per entry kind (nv * 64 + nv_out) for inputs in dgb_host_alloc
    // memory: the last wall time of a call through the staging (0) and of a
    // direct call (1), and the number of such calls
    struct UploadStats {
        double ms[2] = {0.0, 0.0};
        uint64_t calls = 0;
    };
    std::map<int, UploadStats> upload;
    // two compute streams, even and odd chunks: the next chunk's kernel fills
    // the SMs the current one's last work items leave idle.  Odd chunks run
    // on their own derivative workspaces (the parent's serve the even ones).
    cudaStream_t s_h2d = nullptr, s_comp[2] = {nullptr, nullptr}, s_d2h = nullptr;
    double *d_scratch_odd = nullptr, *d_scratch4_odd = nullptr;
    size_t scratch4_odd_doubles = 0;
    std::vector<cudaEvent_t> ev_h2d, ev_comp, ev_d2h;
};

void destroy_pipe(HostPipe *h)
{
    if (!h) return;
    for (dgb_plan *sp : h->sub) dgb_plan_destroy(sp);
    cudaFree(h->d_slots);
    cudaFree(h->d_rows);
    cudaFree(h->d_packed);
    cudaFree(h->d_scratch_odd);
    cudaFree(h->d_scratch4_odd);
    for (int q = 0; q < 2; q++) {
        cudaFreeHost(h->h_in[q]);
        cudaFreeHost(h->h_out[q]);
    }
    for (auto e : h->ev_h2d) if (e) cudaEventDestroy(e);
    for (auto e : h->ev_comp) if (e) cudaEventDestroy(e);
    for (auto e : h->ev_d2h) if (e) cudaEventDestroy(e);
    if (h->s_h2d) cudaStreamDestroy(h->s_h2d);
    for (int q = 0; q < 2; q++)
        if (h->s_comp[q]) cudaStreamDestroy(h->s_comp[q]);
    if (h->s_d2h) cudaStreamDestroy(h->s_d2h);
    delete h;
}

namespace {

bool interior_block(const dgb_block_desc &b) { return b.sz[0] >= 7 && b.sz[1] >= 7 && b.sz[2] >= 7; }

// Split interior extent m into the fewest tiles of size <= t, as even as possible.
void split_extent(int m, int t, std::vector<std::pair<int, int>> &out)
{
    out.clear();
    const int nt = (m + t - 1) / t;
    const int base = m / nt, rem = m % nt;
    int o = 0;
    for (int q = 0; q < nt; q++) {
        const int e = base + (q < rem ? 1 : 0);
        out.push_back({o, e});
        o += e;
    }
}

uint64_t class_key(const dgb_block_desc &d)
{
    return ((uint64_t)d.sz[0] << 42) | ((uint64_t)d.sz[1] << 22) | ((uint64_t)d.sz[2] << 2) |
           (d.bflag != 0 ? 1u : 0u);
}

// Work items of the blocks `sel` accepts, each block cut with its tile cap
// (cap(b) <= the variant's tile), largest tiles first.
template <class Sel, class Cap>
dgb_status make_items(const dgb_plan *p, Sel sel, Cap cap, std::vector<WorkItem> &items)
{
    items.clear();
    std::vector<std::pair<int, int>> sx, sy, sz;
    for (size_t b = 0; b < p->blocks.size(); b++) {
        const dgb_block_desc &d = p->blocks[b];
        if (!sel(d)) continue;
        const TileShape t = cap(d);
        split_extent((int)d.sz[0] - 6, t.tx, sx);
        split_extent((int)d.sz[1] - 6, t.ty, sy);
        split_extent((int)d.sz[2] - 6, t.tz, sz);
        for (auto &kz : sz)
            for (auto &jy : sy)
                for (auto &ix : sx) {
                    if (d.bflag != 0 && (ix.second < 3 || jy.second < 3 || kz.second < 3)) {
                        // a closure reads up to 5 points inward from a face: the tile
                        // holding the face must stage them
                        set_error("tile schedule cuts a boundary block into tiles thinner than 3");
                        return DGB_ERR_INVALID;
                    }
                    WorkItem w;
                    w.blk = (uint32_t)b;
                    w.o[0] = (uint16_t)ix.first; w.o[1] = (uint16_t)jy.first; w.o[2] = (uint16_t)kz.first;
                    w.e[0] = (uint16_t)ix.second; w.e[1] = (uint16_t)jy.second; w.e[2] = (uint16_t)kz.second;
                    items.push_back(w);
                }
    }
    // largest tiles first (longest-processing-time order for the queue)
    std::stable_sort(items.begin(), items.end(), [](const WorkItem &a, const WorkItem &b) {
        return a.e[0] * a.e[1] * a.e[2] > b.e[0] * b.e[1] * b.e[2];
    });
    return DGB_OK;
}

dgb_status upload_items(const std::vector<WorkItem> &items, WorkItem **d)
{
    *d = nullptr;
    if (items.empty()) return DGB_OK;
    DGB_CUDA(cudaMalloc(d, items.size() * sizeof(WorkItem)));
    DGB_CUDA(cudaMemcpy(*d, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    return DGB_OK;
}

// The variant's full-tile schedule (also the CCZ4 and constraint kernels').
dgb_status build_items(dgb_plan *p, int variant)
{
    if (p->d_items[variant]) return DGB_OK;
    const TileShape t = kTileShapes[variant];
    std::vector<WorkItem> items;
    dgb_status s = make_items(p, [](const dgb_block_desc &) { return true; },
                              [&](const dgb_block_desc &) { return t; }, items);
    if (s != DGB_OK) return s;
    WorkItem *d = nullptr;
    s = upload_items(items, &d);
    if (s != DGB_OK) return s;
    p->d_items[variant] = d;
    p->nitems[variant] = (uint32_t)items.size();
    return DGB_OK;
}

TileShape clip(TileShape a, TileShape m)
{
    return TileShape{std::min(a.tx, m.tx), std::min(a.ty, m.ty), std::min(a.tz, m.tz)};
}

// The BSSN RHS's schedule for a precision: the variant's tile, capped per
// block-size class where the autotuner chose a cap.
dgb_status rhs_items(dgb_plan *p, int variant, int prec, const WorkItem **d, uint32_t *n)
{
    dgb_plan::ItemCache &c = p->rhs_items[prec][variant];
    if (p->caps[prec].empty()) {
        dgb_status s = build_items(p, variant);
        *d = p->d_items[variant];
        *n = p->nitems[variant];
        return s;
    }
    if (c.variant != variant || c.gen != p->caps_gen[prec]) {
        if (c.d) p->items_gen++;
        const TileShape m = kTileShapes[variant];
        std::vector<WorkItem> items;
        dgb_status s = make_items(
            p, [](const dgb_block_desc &) { return true; },
            [&](const dgb_block_desc &b) {
                auto it = p->caps[prec].find(class_key(b));
                return it == p->caps[prec].end() ? m : clip(it->second, m);
            },
            items);
        if (s != DGB_OK) return s;
        cudaFree(c.d);
        c.d = nullptr;
        c.n = 0;
        s = upload_items(items, &c.d);
        if (s != DGB_OK) return s;
        c.n = (uint32_t)items.size();
        c.variant = variant;
        c.gen = p->caps_gen[prec];
    }
    *d = c.d;
    *n = c.n;
    return DGB_OK;
}

RhsParams rhs_params(const dgb_bssn_params &q)
{
    RhsParams r;
    r.l1 = q.lambda[0]; r.l2 = q.lambda[1]; r.l3 = q.lambda[2]; r.l4 = q.lambda[3];
    r.lf0 = q.lambda_f[0]; r.lf1 = q.lambda_f[1];
    r.eta_const = q.eta_const; r.eta_r0 = q.eta_r0; r.eta_exp = q.eta_damping_exp;
    r.sigma = q.ko_sigma;
    return r;
}

dgb_status run_rhs_on(dgb_plan *p, double *const *rhs, const double *const *u, int precision,
                      int variant, const WorkItem *items, uint32_t nitems, cudaStream_t st);

dgb_status run_rhs42(dgb_plan *p, double *const *rhs, const double *const *u, int precision,
                     cudaStream_t st);

dgb_status run_rhs(dgb_plan *p, double *const *rhs, const double *const *u, int precision,
                   int variant, cudaStream_t st)
{
    if (precision != DGB_PREC_FP64 && precision != DGB_PREC_MIXED) {
        set_error("precision must be DGB_PREC_FP64 or DGB_PREC_MIXED");
        return DGB_ERR_INVALID;
    }
    if (p->prm.fd_order == 4) return run_rhs42(p, rhs, u, precision, st);
    const WorkItem *items = nullptr;
    uint32_t nitems = 0;
    dgb_status s = rhs_items(p, variant, precision == DGB_PREC_MIXED ? 1 : 0, &items, &nitems);
    if (s != DGB_OK) return s;
    return run_rhs_on(p, rhs, u, precision, variant, items, nitems, st);
}

// The RHS kernel of `variant` over an explicit work-item list.
dgb_status run_rhs_on(dgb_plan *p, double *const *rhs, const double *const *u, int precision,
                      int variant, const WorkItem *items, uint32_t nitems, cudaStream_t st)
{
    if (nitems == 0) return DGB_OK;
    DGB_CUDA(rhs_configure(variant, precision));
    RhsArgs a{};
    for (int v = 0; v < NV; v++) {
        a.u[v] = u[v];
        a.rhs[v] = rhs[v];
    }
    a.blocks = p->d_blocks;
    a.items = items;
    a.nitems = nitems;
    a.queue = p->d_queue;
    a.scratch = p->d_scratch;
    a.prm = rhs_params(p->prm);
    const int grid = p->nsm * p->occupancy[variant][precision == DGB_PREC_MIXED ? 1 : 0];
    DGB_CUDA(cudaMemsetAsync(p->d_queue, 0, sizeof(unsigned int), st));
    DGB_CUDA(rhs_launch(variant, precision, a, grid, st));
    return DGB_OK;
}

}  // namespace

uint64_t dgb::plan_items_gen(const dgb_plan *p) { return p->items_gen; }

dgb_status dgb::run_rhs_gather(dgb_plan *p, double *const *k, const double *const *z,
                               const double *const *ib, const uint32_t *gmap, const uint32_t *zmap,
                               uint32_t ndof, int precision, cudaStream_t st)
{
    if (precision != DGB_PREC_FP64 && precision != DGB_PREC_MIXED) {
        set_error("precision must be DGB_PREC_FP64 or DGB_PREC_MIXED");
        return DGB_ERR_INVALID;
    }
    if (p->prm.fd_order == 4) {
        set_error("the fused-unzip stepper runs the 6th-order binding only (fd_order 4: use the "
                  "unfused stepper)");
        return DGB_ERR_UNSUPPORTED;
    }
    const int prec = precision == DGB_PREC_MIXED ? 1 : 0;
    int variant = p->variant[prec];
    for (int pass = 0; pass < 2; pass++) {
        if (p->occupancy_g[variant][prec] == 0) {
            // the workspace is sized for the plain kernels' residency: never exceed it
            const int occ = rhs_max_ctas_per_sm_gather(variant, precision);
            if (occ < 1) {
                set_error("gather-mode RHS kernel cannot be resident");
                return DGB_ERR_CUDA;
            }
            p->occupancy_g[variant][prec] = std::min(occ, p->occupancy[variant][prec]);
        }
        // a variant whose gather indices cost it resident CTAs runs as 8^3
        // (the same bits: the tiling does not change any point's arithmetic)
        if (variant == 0 || p->occupancy_g[variant][prec] >= p->occupancy[variant][prec]) break;
        variant = 0;
    }
    const WorkItem *items = nullptr;
    uint32_t nitems = 0;
    dgb_status s = rhs_items(p, variant, prec, &items, &nitems);
    if (s != DGB_OK) return s;
    if (nitems == 0) return DGB_OK;
    RhsArgs a{};
    for (int v = 0; v < NV; v++) {
        a.u[v] = z[v];
        a.rhs[v] = k[v];
        a.ib[v] = ib[v];
    }
    a.gmap = gmap;
    a.zmap = zmap;
    a.ndof = ndof;
    a.blocks = p->d_blocks;
    a.items = items;
    a.nitems = nitems;
    a.queue = p->d_queue;
    a.scratch = p->d_scratch;
    a.prm = rhs_params(p->prm);
    const int grid = p->nsm * p->occupancy_g[variant][prec];
    DGB_CUDA(cudaMemsetAsync(p->d_queue, 0, sizeof(unsigned int), st));
    DGB_CUDA(rhs_launch_gather(variant, precision, a, grid, st));
    return DGB_OK;
}

// Page-locked allocations made by dgb_host_alloc: start address -> bytes.
// The host-array entries upload fields lying inside one of them directly.
static std::mutex g_host_mu;
static std::map<uintptr_t, size_t> g_host_allocs;

static bool in_host_alloc(const void *p, size_t bytes)
{
    const uintptr_t a = (uintptr_t)p;
    std::lock_guard<std::mutex> lock(g_host_mu);
    auto it = g_host_allocs.upper_bound(a);
    if (it == g_host_allocs.begin()) return false;
    --it;
    return a >= it->first && a - it->first <= it->second && bytes <= it->second - (a - it->first);
}

extern "C" {

int dgb_version(void) { return 1; }

dgb_status dgb_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr || bytes == 0) return DGB_ERR_INVALID;
    *ptr = nullptr;
    void *q = nullptr;
    if (cudaMallocHost(&q, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMallocHost failed");
        return DGB_ERR_ALLOC;
    }
    std::lock_guard<std::mutex> lock(g_host_mu);
    g_host_allocs[(uintptr_t)q] = bytes;
    *ptr = q;
    return DGB_OK;
}

dgb_status dgb_host_free(void *ptr)
{
    if (!ptr) return DGB_OK;
    {
        std::lock_guard<std::mutex> lock(g_host_mu);
        auto it = g_host_allocs.find((uintptr_t)ptr);
        if (it == g_host_allocs.end()) {
            set_error("dgb_host_free: not an allocation of dgb_host_alloc");
            return DGB_ERR_INVALID;
        }
        g_host_allocs.erase(it);
    }
    DGB_CUDA(cudaFreeHost(ptr));
    return DGB_OK;
}

const char *dgb_last_error(void) { return g_err.c_str(); }

dgb_status dgb_init(int device)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        set_error("no CUDA device");
        return DGB_ERR_NOT_INIT;
    }
    if (device < 0 || device >= n) {
        set_error("device index out of range");
        return DGB_ERR_INVALID;
    }
    DGB_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    DGB_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major * 10 + prop.minor < 100) {
        set_error("this library is built for sm_103a (GB300)");
        return DGB_ERR_UNSUPPORTED;
    }
    g_device = device;
    g_nsm = prop.multiProcessorCount;
    return DGB_OK;
}

dgb_status dgb_plan_create(const dgb_block_desc *blocks, size_t nblk, const dgb_bssn_params *prm,
                           dgb_plan **plan)
{
    if (!plan || !prm || (!blocks && nblk)) {
        set_error("dgb_plan_create: null argument");
        return DGB_ERR_INVALID;
    }
    *plan = nullptr;
    if (g_device < 0) {
        set_error("dgb_init not called");
        return DGB_ERR_NOT_INIT;
    }
    if (nblk > 0xFFFFFFFFull) {
        set_error("too many blocks");
        return DGB_ERR_INVALID;
    }
    if (prm->fd_order != 0 && prm->fd_order != 4 && prm->fd_order != 6) {
        set_error("dgb_plan_create: fd_order must be 4 or 6 (0 = 6)");
        return DGB_ERR_INVALID;
    }
    if (prm->gauge != DGB_GAUGE_ETA_CONST) {
        set_error("dgb_plan_create: only the standard gauge with constant eta "
                  "(bssneqs_eta_const_standard_gauge) is built; the eta-function and "
                  "Rochester-gauge equations are not");
        return DGB_ERR_UNSUPPORTED;
    }
    dgb_plan *p = new dgb_plan();
    p->device = g_device;
    p->nsm = g_nsm;
    p->prm = *prm;
    if (p->prm.fd_order == 0) p->prm.fd_order = 6;
    p->blocks.assign(blocks, blocks + nblk);
    std::vector<DevBlock> db(nblk);
    std::vector<uint64_t> first(nblk);
    for (size_t b = 0; b < nblk; b++) {
        const dgb_block_desc &d = blocks[b];
        if (!interior_block(d) || d.sz[0] > 4096 || d.sz[1] > 4096 || d.sz[2] > 4096) {
            set_error("block " + std::to_string(b) + ": each side must be in [7, 4096]");
            delete p;
            return DGB_ERR_INVALID;
        }
        if (d.bflag > 63u) {
            set_error("block " + std::to_string(b) + ": bflag has bits beyond the six faces");
            delete p;
            return DGB_ERR_INVALID;
        }
        if (d.bflag != 0 && (d.sz[0] < 13 || d.sz[1] < 13 || d.sz[2] < 13)) {
            // the one-sided closures read interior points 3..8 from each flagged face
            set_error("block " + std::to_string(b) +
                      ": domain-boundary blocks need at least 13 points per side");
            delete p;
            return DGB_ERR_INVALID;
        }
        const uint64_t n = (uint64_t)d.sz[0] * d.sz[1] * d.sz[2];
        p->unzipped = std::max(p->unzipped, d.offset + n);
        p->interior += (uint64_t)(d.sz[0] - 6) * (d.sz[1] - 6) * (d.sz[2] - 6);
        db[b].offset = d.offset;
        for (int a = 0; a < 3; a++) {
            db[b].sz[a] = d.sz[a];
            db[b].pmin[a] = d.ptmin[a];
            db[b].h[a] = (d.ptmax[a] - d.ptmin[a]) / (double)(d.sz[a] - 1);
            if (!(db[b].h[a] > 0.0) || !std::isfinite(db[b].h[a])) {
                set_error("block " + std::to_string(b) + ": ptmax must exceed ptmin");
                delete p;
                return DGB_ERR_INVALID;
            }
        }
        db[b].bflag = d.bflag;
        first[b] = d.offset;
    }
    p->d_items.assign(kNumTileShapes, nullptr);
    p->nitems.assign(kNumTileShapes, 0);
    // workspace for the largest resident grid over all compiled schedules
    size_t maxcta = 0;
    for (int v = 0; v < kNumTileShapes; v++)
        for (int q = 0; q < 2; q++) {
            const int occ = rhs_max_ctas_per_sm(v, q);
            p->occupancy[v][q] = std::max(1, std::min(occ, 4));
            maxcta = std::max(maxcta, rhs_scratch_per_cta(v) * (size_t)p->occupancy[v][q]);
        }
    p->scratch_doubles = maxcta * (size_t)p->nsm;
    if (p->occupancy[kDefaultVariantFp64][0] >= 2) p->variant[0] = kDefaultVariantFp64;
    cudaError_t e = cudaSuccess;
    if (nblk) {
        e = cudaMalloc(&p->d_blocks, nblk * sizeof(DevBlock));
        if (e == cudaSuccess) e = cudaMemcpy(p->d_blocks, db.data(), nblk * sizeof(DevBlock), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&p->d_first, nblk * sizeof(uint64_t));
        if (e == cudaSuccess) e = cudaMemcpy(p->d_first, first.data(), nblk * sizeof(uint64_t), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&p->d_queue, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_scratch, p->scratch_doubles * sizeof(double));
    if (e != cudaSuccess) {
        set_error(std::string("dgb_plan_create: ") + cudaGetErrorString(e));
        dgb_plan_destroy(p);
        return DGB_ERR_ALLOC;
    }
    *plan = p;
    return DGB_OK;
}

dgb_status dgb_plan_destroy(dgb_plan *p)
{
    if (!p) return DGB_OK;
    cudaFree(p->d_blocks);
    cudaFree(p->d_first);
    for (auto d : p->d_items) cudaFree(d);
    for (int q = 0; q < 2; q++)
        for (int v = 0; v < kMaxTileShapes; v++) cudaFree(p->rhs_items[q][v].d);
    cudaFree(p->d_queue);
    if (!p->borrowed_scratch) {
        cudaFree(p->d_scratch);
        cudaFree(p->d_scratch4);
    }
    destroy_pipe(p->pipe);
    delete p;
    return DGB_OK;
}

uint64_t dgb_plan_unzipped_size(const dgb_plan *p) { return p ? p->unzipped : 0; }
uint64_t dgb_plan_interior_points(const dgb_plan *p) { return p ? p->interior : 0; }

dgb_status dgb_plan_tile(const dgb_plan *p, int precision, uint32_t *tile3)
{
    if (!p || !tile3) return DGB_ERR_INVALID;
    const TileShape t = kTileShapes[p->variant[precision == DGB_PREC_MIXED ? 1 : 0]];
    tile3[0] = t.tx; tile3[1] = t.ty; tile3[2] = t.tz;
    return DGB_OK;
}

int dgb_num_tile_variants(void) { return kNumTileShapes; }

dgb_status dgb_plan_set_tile_variant(dgb_plan *p, int precision, int variant)
{
    if (!p || variant < 0 || variant >= kNumTileShapes) {
        set_error("dgb_plan_set_tile_variant: bad plan or variant");
        return DGB_ERR_INVALID;
    }
    const int prec = precision == DGB_PREC_MIXED ? 1 : 0;
    p->variant[prec] = variant;
    p->caps[prec].clear();  // the variant's full tile for every block
    p->caps_gen[prec]++;
    return DGB_OK;
}

dgb_status dgb_physical_constraints(dgb_plan *p, double *const *cons, const double *const *u,
                                   void *stream)
{
    if (!p || !cons || !u) {
        set_error("dgb_physical_constraints: null argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV; v++)
        if (!u[v]) {
            set_error("dgb_physical_constraints: null field pointer");
            return DGB_ERR_INVALID;
        }
    for (int c = 0; c < DGB_NUM_CONSTRAINTS; c++)
        if (!cons[c]) {
            set_error("dgb_physical_constraints: null output pointer");
            return DGB_ERR_INVALID;
        }
    dgb_status s = build_items(p, 0);  // the 8x8x8 schedule
    if (s != DGB_OK) return s;
    if (p->nitems[0] == 0) return DGB_OK;
    if (p->pc_occupancy == 0) {
        p->pc_occupancy = physcon_max_ctas_per_sm();
        if (p->pc_occupancy < 1) {
            set_error("dgb_physical_constraints: kernel cannot be resident");
            return DGB_ERR_CUDA;
        }
    }
    DGB_CUDA(physcon_configure());
    const size_t fit = p->scratch_doubles / physcon_scratch_per_cta();
    const int grid = (int)std::min<size_t>((size_t)p->nsm * p->pc_occupancy, fit);
    PcArgs a;
    for (int v = 0; v < NV; v++) a.u[v] = u[v];
    for (int c = 0; c < DGB_NUM_CONSTRAINTS; c++) a.cons[c] = cons[c];
    a.blocks = p->d_blocks;
    a.items = p->d_items[0];
    a.nitems = p->nitems[0];
    a.queue = p->d_queue;
    a.scratch = p->d_scratch;
    cudaStream_t st = (cudaStream_t)stream;
    DGB_CUDA(cudaMemsetAsync(p->d_queue, 0, sizeof(unsigned int), st));
    DGB_CUDA(physcon_launch(a, grid, st));
    return DGB_OK;
}

}  // extern "C"

namespace {

// The 4th-order BSSN kernel's residency and workspace (the buffer the CCZ4
// kernel also uses: a plan runs one kernel at a time), at first use.
dgb_status b4_workspace(dgb_plan *p)
{
    if (p->b4_occupancy != 0) return DGB_OK;
    const int occ = b4_max_ctas_per_sm();
    if (occ < 1) {
        set_error("dgb_bssn_rhs (fd_order 4): kernel cannot be resident");
        return DGB_ERR_CUDA;
    }
    const size_t need = b4_scratch_per_cta() * (size_t)occ * (size_t)p->nsm;
    if (need > p->scratch4_doubles) {
        if (p->borrowed_scratch) {
            set_error("dgb_bssn_rhs (fd_order 4): a chunk plan's borrowed workspace is too small");
            return DGB_ERR_INVALID;
        }
        cudaFree(p->d_scratch4);
        p->d_scratch4 = nullptr;
        p->scratch4_doubles = 0;
        p->c4_occupancy[0] = p->c4_occupancy[1] = 0;  // re-checked against the new buffer
        DGB_CUDA(cudaMalloc(&p->d_scratch4, need * sizeof(double)));
        p->scratch4_doubles = need;
    }
    p->b4_occupancy = occ;
    return DGB_OK;
}

// The BSSN right-hand side with the BSSN_GR solver's 4th-order binding.
dgb_status run_rhs42(dgb_plan *p, double *const *rhs, const double *const *u, int precision,
                     cudaStream_t st)
{
    if (precision != DGB_PREC_FP64) {
        set_error("dgb_bssn_rhs: fd_order 4 runs in FP64 only");
        return DGB_ERR_UNSUPPORTED;
    }
    dgb_status s = build_items(p, 0);  // the 8x8x8 schedule
    if (s != DGB_OK) return s;
    if (p->nitems[0] == 0) return DGB_OK;
    s = b4_workspace(p);
    if (s != DGB_OK) return s;
    DGB_CUDA(b4_configure());
    RhsArgs a{};
    for (int v = 0; v < NV; v++) {
        a.u[v] = u[v];
        a.rhs[v] = rhs[v];
    }
    a.blocks = p->d_blocks;
    a.items = p->d_items[0];
    a.nitems = p->nitems[0];
    a.queue = p->d_queue;
    a.scratch = p->d_scratch4;
    a.prm = rhs_params(p->prm);
    DGB_CUDA(cudaMemsetAsync(p->d_queue, 0, sizeof(unsigned int), st));
    DGB_CUDA(b4_launch(a, p->nsm * p->b4_occupancy, st));
    return DGB_OK;
}

// The CCZ4 kernel's residency and workspace, at first use per precision.
dgb_status c4_workspace(dgb_plan *p, int precision)
{
    const int pq = precision == DGB_PREC_MIXED ? 1 : 0;
    if (p->c4_occupancy[pq] != 0) return DGB_OK;
    const int occ = c4_max_ctas_per_sm(precision);
    if (occ < 1) {
        set_error("dgb_ccz4_rhs: kernel cannot be resident");
        return DGB_ERR_CUDA;
    }
    const size_t need = c4_scratch_per_cta() * (size_t)occ * (size_t)p->nsm;
    if (need > p->scratch4_doubles) {
        if (p->borrowed_scratch) {
            set_error("dgb_ccz4_rhs: a chunk plan's borrowed workspace is too small");
            return DGB_ERR_INVALID;
        }
        cudaFree(p->d_scratch4);
        p->d_scratch4 = nullptr;
        p->scratch4_doubles = 0;
        DGB_CUDA(cudaMalloc(&p->d_scratch4, need * sizeof(double)));
        p->scratch4_doubles = need;
    }
    p->c4_occupancy[pq] = occ;
    return DGB_OK;
}

}  // namespace

extern "C" {

dgb_status dgb_ccz4_rhs(dgb_plan *p, const dgb_ccz4_params *prm, double *const *rhs,
                        const double *const *u, int precision, void *stream)
{
    if (!p || !prm || !rhs || !u) {
        set_error("dgb_ccz4_rhs: null argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV4; v++)
        if (!rhs[v] || !u[v]) {
            set_error("dgb_ccz4_rhs: null field pointer");
            return DGB_ERR_INVALID;
        }
    if (precision != DGB_PREC_FP64 && precision != DGB_PREC_MIXED) {
        set_error("precision must be DGB_PREC_FP64 or DGB_PREC_MIXED");
        return DGB_ERR_INVALID;
    }
    const int pq = precision == DGB_PREC_MIXED ? 1 : 0;
    dgb_status s = build_items(p, 0);  // the 8x8x8 schedule
    if (s != DGB_OK) return s;
    if (p->nitems[0] == 0) return DGB_OK;
    s = c4_workspace(p, precision);
    if (s != DGB_OK) return s;
    DGB_CUDA(c4_configure(precision));
    C4Args a;
    for (int v = 0; v < NV4; v++) {
        a.u[v] = u[v];
        a.rhs[v] = rhs[v];
    }
    a.blocks = p->d_blocks;
    a.items = p->d_items[0];
    a.nitems = p->nitems[0];
    a.queue = p->d_queue;
    a.scratch = p->d_scratch4;
    a.prm = C4Params{prm->lambda[0], prm->lambda[1], prm->lambda[2], prm->lambda[3],
                     prm->lambda_f[0], prm->lambda_f[1], prm->kappa[0], prm->kappa[1],
                     prm->p_expo, prm->eta_const, prm->eta_r0, prm->eta_damping_exp,
                     prm->ko_sigma};
    cudaStream_t st = (cudaStream_t)stream;
    DGB_CUDA(cudaMemsetAsync(p->d_queue, 0, sizeof(unsigned int), st));
    DGB_CUDA(c4_launch(precision, a, p->nsm * p->c4_occupancy[pq], st));
    return DGB_OK;
}

dgb_status dgb_constraint_l2(const double *const *fields, int nvars, const double *mask,
                             double threshold, uint64_t ndof, double *out, void *stream)
{
    if (!fields || !out || nvars < 1 || nvars > DGB_NUM_CONSTRAINTS) {
        set_error("dgb_constraint_l2: bad argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < nvars; v++)
        if (!fields[v]) {
            set_error("dgb_constraint_l2: null field pointer");
            return DGB_ERR_INVALID;
        }
    cudaStream_t st = (cudaStream_t)stream;
    NormArgs a{};
    for (int v = 0; v < nvars; v++) a.f[v] = fields[v];
    a.nvars = nvars;
    a.mask = mask;
    a.threshold = threshold;
    a.ndof = ndof;
    const size_t np = (size_t)norm_partials() * (DGB_NUM_CONSTRAINTS + 1);
    double *buf = nullptr;
    DGB_CUDA(cudaMallocAsync(&buf, (np + DGB_NUM_CONSTRAINTS + 1) * sizeof(double), st));
    a.partial = buf;
    double res[DGB_NUM_CONSTRAINTS + 1];
    cudaError_t e = l2_norm_launch(a, buf + np, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(res, buf + np, sizeof(res), cudaMemcpyDeviceToHost, st);
    cudaError_t e2 = cudaFreeAsync(buf, st);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error(std::string("dgb_constraint_l2: ") + cudaGetErrorString(e));
        return DGB_ERR_CUDA;
    }
    for (int v = 0; v < nvars; v++) out[v] = res[v];
    return DGB_OK;
}

dgb_status dgb_bssn_rhs(dgb_plan *p, double *const *rhs, const double *const *u, int precision,
                        void *stream)
{
    if (!p || !rhs || !u) {
        set_error("dgb_bssn_rhs: null argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV; v++)
        if (!rhs[v] || !u[v]) {
            set_error("dgb_bssn_rhs: null field pointer");
            return DGB_ERR_INVALID;
        }
    const int prec = precision == DGB_PREC_MIXED ? 1 : 0;
    return run_rhs(p, rhs, u, precision, p->variant[prec], (cudaStream_t)stream);
}

dgb_status dgb_plan_autotune(dgb_plan *p, double *const *rhs, const double *const *u,
                             int precision, void *stream)
{
    if (!p || !rhs || !u) return DGB_ERR_INVALID;
    if (precision != DGB_PREC_FP64 && precision != DGB_PREC_MIXED) {
        set_error("precision must be DGB_PREC_FP64 or DGB_PREC_MIXED");
        return DGB_ERR_INVALID;
    }
    // the 4th-order kernel has one compiled schedule (8^3 tiles): nothing to choose
    if (p->prm.fd_order == 4) return DGB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = precision == DGB_PREC_MIXED ? 1 : 0;
    // block-size classes
    std::map<uint64_t, size_t> classes;
    for (const dgb_block_desc &d : p->blocks) classes[class_key(d)]++;
    cudaEvent_t e0, e1;
    DGB_CUDA(cudaEventCreate(&e0));
    DGB_CUDA(cudaEventCreate(&e1));
    dgb_status s = DGB_OK;
    std::vector<WorkItem> items;
    WorkItem *d = nullptr;
    // one class on one variant with one cap: time of a launch over that class
    auto time_class = [&](int v, uint64_t key, TileShape cap, float *ms) -> dgb_status {
        dgb_status r = make_items(
            p, [&](const dgb_block_desc &b) { return class_key(b) == key; },
            [&](const dgb_block_desc &) { return cap; }, items);
        if (r != DGB_OK) return r;
        cudaFree(d);
        d = nullptr;
        r = upload_items(items, &d);
        if (r != DGB_OK) return r;
        const uint32_t n = (uint32_t)items.size();
        r = run_rhs_on(p, rhs, u, precision, v, d, n, st);  // warm-up
        if (r != DGB_OK) return r;
        DGB_CUDA(cudaEventRecord(e0, st));
        r = run_rhs_on(p, rhs, u, precision, v, d, n, st);
        if (r != DGB_OK) return r;
        DGB_CUDA(cudaEventRecord(e1, st));
        DGB_CUDA(cudaEventSynchronize(e1));
        DGB_CUDA(cudaEventElapsedTime(ms, e0, e1));
        return DGB_OK;
    };
    float best_total = 1e30f;
    int best_v = p->variant[prec];
    std::map<uint64_t, TileShape> best_caps;
    for (int v = 0; v < kNumTileShapes && s == DGB_OK; v++) {
        const TileShape m = kTileShapes[v];
        // candidate caps: every compiled tile shape clipped to this variant's tile
        std::vector<TileShape> cands;
        for (int q = 0; q < kNumTileShapes; q++) {
            const TileShape c = clip(kTileShapes[q], m);
            bool dup = false;
            for (const TileShape &x : cands) dup = dup || (x.tx == c.tx && x.ty == c.ty && x.tz == c.tz);
            if (!dup) cands.push_back(c);
        }
        float total = 0.f;
        std::map<uint64_t, TileShape> caps;
        for (const auto &kv : classes) {
            float best = 1e30f;
            TileShape bc = m;
            for (const TileShape &c : cands) {
                float ms = 0.f;
                s = time_class(v, kv.first, c, &ms);
                if (s == DGB_ERR_INVALID) {  // a cap too thin for a boundary block: skip it
                    s = DGB_OK;
                    continue;
                }
                if (s != DGB_OK) break;
                if (ms < best) {
                    best = ms;
                    bc = c;
                }
            }
            if (s != DGB_OK) break;
            total += best;
            caps[kv.first] = bc;
        }
        if (s == DGB_OK && total < best_total) {
            best_total = total;
            best_v = v;
            best_caps = caps;
        }
    }
    cudaFree(d);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != DGB_OK) return s;
    p->variant[prec] = best_v;
    p->caps[prec] = best_caps;
    p->caps_gen[prec]++;
    return DGB_OK;
}

dgb_status dgb_plan_class_tiles(const dgb_plan *p, int precision, uint32_t *rows, size_t cap,
                                size_t *count)
{
    if (!p || !count) return DGB_ERR_INVALID;
    const int prec = precision == DGB_PREC_MIXED ? 1 : 0;
    *count = p->caps[prec].size();
    if (!rows) return DGB_OK;
    size_t i = 0;
    for (const auto &kv : p->caps[prec]) {
        if (i >= cap) break;
        uint32_t *r = rows + 7 * i++;
        r[0] = (uint32_t)(kv.first >> 42);
        r[1] = (uint32_t)((kv.first >> 22) & 0xFFFFF);
        r[2] = (uint32_t)((kv.first >> 2) & 0xFFFFF);
        r[3] = (uint32_t)(kv.first & 1u);
        r[4] = kv.second.tx;
        r[5] = kv.second.ty;
        r[6] = kv.second.tz;
    }
    return DGB_OK;
}

}  // extern "C"

namespace {

// Packs the interior rows of a chunk's right-hand side (nv fields, field v at
// slot + v * slot_pts) into packed (field v at packed + v * islot): one warp
// per (row, field).
__global__ void __launch_bounds__(256) pack_rows_kernel(const double *__restrict__ slot,
                                                        size_t slot_pts, double *__restrict__ packed,
                                                        size_t islot, const IRow *__restrict__ rows,
                                                        uint64_t nrows, int nv)
{
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; w < nrows * nv;
         w += nw) {
        const IRow r = rows[w % nrows];
        const uint64_t v = w / nrows;
        const double *src = slot + v * slot_pts + r.src;
        double *dst = packed + v * islot + r.dst;
        for (uint32_t i = lane; i < r.len; i += 32) dst[i] = __ldg(src + i);
    }
}

cudaError_t pack_rows_launch(const double *slot, size_t slot_pts, double *packed, size_t islot,
                             const IRow *rows, uint64_t nrows, int nv, cudaStream_t st)
{
    const uint64_t warps = nrows * (uint64_t)nv;
    const unsigned grid = (unsigned)std::min<uint64_t>((warps + 7) / 8, (uint64_t)g_nsm * 16);
    pack_rows_kernel<<<grid, 256, 0, st>>>(slot, slot_pts, packed, islot, rows, nrows, nv);
    return cudaGetLastError();
}

// Padded points per chunk: ~1.2 GB of fields each way per chunk, small next to
// the 20k-block batch (~40 chunks) and large next to any block.
constexpr uint64_t kChunkPts = 6u << 20;

dgb_status build_pipe_into(dgb_plan *p, HostPipe *h)
{
    uint64_t chunk_pts = kChunkPts;
    if (const char *env = getenv("DGB_HOST_CHUNK_PTS")) {  // tests: force many chunks
        const long long v = atoll(env);
        if (v > 0) chunk_pts = (uint64_t)v;
    }
    std::vector<uint32_t> order(p->blocks.size());
    for (size_t b = 0; b < order.size(); b++) order[b] = (uint32_t)b;
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return p->blocks[a].offset < p->blocks[b].offset;
    });
    auto npts = [&](uint32_t b) {
        const dgb_block_desc &d = p->blocks[b];
        return (uint64_t)d.sz[0] * d.sz[1] * d.sz[2];
    };
    for (size_t q = 0; q < order.size();) {
        // the first two chunks a quarter and a half of the others: the GPU
        // waits only for the first, short upload before its first kernel
        const size_t k = h->members.size();
        const uint64_t cap = k == 0 ? chunk_pts / 4 : k == 1 ? chunk_pts / 2 : chunk_pts;
        const uint64_t s0 = p->blocks[order[q]].offset;
        uint64_t end = s0 + npts(order[q]);
        std::vector<uint32_t> mem{order[q]};
        size_t r = q + 1;
        while (r < order.size()) {
            const uint64_t e2 = std::max(end, p->blocks[order[r]].offset + npts(order[r]));
            if (e2 - s0 > cap) break;
            end = e2;
            mem.push_back(order[r]);
            r++;
        }
        h->start.push_back(s0);
        h->span.push_back(end - s0);
        h->slot_pts = std::max<size_t>(h->slot_pts, end - s0);
        h->members.push_back(std::move(mem));
        q = r;
    }
    // one sub-plan per chunk, offsets relative to the chunk start; even
    // chunks share the parent's derivative workspace, odd chunks a second one
    // (consecutive chunks may run at the same time, chunks two apart never:
    // each compute stream runs its chunks in order)
    if (h->members.size() > 1)
        DGB_CUDA(cudaMalloc(&h->d_scratch_odd, p->scratch_doubles * sizeof(double)));
    for (size_t c = 0; c < h->members.size(); c++) {
        std::vector<dgb_block_desc> d;
        for (uint32_t b : h->members[c]) {
            dgb_block_desc x = p->blocks[b];
            x.offset -= h->start[c];
            d.push_back(x);
        }
        dgb_plan *sp = nullptr;
        dgb_status s = dgb_plan_create(d.data(), d.size(), &p->prm, &sp);
        if (s != DGB_OK) return s;
        h->sub.push_back(sp);
        cudaFree(sp->d_scratch);
        sp->d_scratch = (c & 1) ? h->d_scratch_odd : p->d_scratch;
        sp->borrowed_scratch = true;
        for (int q = 0; q < 2; q++) sp->variant[q] = p->variant[q];
    }
    // interior rows of each chunk, blocks in chunk order
    h->row_ptr.assign(1, 0);
    for (size_t c = 0; c < h->members.size(); c++) {
        uint32_t packed = 0;
        for (uint32_t b : h->members[c]) {
            const dgb_block_desc &d = p->blocks[b];
            const uint64_t base = d.offset - h->start[c];
            const uint32_t nx = d.sz[0], ny = d.sz[1], nz = d.sz[2];
            for (uint32_t k = 3; k + 3 < nz; k++)
                for (uint32_t j = 3; j + 3 < ny; j++) {
                    h->rows.push_back(IRow{(uint32_t)(base + 3 + (uint64_t)nx * (j + (uint64_t)ny * k)),
                                           packed, nx - 6});
                    packed += nx - 6;
                }
        }
        h->ispan.push_back(packed);
        h->islot = std::max<size_t>(h->islot, packed);
        h->row_ptr.push_back(h->rows.size());
    }
    const size_t slot = (size_t)NV4 * h->slot_pts;
    const size_t pslot = (size_t)NV4 * h->islot;
    DGB_CUDA(cudaMalloc(&h->d_slots, 6 * slot * sizeof(double)));
    DGB_CUDA(cudaMalloc(&h->d_packed, 3 * std::max<size_t>(pslot, 1) * sizeof(double)));
    DGB_CUDA(cudaMalloc(&h->d_rows, std::max<size_t>(h->rows.size(), 1) * sizeof(IRow)));
    if (!h->rows.empty())
        DGB_CUDA(cudaMemcpy(h->d_rows, h->rows.data(), h->rows.size() * sizeof(IRow),
                            cudaMemcpyHostToDevice));
    for (int q = 0; q < 2; q++) {
        DGB_CUDA(cudaMallocHost(&h->h_in[q], slot * sizeof(double)));
        DGB_CUDA(cudaMallocHost(&h->h_out[q], std::max<size_t>(pslot, 1) * sizeof(double)));
    }
    DGB_CUDA(cudaStreamCreateWithFlags(&h->s_h2d, cudaStreamNonBlocking));
    for (int q = 0; q < 2; q++) DGB_CUDA(cudaStreamCreateWithFlags(&h->s_comp[q], cudaStreamNonBlocking));
    DGB_CUDA(cudaStreamCreateWithFlags(&h->s_d2h, cudaStreamNonBlocking));
    const size_t nch = h->members.size();
    h->ev_h2d.resize(nch);
    h->ev_comp.resize(nch);
    h->ev_d2h.resize(nch);
    for (size_t c = 0; c < nch; c++) {
        DGB_CUDA(cudaEventCreateWithFlags(&h->ev_h2d[c], cudaEventDisableTiming));
        DGB_CUDA(cudaEventCreateWithFlags(&h->ev_comp[c], cudaEventDisableTiming));
        DGB_CUDA(cudaEventCreateWithFlags(&h->ev_d2h[c], cudaEventDisableTiming));
    }
    return DGB_OK;
}

// The pipeline over the chunks for nv fields; compute(sub-plan, rhs, u, stream)
// runs the kernel of one chunk.
template <class Compute>
dgb_status run_pipe_steps(dgb_plan *p, double *const *rhs, const double *const *u, int nv,
                          Compute compute, int nv_out, bool direct, bool out_direct, bool out_last)
{
    // nv fields in, nv_out fields out; direct: upload from the caller's arrays;
    // out_direct: the kernel stores the right-hand side's interior points
    // straight into the caller's page-locked arrays (no pack, download or
    // host scatter); out_last: the last chunk does, so that no download and
    // scatter trail the last kernel
    HostPipe *h = p->pipe;
    const long nch = (long)h->members.size();
    auto od = [&](long c) { return out_direct || (out_last && c == nch - 1); };
    const size_t slot = (size_t)NV4 * h->slot_pts;
    const size_t pslot = (size_t)NV4 * h->islot;
    auto ptrs = [&](int kind, long c, double **out) {  // kind 0: u slot, 1: rhs slot
        double *base = h->d_slots + (size_t)(3 * kind + (int)(c % 3)) * slot;
        for (int v = 0; v < NV4; v++) out[v] = base + (size_t)v * h->slot_pts;
    };
    for (long step = 0; step < nch + 3; step++) {
        const long c = step - 1, d = step - 2, a = step, e = step - 3;
        if (c >= 0 && c < nch) {  // compute chunk c once its upload is done
            cudaStream_t sc = h->s_comp[c & 1];
            DGB_CUDA(cudaStreamWaitEvent(sc, h->ev_h2d[c], 0));
            if (c >= 3) DGB_CUDA(cudaStreamWaitEvent(sc, h->ev_d2h[c - 3], 0));
            double *du[NV4], *dr[NV4];
            ptrs(0, c, du);
            ptrs(1, c, dr);
            if (od(c))  // the sub-plan's offsets are relative to the chunk start
                for (int v = 0; v < nv_out; v++) dr[v] = rhs[v] + h->start[c];
            dgb_status s = compute(h->sub[c], dr, (const double *const *)du, sc);
            if (s != DGB_OK) return s;
            const size_t nr = h->row_ptr[c + 1] - h->row_ptr[c];
            if (nr && !od(c)) {
                DGB_CUDA(pack_rows_launch(dr[0], h->slot_pts, h->d_packed + (size_t)(c % 3) * pslot,
                                          h->islot, h->d_rows + h->row_ptr[c], nr, nv_out, sc));
            }
            DGB_CUDA(cudaEventRecord(h->ev_comp[c], sc));
        }
        if (d >= 0 && d < nch) {  // download chunk d's packed interior once computed
            DGB_CUDA(cudaStreamWaitEvent(h->s_d2h, h->ev_comp[d], 0));
            const double *pk = h->d_packed + (size_t)(d % 3) * pslot;
            for (int v = 0; v < nv_out && h->ispan[d] && !od(d); v++)
                DGB_CUDA(cudaMemcpyAsync(h->h_out[d % 2] + (size_t)v * h->islot,
                                         pk + (size_t)v * h->islot, h->ispan[d] * sizeof(double),
                                         cudaMemcpyDeviceToHost, h->s_d2h));
            DGB_CUDA(cudaEventRecord(h->ev_d2h[d], h->s_d2h));
        }
        if (a < nch) {  // gather (unless direct) and upload chunk a
            if (!direct) {
                if (a >= 2) DGB_CUDA(cudaEventSynchronize(h->ev_h2d[a - 2]));
                host_gather(h->h_in[a % 2], h->slot_pts, u, nv, h->start[a], h->span[a]);
            }
            if (a >= 3) DGB_CUDA(cudaStreamWaitEvent(h->s_h2d, h->ev_comp[a - 3], 0));
            double *du[NV4];
            ptrs(0, a, du);
            for (int v = 0; v < nv; v++) {
                const double *src = direct ? u[v] + h->start[a]
                                           : h->h_in[a % 2] + (size_t)v * h->slot_pts;
                DGB_CUDA(cudaMemcpyAsync(du[v], src, h->span[a] * sizeof(double),
                                         cudaMemcpyHostToDevice, h->s_h2d));
            }
            DGB_CUDA(cudaEventRecord(h->ev_h2d[a], h->s_h2d));
        }
        if (e >= 0 && e < nch && !od(e)) {  // scatter chunk e's interior rows back
            DGB_CUDA(cudaEventSynchronize(h->ev_d2h[e]));
            host_scatter_rows(rhs, h->h_out[e % 2], h->islot, nv_out,
                              h->rows.data() + h->row_ptr[e], h->row_ptr[e + 1] - h->row_ptr[e],
                              h->start[e]);
        }
    }
    return DGB_OK;
}

// Whether every field lies inside dgb_host_alloc memory over the pipeline's
// extent: inputs so that the upload can read the caller's arrays, outputs
// so that the kernel can store into them.
bool fields_page_locked(const HostPipe *h, const double *const *u, int nv)
{
    if (h->members.empty()) return false;
    uint64_t lo = UINT64_MAX, hi = 0;
    for (size_t c = 0; c < h->members.size(); c++) {
        lo = std::min(lo, h->start[c]);
        hi = std::max(hi, h->start[c] + h->span[c]);
    }
    for (int v = 0; v < nv; v++)
        if (!in_host_alloc(u[v] + lo, (size_t)(hi - lo) * sizeof(double))) return false;
    return true;
}

// The upload mode of a call whose inputs are page-locked.  Reading the
// caller's arrays saves the host the gather, but the DMA rate from a large
// page-locked region has been seen to vary between hosts and to drift within
// a process, while the staging copy's does not; so the plan times both: the
// first three calls go direct (the first two untimed: the first DMA passes
// over freshly written page-locked arrays ran at a fraction of the later
// rate, 1,190 and 921 against ~605 ms per call on the 20,000-block batch),
// the fourth through the staging, later calls take the mode whose last call
// was faster and every eighth call re-times the other.
// DGB_HOST_UPLOAD=direct|staged fixes the mode.
bool choose_direct(HostPipe *h, int key)
{
    if (const char *env = getenv("DGB_HOST_UPLOAD")) {
        if (!strcmp(env, "direct")) return true;
        if (!strcmp(env, "staged")) return false;
    }
    const HostPipe::UploadStats &st = h->upload[key];
    if (st.calls < 3) return true;
    if (st.ms[0] == 0.0) return false;
    const bool best = st.ms[1] <= st.ms[0];
    return (st.calls % 8 == 7) ? !best : best;
}

// every stream of the pipeline idle
void sync_pipe(HostPipe *h)
{
    cudaStreamSynchronize(h->s_h2d);
    cudaStreamSynchronize(h->s_comp[0]);
    cudaStreamSynchronize(h->s_comp[1]);
    cudaStreamSynchronize(h->s_d2h);
}

// run_pipe_steps in the chosen upload mode, timed for the mode choice; on an
// error, a wait for the copies still in flight, so that no transfer touches
// the caller's arrays after the call returns.
template <class Compute>
dgb_status run_pipe(dgb_plan *p, double *const *rhs, const double *const *u, int nv,
                    Compute compute, int nv_out = -1)
{
    if (nv_out < 0) nv_out = nv;
    HostPipe *h = p->pipe;
    const bool locked = fields_page_locked(h, u, nv);
    const int key = nv * 64 + nv_out;
    const bool direct = locked && choose_direct(h, key);
    // Outputs in dgb_host_alloc memory while the inputs go through the
    // staging: the kernel stores the interior points into the caller's arrays
    // over the host link as it runs, which leaves the host thread only the
    // gather (gather and scatter together take longer per chunk than the
    // kernel; the stores to host memory cost the kernel about 8 %).  With
    // direct uploads the host thread has time for the scatter and the
    // download path is faster.  DGB_HOST_DOWNLOAD=copy|store fixes it.
    const char *dl = getenv("DGB_HOST_DOWNLOAD");
    const bool out_locked = fields_page_locked(h, (const double *const *)rhs, nv_out);
    const bool out_direct = out_locked && (dl && !strcmp(dl, "store")   ? true
                                           : dl && !strcmp(dl, "copy") ? false
                                                                       : !direct);
    const auto t0 = std::chrono::steady_clock::now();
    const bool out_last = out_locked && !(dl && !strcmp(dl, "copy"));
    const dgb_status s = run_pipe_steps(p, rhs, u, nv, compute, nv_out, direct, out_direct, out_last);
    if (s != DGB_OK) {
        sync_pipe(h);
        return s;
    }
    if (locked) {
        HostPipe::UploadStats &st = h->upload[key];
        if (st.calls >= 2) {  // the whole call, to its last download
            sync_pipe(h);
            st.ms[direct ? 1 : 0] = std::chrono::duration<double, std::milli>(
                                        std::chrono::steady_clock::now() - t0).count();
        }
        st.calls++;
    }
    return s;
}

// The plan's pipeline, built at first use; the sub-plans take the parent's
// schedule choice.
dgb_status ensure_pipe(dgb_plan *p)
{
    if (!p->pipe) {
        HostPipe *h = new HostPipe();
        dgb_status s = build_pipe_into(p, h);
        if (s != DGB_OK) {
            destroy_pipe(h);
            return s;
        }
        p->pipe = h;
    }
    auto same = [](const std::map<uint64_t, TileShape> &a, const std::map<uint64_t, TileShape> &b) {
        if (a.size() != b.size()) return false;
        for (auto i = a.begin(), j = b.begin(); i != a.end(); ++i, ++j)
            if (i->first != j->first || i->second.tx != j->second.tx ||
                i->second.ty != j->second.ty || i->second.tz != j->second.tz)
                return false;
        return true;
    };
    for (dgb_plan *sp : p->pipe->sub)
        for (int q = 0; q < 2; q++) {
            sp->variant[q] = p->variant[q];
            if (!same(sp->caps[q], p->caps[q])) {
                sp->caps[q] = p->caps[q];
                sp->caps_gen[q]++;
            }
        }
    return DGB_OK;
}

// The parent's 4th-order / CCZ4 workspace for the even chunks, a copy of its
// size for the odd ones (consecutive chunks may overlap on the GPU).
dgb_status pipe_scratch4(dgb_plan *p)
{
    HostPipe *h = p->pipe;
    if (h->sub.size() > 1 && h->scratch4_odd_doubles < p->scratch4_doubles) {
        cudaFree(h->d_scratch4_odd);
        h->d_scratch4_odd = nullptr;
        h->scratch4_odd_doubles = 0;
        DGB_CUDA(cudaMalloc(&h->d_scratch4_odd, p->scratch4_doubles * sizeof(double)));
        h->scratch4_odd_doubles = p->scratch4_doubles;
    }
    for (size_t c = 0; c < h->sub.size(); c++) {
        h->sub[c]->d_scratch4 = (c & 1) ? h->d_scratch4_odd : p->d_scratch4;
        h->sub[c]->scratch4_doubles = p->scratch4_doubles;
    }
    return DGB_OK;
}

// whatever happened, nothing may still be copying into the staging buffers
dgb_status finish_pipe(dgb_plan *p, dgb_status s, const char *what)
{
    HostPipe *h = p->pipe;
    cudaError_t e1 = cudaStreamSynchronize(h->s_h2d);
    cudaError_t e2 = cudaStreamSynchronize(h->s_comp[0]);
    const cudaError_t e2b = cudaStreamSynchronize(h->s_comp[1]);
    if (e2 == cudaSuccess) e2 = e2b;
    cudaError_t e3 = cudaStreamSynchronize(h->s_d2h);
    if (s != DGB_OK) return s;
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
        set_error(std::string(what) + ": " +
                  cudaGetErrorString(e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3));
        return DGB_ERR_CUDA;
    }
    return DGB_OK;
}

}  // namespace

extern "C" {

dgb_status dgb_bssn_rhs_host(dgb_plan *p, double *const *rhs, const double *const *u, int precision)
{
    if (!p || !rhs || !u) {
        set_error("dgb_bssn_rhs_host: null argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV; v++)
        if (!rhs[v] || !u[v]) {
            set_error("dgb_bssn_rhs_host: null field pointer");
            return DGB_ERR_INVALID;
        }
    if (precision != DGB_PREC_FP64 && precision != DGB_PREC_MIXED) {
        set_error("precision must be DGB_PREC_FP64 or DGB_PREC_MIXED");
        return DGB_ERR_INVALID;
    }
    if (p->blocks.empty()) return DGB_OK;
    if (p->prm.fd_order == 4 && precision != DGB_PREC_FP64) {
        set_error("dgb_bssn_rhs_host: fd_order 4 runs in FP64 only");
        return DGB_ERR_UNSUPPORTED;
    }
    // fd_order 4: the chunks run on the parent's 4th-order workspace and its odd copy
    dgb_status s = p->prm.fd_order == 4 ? b4_workspace(p) : DGB_OK;
    if (s == DGB_OK) s = ensure_pipe(p);
    if (s == DGB_OK && p->prm.fd_order == 4) s = pipe_scratch4(p);
    if (s != DGB_OK) return s;
    if (p->prm.fd_order == 4)
        for (dgb_plan *sp : p->pipe->sub) sp->b4_occupancy = p->b4_occupancy;
    const int variant = p->variant[precision == DGB_PREC_MIXED ? 1 : 0];
    s = run_pipe(p, rhs, u, NV,
                 [&](dgb_plan *sp, double *const *dr, const double *const *du, cudaStream_t st) {
                     return run_rhs(sp, dr, du, precision, variant, st);
                 });
    return finish_pipe(p, s, "dgb_bssn_rhs_host");
}

dgb_status dgb_ccz4_rhs_host(dgb_plan *p, const dgb_ccz4_params *prm, double *const *rhs,
                             const double *const *u, int precision)
{
    if (!p || !prm || !rhs || !u) {
        set_error("dgb_ccz4_rhs_host: null argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV4; v++)
        if (!rhs[v] || !u[v]) {
            set_error("dgb_ccz4_rhs_host: null field pointer");
            return DGB_ERR_INVALID;
        }
    if (precision != DGB_PREC_FP64 && precision != DGB_PREC_MIXED) {
        set_error("precision must be DGB_PREC_FP64 or DGB_PREC_MIXED");
        return DGB_ERR_INVALID;
    }
    if (p->blocks.empty()) return DGB_OK;
    // the chunks run on the parent's CCZ4 workspace and its odd copy
    dgb_status s = c4_workspace(p, precision);
    if (s == DGB_OK) s = ensure_pipe(p);
    if (s == DGB_OK) s = pipe_scratch4(p);
    if (s != DGB_OK) return s;
    const int pq = precision == DGB_PREC_MIXED ? 1 : 0;
    for (dgb_plan *sp : p->pipe->sub) sp->c4_occupancy[pq] = p->c4_occupancy[pq];
    s = run_pipe(p, rhs, u, NV4,
                 [&](dgb_plan *sp, double *const *dr, const double *const *du, cudaStream_t st) {
                     return dgb_ccz4_rhs(sp, prm, dr, du, precision, st);
                 });
    return finish_pipe(p, s, "dgb_ccz4_rhs_host");
}

dgb_status dgb_physical_constraints_host(dgb_plan *p, double *const *cons, const double *const *u)
{
    if (!p || !cons || !u) {
        set_error("dgb_physical_constraints_host: null argument");
        return DGB_ERR_INVALID;
    }
    for (int v = 0; v < NV; v++)
        if (!u[v]) {
            set_error("dgb_physical_constraints_host: null field pointer");
            return DGB_ERR_INVALID;
        }
    for (int c = 0; c < DGB_NUM_CONSTRAINTS; c++)
        if (!cons[c]) {
            set_error("dgb_physical_constraints_host: null output pointer");
            return DGB_ERR_INVALID;
        }
    if (p->blocks.empty()) return DGB_OK;
    dgb_status s = ensure_pipe(p);
    if (s != DGB_OK) return s;
    s = run_pipe(
        p, cons, u, NV,
        [&](dgb_plan *sp, double *const *dr, const double *const *du, cudaStream_t st) {
            return dgb_physical_constraints(sp, dr, du, st);
        },
        DGB_NUM_CONSTRAINTS);
    return finish_pipe(p, s, "dgb_physical_constraints_host");
}

dgb_status dgb_bssnrhs_block_host(double *const *rhs, const double *const *u, uint64_t offset,
                                  const double *ptmin, const double *ptmax, const uint32_t *sz,
                                  uint32_t bflag, const dgb_bssn_params *prm, int precision)
{
    if (!rhs || !u || !ptmin || !ptmax || !sz || !prm) {
        set_error("dgb_bssnrhs_block_host: null argument");
        return DGB_ERR_INVALID;
    }
    dgb_block_desc d;
    memset(&d, 0, sizeof d);
    d.offset = 0;
    for (int a = 0; a < 3; a++) {
        d.sz[a] = sz[a];
        d.ptmin[a] = ptmin[a];
        d.ptmax[a] = ptmax[a];
    }
    d.bflag = bflag;
    dgb_plan *p = nullptr;
    dgb_status s = dgb_plan_create(&d, 1, prm, &p);
    if (s != DGB_OK) return s;
    const double *uo[NV];
    double *ro[NV];
    for (int v = 0; v < NV; v++) {
        uo[v] = u[v] + offset;
        ro[v] = rhs[v] + offset;
    }
    s = dgb_bssn_rhs_host(p, ro, uo, precision);
    dgb_plan_destroy(p);
    return s;
}

dgb_status dgb_rk4_stage(int stage, double *const *dst, const double *const *prev,
                         const double *const *k, uint64_t nnodes, double dt, double chi_floor,
                         void *stream)
{
    if (stage < 0 || stage > 3 || !dst || !prev || !k) {
        set_error("dgb_rk4_stage: bad argument");
        return DGB_ERR_INVALID;
    }
    if (nnodes == 0) return DGB_OK;
    static unsigned int *d_status = nullptr;
    if (!d_status) DGB_CUDA(cudaMalloc(&d_status, sizeof(unsigned int)));
    cudaStream_t st = (cudaStream_t)stream;
    DGB_CUDA(cudaMemsetAsync(d_status, 0, sizeof(unsigned int), st));
    DGB_CUDA(rk4_launch(stage, dst, prev, k, nnodes, dt, chi_floor, d_status, st));
    unsigned int h = 0;
    DGB_CUDA(cudaMemcpyAsync(&h, d_status, sizeof h, cudaMemcpyDeviceToHost, st));
    DGB_CUDA(cudaStreamSynchronize(st));
    if (h & 1u) {
        set_error("dgb_rk4_stage: det(gt) <= 0 at some node (the reference exits here)");
        return DGB_ERR_CONSTRAINT;
    }
    return DGB_OK;
}

dgb_status dgb_synth_fill_device(dgb_plan *p, double *const *u, uint64_t seed, double noise,
                                 void *stream)
{
    if (!p || !u) return DGB_ERR_INVALID;
    if (p->blocks.empty()) return DGB_OK;
    DGB_CUDA(synth_fill_launch(p->d_blocks, (uint32_t)p->blocks.size(), p->d_first, p->unzipped, u,
                               0, NV, seed, noise, (cudaStream_t)stream));
    return DGB_OK;
}

dgb_status dgb_synth_fill_var_device(dgb_plan *p, int var, double *dst, uint64_t seed, double noise,
                                     void *stream)
{
    if (!p || !dst || var < 0 || var > NV) return DGB_ERR_INVALID;
    if (p->blocks.empty()) return DGB_OK;
    double *u[1] = {dst};
    DGB_CUDA(synth_fill_launch(p->d_blocks, (uint32_t)p->blocks.size(), p->d_first, p->unzipped, u,
                               var, var + 1, seed, noise, (cudaStream_t)stream));
    return DGB_OK;
}

}  // extern "C"
