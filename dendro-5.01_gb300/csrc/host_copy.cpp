// Host side of the pipelined host-array entry points: the copies between
// the caller's field arrays and the library's pinned staging buffers, spread
// over all host threads (OpenMP).  A staging buffer holds one chunk of
// blocks as NV field planes of `slot_pts` doubles, plane v at v * slot_pts,
// point p of the chunk at (offset - chunk start).
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "../../include/dendro_gb300.h"

namespace dgb {

// dst[v * slot_pts + i] = u[v][start + i] for i < span
void host_gather(double *dst, size_t slot_pts, const double *const *u, int nv, uint64_t start,
                 uint64_t span)
{
    const size_t piece = (size_t)1 << 16;  // 512 KiB per task
    const long npieces = (long)((span + piece - 1) / piece);
#pragma omp parallel for schedule(dynamic, 4)
    for (long t = 0; t < (long)nv * npieces; t++) {
        const int v = (int)(t / npieces);
        const size_t b = (size_t)(t % npieces) * piece;
        const size_t n = std::min<size_t>(piece, span - b);
        memcpy(dst + (size_t)v * slot_pts + b, u[v] + start + b, n * sizeof(double));
    }
}

// The interior points of every block of the chunk go back to rhs; the
// padding of rhs is not written (the reference leaves it untouched).
void host_scatter_interior(double *const *rhs, const double *src, size_t slot_pts, int nv,
                           const dgb_block_desc *blocks, const uint32_t *members, size_t nmem,
                           uint64_t start)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (long t = 0; t < (long)nv * (long)nmem; t++) {
        const int v = (int)(t / (long)nmem);
        const dgb_block_desc &d = blocks[members[t % (long)nmem]];
        const size_t nx = d.sz[0], ny = d.sz[1], nz = d.sz[2];
        const size_t row = (nx - 6) * sizeof(double);
        double *out = rhs[v] + d.offset;
        const double *in = src + (size_t)v * slot_pts + (d.offset - start);
        for (size_t k = 3; k < nz - 3; k++)
            for (size_t j = 3; j < ny - 3; j++) {
                const size_t o = 3 + nx * (j + ny * k);
                memcpy(out + o, in + o, row);
            }
    }
}

}  // namespace dgb
