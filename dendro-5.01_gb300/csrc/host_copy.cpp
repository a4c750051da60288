// Host side of the pipelined host-array entry points: the copies between
// the caller's field arrays and the library's pinned staging buffers, spread
// over all host threads (OpenMP).  An upload staging buffer holds one chunk
// of blocks as field planes of `slot_pts` doubles, plane v at v * slot_pts,
// point p of the chunk at (offset - chunk start); a download staging buffer
// holds the chunk's interior rows packed, plane v at v * islot.
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "../../include/dendro_gb300.h"
#include "host_rows.h"

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

// rhs[v][start + row.src ...] = src[v * islot + row.dst ...] for each interior
// row of the chunk (the packed download)
void host_scatter_rows(double *const *rhs, const double *src, size_t islot, int nv,
                       const IRow *rows, size_t nrows, uint64_t start)
{
    const long piece = 256;  // rows per task
    const long npieces = (long)((nrows + piece - 1) / piece);
#pragma omp parallel for schedule(dynamic, 4)
    for (long t = 0; t < (long)nv * npieces; t++) {
        const int v = (int)(t / npieces);
        const size_t r0 = (size_t)(t % npieces) * piece;
        const size_t r1 = std::min<size_t>(nrows, r0 + piece);
        double *out = rhs[v] + start;
        const double *in = src + (size_t)v * islot;
        for (size_t r = r0; r < r1; r++)
            memcpy(out + rows[r].src, in + rows[r].dst, rows[r].len * sizeof(double));
    }
}

}  // namespace dgb
