// Host side of the synthetic workloads: block lists and the seeded
// Brill-Lindquist + noise fill (bit-identical to the device fill, see
// synth.cuh).  Compiled with -ffp-contract=off.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/dendro_gb300.h"
#include "synth.cuh"

namespace {

// Uniform 13^3 tiling used by the 512-block workload: block (i,j,k) owns the
// nodes [x0, x0 + 6 dx] per axis with x0 = -1.2 + 0.3 i and carries a 3-point
// pad, ptmin = x0 - 3dx, ptmax = x0 + 9dx, so h = (ptmax-ptmin)/12 = dx
// (the convention of BSSN_GR/src/rhs.cpp:56-62, :148-150).
void blocks_uniform512(std::vector<dgb_block_desc> &out)
{
    const double dx = 0.05;
    uint64_t off = 0;
    for (int k = 0; k < 8; k++)
        for (int j = 0; j < 8; j++)
            for (int i = 0; i < 8; i++) {
                dgb_block_desc b;
                memset(&b, 0, sizeof b);
                const int ijk[3] = {i, j, k};
                for (int d = 0; d < 3; d++) {
                    const double x0 = -1.2 + 0.3 * ijk[d];
                    b.sz[d] = 13;
                    b.ptmin[d] = x0 - 3 * dx;
                    b.ptmax[d] = x0 + 9 * dx;
                }
                b.offset = off;
                b.bflag = 0;
                off += 13ull * 13 * 13;
                out.push_back(b);
            }
}

// 20,000 blocks: 14,000 x 13^3, 4,000 x 19^3, 1,600 x 31^3, 400 x 61^3,
// shuffled.  Level L in [4,10] gives dx = 64 / (2^L * 6) on [-32,32]^3
// (ot::Block::computeDx, src/block.cpp:85-98, eleOrder 6).  Half the blocks
// sit within 2 * 2^(10-L) of a puncture, the rest anywhere in the domain;
// block corners are snapped to the level's lattice.
void blocks_uneven20k(uint64_t seed, std::vector<dgb_block_desc> &out)
{
    const int counts[4] = {14000, 4000, 1600, 400};
    const uint32_t sides[4] = {13, 19, 31, 61};
    std::vector<uint32_t> side;
    for (int c = 0; c < 4; c++) side.insert(side.end(), counts[c], sides[c]);
    // Fisher-Yates with the counter-based generator
    for (size_t i = side.size() - 1; i > 0; i--) {
        const uint64_t r = dgb_mix64(seed * 0x9E37ull + i);
        const size_t j = (size_t)(r % (i + 1));
        std::swap(side[i], side[j]);
    }
    uint64_t off = 0;
    for (size_t b = 0; b < side.size(); b++) {
        const uint64_t r0 = dgb_mix64(dgb_mix64(seed) ^ (0xB10C0000ull + b));
        const int L = 4 + (int)(r0 % 7);
        const double dx = 64.0 / ((double)(1u << L) * 6.0);
        const double ext = (side[b] - 7) * dx;  // owned extent
        const bool near = ((r0 >> 8) & 1) != 0;
        const double px = ((r0 >> 9) & 1) ? 1.0 : -1.0;
        dgb_block_desc d;
        memset(&d, 0, sizeof d);
        for (int a = 0; a < 3; a++) {
            const uint64_t ra = dgb_mix64(r0 + 0x51ull * (a + 1));
            const double u01 = (double)(ra >> 11) * (1.0 / 9007199254740992.0);
            double x0;
            if (near) {
                const double R = 2.0 * (double)(1u << (10 - L));
                const double c = (a == 0) ? px : (a == 2 ? DGB_SYNTH_PUNCTURE_Z : 0.0);
                x0 = c + (2.0 * u01 - 1.0) * R - 0.5 * ext;
            } else {
                x0 = -32.0 + u01 * (64.0 - ext);
            }
            if (x0 < -32.0) x0 = -32.0;
            if (x0 > 32.0 - ext) x0 = 32.0 - ext;
            x0 = -32.0 + dx * floor((x0 + 32.0) / dx);
            d.sz[a] = side[b];
            d.ptmin[a] = x0 - 3 * dx;
            d.ptmax[a] = x0 + ext + 3 * dx;
        }
        d.offset = off;
        d.bflag = 0;
        off += (uint64_t)side[b] * side[b] * side[b];
        out.push_back(d);
    }
}

}  // namespace

extern "C" dgb_status dgb_synth_blocks(int which, uint64_t seed, dgb_block_desc *blocks,
                                       size_t *nblk)
{
    if (!nblk) return DGB_ERR_INVALID;
    std::vector<dgb_block_desc> v;
    if (which == 1) {
        blocks_uniform512(v);
    } else if (which == 2) {
        blocks_uneven20k(seed, v);
    } else {
        return DGB_ERR_INVALID;
    }
    if (blocks) {
        if (*nblk < v.size()) return DGB_ERR_INVALID;
        memcpy(blocks, v.data(), v.size() * sizeof(dgb_block_desc));
    }
    *nblk = v.size();
    return DGB_OK;
}

extern "C" dgb_status dgb_synth_fill_host(const dgb_block_desc *blocks, size_t nblk,
                                          double *const *u, uint64_t seed, double noise,
                                          int nthreads)
{
    if (!blocks || !u) return DGB_ERR_INVALID;
    for (int v = 0; v < DGB_NUM_VARS; v++)
        if (!u[v]) return DGB_ERR_INVALID;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
#endif
    for (long b = 0; b < (long)nblk; b++) {
        const dgb_block_desc &d = blocks[b];
        const int nx = d.sz[0], ny = d.sz[1], nz = d.sz[2];
        double h[3];
        for (int a = 0; a < 3; a++) h[a] = (d.ptmax[a] - d.ptmin[a]) / (double)(d.sz[a] - 1);
        for (int v = 0; v < DGB_NUM_VARS; v++) {
            const uint64_t key = dgb_noise_key(seed, (uint64_t)b, (uint32_t)v);
            double *dst = u[v] + d.offset;
            for (int k = 0; k < nz; k++)
                for (int j = 0; j < ny; j++)
                    for (int i = 0; i < nx; i++) {
                        const uint64_t p = (uint64_t)i + (uint64_t)nx * (j + (uint64_t)ny * k);
                        dst[p] = dgb_synth_value(v, key, p, i, j, k, d.ptmin, h, noise);
                    }
        }
    }
    (void)nthreads;
    return DGB_OK;
}

extern "C" dgb_status dgb_synth_fill_var_host(const dgb_block_desc *blocks, size_t nblk, int var,
                                              double *dst, uint64_t seed, double noise,
                                              int nthreads)
{
    if (!blocks || !dst || var < 0 || var > DGB_NUM_VARS) return DGB_ERR_INVALID;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
#endif
    for (long b = 0; b < (long)nblk; b++) {
        const dgb_block_desc &d = blocks[b];
        const int nx = d.sz[0], ny = d.sz[1], nz = d.sz[2];
        double h[3];
        for (int a = 0; a < 3; a++) h[a] = (d.ptmax[a] - d.ptmin[a]) / (double)(d.sz[a] - 1);
        const uint64_t key = dgb_noise_key(seed, (uint64_t)b, (uint32_t)var);
        double *out = dst + d.offset;
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    const uint64_t p = (uint64_t)i + (uint64_t)nx * (j + (uint64_t)ny * k);
                    out[p] = dgb_synth_value(var, key, p, i, j, k, d.ptmin, h, noise);
                }
    }
    (void)nthreads;
    return DGB_OK;
}

extern "C" dgb_status dgb_synth_fill_points_host(const double *xyz, uint64_t n, double *const *u,
                                                 uint64_t seed, double noise, int nthreads)
{
    if ((!xyz && n) || !u) return DGB_ERR_INVALID;
    for (int v = 0; v < DGB_NUM_VARS; v++)
        if (!u[v]) return DGB_ERR_INVALID;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (long long p = 0; p < (long long)n; p++) {
        const double x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
        for (int v = 0; v < DGB_NUM_VARS; v++) {
            const uint64_t key = dgb_noise_key(seed, (uint64_t)p, (uint32_t)v);
            u[v][p] = SY_ADD(dgb_bl_value(v, x, y, z), SY_MUL(noise, dgb_noise_unit(key, 0)));
        }
    }
    (void)nthreads;
    return DGB_OK;
}
