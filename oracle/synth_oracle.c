/* ORACLE — test infrastructure only.  The seeded synthetic workloads, restated
 * in plain C so that the CPU arms of the benchmark (the reference path on the
 * host cores) build their inputs without the CUDA library: block lists of the
 * 512-block and 20,000-block workloads and the Brill-Lindquist + noise fill.
 * The generator is this project's own benchmark definition (not reference
 * code); tests check these functions against the library's bit for bit.
 *
 * Brill-Lindquist two-puncture data is the zero-momentum, zero-spin case of
 * the reference's punctureData (BSSN_GR/src/grUtils.cpp:398-712):
 *   psi = 1 + sum_i m_i / (2 r_i), chi = psi^-4, alpha = psi^-2, gt = delta,
 *   K = At = Gt = beta = B = 0, chi and alpha floored at 1e-4,
 * masses 0.5 at (+-1, 0, 0.00123), plus U(-1,1) * noise from a counter-based
 * SplitMix64 keyed by (seed, block, variable, point).  Build with
 * -ffp-contract=off: every operation rounds once. */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct {
    uint64_t offset;
    uint32_t sz[3];
    uint32_t bflag;
    double ptmin[3];
    double ptmax[3];
} orc_block;

#define CHI_FLOOR 1e-4
#define PUNCTURE_Z 0.00123

static uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static double unit_noise(uint64_t key, uint64_t point)
{
    const uint64_t r = mix64(key ^ mix64(point));
    return 2.0 * ((double)(r >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
}

static uint64_t noise_key(uint64_t seed, uint64_t block, uint32_t var)
{
    return mix64(mix64(seed ^ 0xD1B54A32D192ED03ull) ^ (block * 64u + var));
}

static double bl_value(int v, double x, double y, double z)
{
    if (v == 0 || v == 1) {
        const double zz = z - PUNCTURE_Z;
        const double dx1 = x - 1.0, dx2 = x + 1.0;
        const double yz = y * y + zz * zz;
        const double r1 = sqrt(dx1 * dx1 + yz), r2 = sqrt(dx2 * dx2 + yz);
        const double psi = (1.0 + 0.5 / (2.0 * r1)) + 0.5 / (2.0 * r2);
        const double psi2 = psi * psi;
        const double f = v == 0 ? 1.0 / psi2 : 1.0 / (psi2 * psi2);
        return f < CHI_FLOOR ? CHI_FLOOR : f;
    }
    if (v == 12 || v == 15 || v == 17) return 1.0;
    return 0.0;
}

/* which = 1: 512 blocks of 13^3 tiled 8x8x8 over [-1.2, 1.2]^3 at dx = 0.05;
 * which = 2: 20,000 blocks (14,000 x 13^3, 4,000 x 19^3, 1,600 x 31^3,
 * 400 x 61^3) shuffled, levels 4-10 on [-32, 32]^3, half near a puncture.
 * Returns the count; fills out when it is not NULL. */
long orc_synth_blocks(int which, uint64_t seed, orc_block *out)
{
    if (which == 1) {
        const double dx = 0.05;
        uint64_t off = 0;
        long n = 0;
        for (int k = 0; k < 8; k++)
            for (int j = 0; j < 8; j++)
                for (int i = 0; i < 8; i++, n++) {
                    if (!out) continue;
                    orc_block b;
                    memset(&b, 0, sizeof b);
                    const int ijk[3] = {i, j, k};
                    for (int d = 0; d < 3; d++) {
                        const double x0 = -1.2 + 0.3 * ijk[d];
                        b.sz[d] = 13;
                        b.ptmin[d] = x0 - 3 * dx;
                        b.ptmax[d] = x0 + 9 * dx;
                    }
                    b.offset = off;
                    off += 13ull * 13 * 13;
                    out[n] = b;
                }
        return n;
    }
    if (which != 2) return -1;
    enum { NB = 20000 };
    if (!out) return NB;
    static const int counts[4] = {14000, 4000, 1600, 400};
    static const uint32_t sides[4] = {13, 19, 31, 61};
    static uint32_t side[NB];
    long m = 0;
    for (int c = 0; c < 4; c++)
        for (int q = 0; q < counts[c]; q++) side[m++] = sides[c];
    for (size_t i = NB - 1; i > 0; i--) {  /* Fisher-Yates on the counter generator */
        const uint64_t r = mix64(seed * 0x9E37ull + i);
        const size_t j = (size_t)(r % (i + 1));
        const uint32_t t = side[i];
        side[i] = side[j];
        side[j] = t;
    }
    uint64_t off = 0;
    for (long b = 0; b < NB; b++) {
        const uint64_t r0 = mix64(mix64(seed) ^ (0xB10C0000ull + (uint64_t)b));
        const int L = 4 + (int)(r0 % 7);
        const double dx = 64.0 / ((double)(1u << L) * 6.0);
        const double ext = (side[b] - 7) * dx;
        const int near = (int)((r0 >> 8) & 1);
        const double px = ((r0 >> 9) & 1) ? 1.0 : -1.0;
        orc_block d;
        memset(&d, 0, sizeof d);
        for (int a = 0; a < 3; a++) {
            const uint64_t ra = mix64(r0 + 0x51ull * (uint64_t)(a + 1));
            const double u01 = (double)(ra >> 11) * (1.0 / 9007199254740992.0);
            double x0;
            if (near) {
                const double R = 2.0 * (double)(1u << (10 - L));
                const double c = a == 0 ? px : (a == 2 ? PUNCTURE_Z : 0.0);
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
        off += (uint64_t)side[b] * side[b] * side[b];
        out[b] = d;
    }
    return NB;
}

/* Fields 0 .. nvars-1 of every block: u[v][offset + i + nx (j + ny k)] at
 * x = ptmin + i h (h = (ptmax - ptmin)/(n - 1)); the noise of block b is
 * keyed by b, the block's place in this list. */
void orc_synth_fill(const orc_block *blocks, long nblk, double *const *u, int nvars, uint64_t seed,
                    double noise, int nthreads)
{
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (long b = 0; b < nblk; b++) {
        const orc_block *d = &blocks[b];
        const int nx = (int)d->sz[0], ny = (int)d->sz[1], nz = (int)d->sz[2];
        double h[3];
        for (int a = 0; a < 3; a++) h[a] = (d->ptmax[a] - d->ptmin[a]) / (double)(d->sz[a] - 1);
        for (int v = 0; v < nvars; v++) {
            const uint64_t key = noise_key(seed, (uint64_t)b, (uint32_t)v);
            double *dst = u[v] + d->offset;
            for (int k = 0; k < nz; k++)
                for (int j = 0; j < ny; j++)
                    for (int i = 0; i < nx; i++) {
                        const uint64_t p = (uint64_t)i + (uint64_t)nx * ((uint64_t)j + (uint64_t)ny * k);
                        const double x = d->ptmin[0] + (double)i * h[0];
                        const double y = d->ptmin[1] + (double)j * h[1];
                        const double z = d->ptmin[2] + (double)k * h[2];
                        dst[p] = bl_value(v, x, y, z) + noise * unit_noise(key, p);
                    }
        }
    }
}
