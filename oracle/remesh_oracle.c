/* Test infrastructure only (the oracle): CPU restatement of the wavelet
 * refinement indicator of the octree mesh, element order 6.
 *
 *   Mesh::isReMeshUnzip              include/mesh.tcc:2035-2197
 *   WaveletEl::WaveletEl             src/waveletRefEl.cpp:15-80
 *   WaveletEl::compute_wavelets_3D   src/waveletRefEl.cpp:92-271
 *   RefElement::I3D_Parent2Child     FEM/include/refel.h:249-296 (x, y, z passes)
 *   uniform element nodes            FEM/src/refel.cpp:87, 105-106
 *
 * Parity against the reference binary is unpinned: the wavelet element needs
 * the reference's RefElement (LAPACK builds its interpolation matrices) and
 * the MPI headers, neither of which is available here.  The restatement is
 * pinned by known answers instead (tests/test_remesh_oracle.py): the
 * wavelets vanish to rounding for polynomials of degree <= 6 on interior
 * elements and <= 3 on boundary elements, and equal the analytic
 * interpolation error prod(x - x_b) for x^7 and x^4.
 *
 * Deliberate differences from the reference, at the rounding level only:
 *   - the 1-D interpolation matrices are the Lagrange weights of the uniform
 *     parent nodes at the child nodes, each formed as one correctly rounded
 *     quotient of two exact integers (the reference inverts a Vandermonde
 *     matrix with LAPACK, which is accurate to a few ulp);
 *   - each interpolated value is one fused multiply-add chain over the
 *     parent nodes in ascending order (first term a plain product).
 * Everything else (patch layout, which nodes are parents and which are
 * wavelets, the relative form |u - Pu| / max(1, |u|), the RMS over the 64
 * wavelet slots, the per-variable early exit, the flag thresholds) follows the
 * reference step by step. */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define P 6                /* element order */
#define NP (P + 1)         /* parent nodes per axis, interior element */
#define PW (P / 2)         /* padding width of the unzipped patch */
#define PATCH (2 * P + 1)  /* 13: side of an element's padded patch */
#define BP (P / 2)         /* order of the boundary element's parent (3) */
#define BNP (BP + 1)       /* its parent nodes per axis */
#define BCH (2 * BP + 1)   /* its child grid per axis */
#define NWC 64             /* wavelet slots (4^3), zero-filled for boundary elements */

/* Lagrange weight of node a of nn uniform nodes 0..nn-1 at x = tx / 2:
 * prod_{b != a} (tx - 2b) / prod_{b != a} (2a - 2b), both exact integers. */
static double lagrange_w(int nn, int tx, int a)
{
    int64_t num = 1, den = 1;
    for (int b = 0; b < nn; b++) {
        if (b == a) continue;
        num *= (int64_t)(tx - 2 * b);
        den *= (int64_t)(2 * a - 2 * b);
    }
    return (double)num / (double)den;
}

/* child c (0 or 1) of an order-p element: row m is the child node m, at
 * parent coordinate (c * p + m) / 2 in parent node units */
static void child_matrix(int p, int c, double *ip)
{
    for (int m = 0; m <= p; m++)
        for (int a = 0; a <= p; a++) ip[m * (p + 1) + a] = lagrange_w(p + 1, c * p + m, a);
}

static double dot_fma(const double *w, const double *x, int sx, int n)
{
    double t = w[0] * x[0];
    for (int a = 1; a < n; a++) t = fma(w[a], x[a * sx], t);
    return t;
}

/* I3D_Parent2Child: out[m3][m2][m1] for the child with bits (cx, cy, cz), np
 * nodes per axis, x pass, then y, then z. */
static void parent_to_child(int np, const double *ipx, const double *ipy, const double *ipz,
                            const double *in, double *im1, double *im2, double *out)
{
    for (int k = 0; k < np; k++)
        for (int j = 0; j < np; j++)
            for (int m = 0; m < np; m++)
                im1[(k * np + j) * np + m] = dot_fma(ipx + m * np, in + (k * np + j) * np, 1, np);
    for (int k = 0; k < np; k++)
        for (int m = 0; m < np; m++)
            for (int i = 0; i < np; i++)
                im2[(k * np + m) * np + i] = dot_fma(ipy + m * np, im1 + k * np * np + i, np, np);
    for (int m = 0; m < np; m++)
        for (int j = 0; j < np; j++)
            for (int i = 0; i < np; i++)
                out[(m * np + j) * np + i] = dot_fma(ipz + m * np, im2 + j * np + i, np * np, np);
}

static double max1(double a) { return 1.0 < a ? a : 1.0; } /* std::max(1.0, a) */

/* compute_wavelets_3D on one element's 13^3 patch (x fastest): the 64
 * relative wavelet slots, boundary elements fill the first 27. */
void orc_wavelet_patch(const double *in, int boundary, double *wc)
{
    double vin[NP * NP * NP], nvec[NP * NP * NP], im1[NP * NP * NP], im2[NP * NP * NP];
    double vout[PATCH * PATCH * PATCH];
    double ip[2][NP * NP];
    for (int i = 0; i < NWC; i++) wc[i] = 0.0;

    if (boundary) {
        /* order-3 element on the leaf's own nodes: parents at 3, 5, 7, 9,
         * wavelets at 4, 6, 8 (waveletRefEl.cpp:117-185) */
        child_matrix(BP, 0, ip[0]);
        child_matrix(BP, 1, ip[1]);
        for (int k = 0; k < BNP; k++)
            for (int j = 0; j < BNP; j++)
                for (int i = 0; i < BNP; i++)
                    vin[(k * BNP + j) * BNP + i] =
                        in[(PW + 2 * k) * PATCH * PATCH + (PW + 2 * j) * PATCH + PW + 2 * i];
        for (int c = 0; c < 8; c++) {
            const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
            parent_to_child(BNP, ip[bx], ip[by], ip[bz], vin, im1, im2, nvec);
            for (int k = 0; k < BNP; k++)
                for (int j = 0; j < BNP; j++)
                    for (int i = 0; i < BNP; i++)
                        vout[((BP * bz + k) * BCH + BP * by + j) * BCH + BP * bx + i] =
                            nvec[(k * BNP + j) * BNP + i];
        }
        int w = 0;
        for (int k = PW + 1; k < PW + P + 1; k += 2)
            for (int j = PW + 1; j < PW + P + 1; j += 2)
                for (int i = PW + 1; i < PW + P + 1; i += 2, w++) {
                    const double u = in[k * PATCH * PATCH + j * PATCH + i];
                    const double o = vout[((k - PW) * BCH + (j - PW)) * BCH + (i - PW)];
                    wc[w] = fabs(u - o) / max1(fabs(u));
                }
        return;
    }

    /* interior: parents at the even patch indices 0..12, wavelets at 3, 5, 7, 9
     * (waveletRefEl.cpp:191-255) */
    child_matrix(P, 0, ip[0]);
    child_matrix(P, 1, ip[1]);
    for (int k = 0; k < NP; k++)
        for (int j = 0; j < NP; j++)
            for (int i = 0; i < NP; i++)
                vin[(k * NP + j) * NP + i] = in[(2 * k) * PATCH * PATCH + (2 * j) * PATCH + 2 * i];
    for (int c = 0; c < 8; c++) {
        const int bx = c & 1, by = (c >> 1) & 1, bz = (c >> 2) & 1;
        parent_to_child(NP, ip[bx], ip[by], ip[bz], vin, im1, im2, nvec);
        for (int k = 0; k < NP; k++)
            for (int j = 0; j < NP; j++)
                for (int i = 0; i < NP; i++)
                    vout[((P * bz + k) * PATCH + P * by + j) * PATCH + P * bx + i] =
                        nvec[(k * NP + j) * NP + i];
    }
    int w = 0;
    for (int k = PW; k < P + PW + 1; k += 2)
        for (int j = PW; j < P + PW + 1; j += 2)
            for (int i = PW; i < P + PW + 1; i += 2, w++) {
                const int pp = k * PATCH * PATCH + j * PATCH + i;
                wc[w] = fabs(vout[pp] - in[pp]) / max1(fabs(in[pp]));
            }
}

/* normL2(wc, 64) / sqrt(64) (include/mathUtils.tcc:51-65) */
double orc_wavelet_rms(const double *wc)
{
    double l2 = 0.0;
    for (int i = 0; i < NWC; i++) {
        if (isnan(wc[i])) return NAN;
        l2 += wc[i] * wc[i];
    }
    return sqrt(l2) / sqrt((double)NWC);
}

/* isReMeshUnzip over a leaf list.  Per leaf e: its patch starts at
 * patch_base[e] in every unzipped field, rows of block_side[e] points;
 * boundary[e] selects the boundary element; tol[e] is wavelet_tol at the
 * leaf.  wmax[e] = eleWMax, flags[e] = OCT_SPLIT (1) if wmax > tol,
 * OCT_COARSE (2) if wmax < coarse_fac * tol, else OCT_NO_CHANGE (0).
 * Returns the number of leaves flagged split or coarse. */
uint64_t orc_remesh_wavelets(const double *const *unzipped, const uint32_t *var_ids, int nvars,
                             uint64_t nleaves, const uint64_t *patch_base,
                             const uint32_t *block_side, const uint8_t *boundary, const double *tol,
                             double coarse_fac, double *wmax, uint8_t *flags, int nthreads)
{
    uint64_t changed = 0;
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads) reduction(+ : changed)
    for (int64_t e = 0; e < (int64_t)nleaves; e++) {
        double patch[PATCH * PATCH * PATCH], wc[NWC];
        const uint64_t n = block_side[e];
        double wm = 0.0;
        for (int v = 0; v < nvars; v++) {
            const double *u = unzipped[var_ids[v]] + patch_base[e];
            for (int k = 0; k < PATCH; k++)
                for (int j = 0; j < PATCH; j++)
                    memcpy(patch + (k * PATCH + j) * PATCH, u + (uint64_t)k * n * n + (uint64_t)j * n,
                           PATCH * sizeof(double));
            orc_wavelet_patch(patch, boundary[e], wc);
            const double l = orc_wavelet_rms(wc);
            if (wm < l) wm = l;
            if (wm > tol[e]) break;
        }
        wmax[e] = wm;
        uint8_t f = 0;
        if (wm > tol[e])
            f = 1;
        else if (wm < coarse_fac * tol[e])
            f = 2;
        flags[e] = f;
        changed += f != 0;
    }
    return changed;
}
