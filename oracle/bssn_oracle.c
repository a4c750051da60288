/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the
 * reference's per-block BSSN hot path, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker
 * and CPU timing arm.  Never linked into, or called by, the product library.
 *
 * Parity pin: tests/test_oracle.py compares every function here with the
 * reference's own code compiled from its sources (oracle/Makefile.ref,
 * machines that hold the reference tree) and with the golden vectors in
 * tests/golden/ that the same reference build produced.
 *
 * What follows which reference lines:
 *   stencils      QuadGrav/src/derivs.cpp:2141-2953 (deriv64_*, centred
 *                 "advective" = deriv64), BSSN_GR/src/derivs.cpp:914-1410
 *                 (ko_deriv42_*), with the reference loop ranges and the
 *                 one-sided closures of flagged faces; for the BSSN_GR
 *                 solver's 4th-order binding (BSSN_GR/include/rhs.h:23-37)
 *                 deriv42_* and the upwinded deriv42adv_* (BSSN_GR/src/
 *                 derivs.cpp:11-913, restated in physcon_oracle.c and
 *                 ccz4_oracle.c).
 *   BCs           bssn_bcs (BSSN_GR/src/rhs.cpp:838-982) on flagged faces.
 *   rhs driver    BSSN_GR/src/rhs.cpp:86-392 (bssnrhs: h = (pmax-pmin)/(n-1),
 *                 derivative staging per BSSN_GR/scripts/bssnrhs_derivs.h,
 *                 eta(r) at rhs.cpp:219-223, KO accumulate at :336-373).
 *   point algebra the BSSN system of CodeGen/bssn.py:36-96 with the tensor
 *                 helpers of CodeGen/dendro.py (lie :211, trace_free :317,
 *                 DiDj :160, laplacian :259, sqr :305, up_up :188,
 *                 christoffels :368-440, compute_ricci :443-527), written as
 *                 explicit index loops (the reference emits the same system
 *                 as 970 CSE temporaries, BSSN_GR/src/
 *                 bssneqs_eta_const_standard_gauge.cpp), with eta const
 *                 (B_rhs = Gt_rhs - eta B + ...).
 *   RK4 stage     BSSN_GR/src/rkBSSN.cpp:895-905 and :996-1011, tableau
 *                 BSSN_GR/include/rkBSSN.h:55-58.
 *   constraints   BSSN_GR/src/bssn_constraints.cpp:12-172.
 *
 * Parameter vector prm[] (doubles): lambda[0..3], lambda_f[0..1], eta_const,
 * eta_r0, eta_damping_exp, ko_sigma.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NV 24
enum { A_ = 0, CHI_, K_, GT0_, GT1_, GT2_, BETA0_, BETA1_, BETA2_, B0_, B1_, B2_,
       SGT0_, SGT1_, SGT2_, SGT3_, SGT4_, SGT5_, SAT0_, SAT1_, SAT2_, SAT3_, SAT4_, SAT5_ };

static const int SYM[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};

#define IX(i, j, k) ((i) + nx * ((j) + ny * (k)))

/* ---------------- stencils (QuadGrav/src/derivs.cpp) ---------------- */
/* First derivative, 6th order, along a stride s; the reference evaluates the
 * six taps left to right and scales by (1/h)/60 (derivs.cpp:2144-2170). */
static inline double d1_6(const double *u, long s, double c60)
{
    return (-1.0 * u[-3 * s] + 9.0 * u[-2 * s] - 45.0 * u[-s] + 45.0 * u[s]
            - 9.0 * u[2 * s] + 1.0 * u[3 * s]) * c60;
}
static inline double d2_6(const double *u, long s, double c180)
{
    return (2.0 * u[-3 * s] - 27.0 * u[-2 * s] + 270.0 * u[-s] - 490.0 * u[0]
            + 270.0 * u[s] - 27.0 * u[2 * s] + 2.0 * u[3 * s]) * c180;
}
static inline double ko_4(const double *u, long s, double pre)
{
    return pre * (-u[-3 * s] + 6.0 * u[-2 * s] - 15.0 * u[-s] + 20.0 * u[0]
                  - 15.0 * u[s] + 6.0 * u[2 * s] - u[3 * s]);
}

/* One-sided closures at domain-boundary faces (bflag bit 2*dir: low side,
 * bit 2*dir+1: high side; OCT_DIR_* in include/dendro.h:84-89), taps listed
 * in the reference's evaluation order as (index along dir, coefficient).
 * Low-side indices are absolute (3..8); high-side ones are relative to
 * ie = n - 3.  First/second derivatives: QuadGrav/src/derivs.cpp:2174-2230
 * (deriv64_x) and :2602-2650 (deriv64_xx), scaled by (1/h)/12 and
 * (1/h^2)/12; KO: BSSN_GR/src/derivs.cpp:997-1075, divided by
 * smr = {49,43,59}/48*64*h. */
typedef struct { int n; int idx[6]; double c[6]; } orc_taps;
static const orc_taps D1_LO[3] = {
    {5, {3, 4, 5, 6, 7}, {-25.0, 48.0, -36.0, 16.0, -3.0}},
    {5, {3, 4, 5, 6, 7}, {-3.0, -10.0, 18.0, -6.0, 1.0}},
    {4, {3, 4, 6, 7}, {1.0, -8.0, 8.0, -1.0}}};
static const orc_taps D1_HI[3] = {
    {4, {-5, -4, -2, -1}, {1.0, -8.0, 8.0, -1.0}},
    {5, {-5, -4, -3, -2, -1}, {-1.0, 6.0, -18.0, 10.0, 3.0}},
    {5, {-5, -4, -3, -2, -1}, {3.0, -16.0, 36.0, -48.0, 25.0}}};
static const orc_taps D2_LO[3] = {
    {5, {3, 4, 5, 6, 7}, {35.0, -104.0, 114.0, -56.0, 11.0}},
    {5, {3, 4, 5, 6, 7}, {11.0, -20.0, 6.0, 4.0, -1.0}},
    {5, {3, 4, 5, 6, 7}, {-1.0, 16.0, -30.0, 16.0, -1.0}}};
static const orc_taps D2_HI[3] = {
    {5, {-5, -4, -3, -2, -1}, {-1.0, 16.0, -30.0, 16.0, -1.0}},
    {5, {-5, -4, -3, -2, -1}, {-1.0, 4.0, 6.0, -20.0, 11.0}},
    {5, {-5, -4, -3, -2, -1}, {11.0, -56.0, 114.0, -104.0, 35.0}}};
static const orc_taps KO_LO[3] = {
    {4, {6, 5, 4, 3}, {1.0, -3.0, 3.0, -1.0}},
    {5, {7, 6, 5, 4, 3}, {1.0, -6.0, 12.0, -10.0, 3.0}},
    {6, {8, 7, 6, 5, 4, 3}, {1.0, -6.0, 15.0, -19.0, 12.0, -3.0}}};
static const orc_taps KO_HI[3] = {
    {6, {-6, -5, -4, -3, -2, -1}, {1.0, -6.0, 15.0, -19.0, 12.0, -3.0}},
    {5, {-5, -4, -3, -2, -1}, {1.0, -6.0, 12.0, -10.0, 3.0}},
    {4, {-4, -3, -2, -1}, {1.0, -3.0, 3.0, -1.0}}};

/* line = u at index 0 along dir; s = stride; base = 0 (low) or n-3 (high) */
static double eval_taps(const double *line, long s, int base, const orc_taps *t)
{
    double acc = t->c[0] * line[(base + t->idx[0]) * s];
    for (int q = 1; q < t->n; q++) acc = acc + t->c[q] * line[(base + t->idx[q]) * s];
    return acc;
}

enum { ORC_D1 = 0, ORC_D2 = 1, ORC_KO = 2 };

/* Overwrite the three closure points at each flagged end of dir, over the
 * same (other-axis) ranges as the main loop. */
static void apply_closures(int kind, int dir, double *D, const double *u, double h,
                           const unsigned *sz, unsigned bflag, int jb, int je, int kb, int ke)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const int n = dir == 0 ? nx : dir == 1 ? ny : nz;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    const int lo = (bflag >> (2 * dir)) & 1u, hi = (bflag >> (2 * dir + 1)) & 1u;
    if (!lo && !hi) return;
    const orc_taps *TL = kind == ORC_D1 ? D1_LO : kind == ORC_D2 ? D2_LO : KO_LO;
    const orc_taps *TH = kind == ORC_D1 ? D1_HI : kind == ORC_D2 ? D2_HI : KO_HI;
    const double idx_by_12 = (1.0 / h) / 12.0;
    const double idx_sqrd_by_12 = (1.0 / (h * h)) / 12.0;
    const double smr[3] = {59.0 / 48.0 * 64 * h, 43.0 / 48.0 * 64 * h, 49.0 / 48.0 * 64 * h};
    /* (a, b) run over the two other axes with the caller's ranges */
    for (int b = kb; b < ke; b++)
        for (int a = jb; a < je; a++) {
            int i0, j0, k0; /* index of position 0 along dir */
            if (dir == 0) { i0 = 0; j0 = a; k0 = b; }
            else if (dir == 1) { i0 = a; j0 = 0; k0 = b; }
            else { i0 = a; j0 = b; k0 = 0; }
            const double *line = &u[IX(i0, j0, k0)];
            double *out = &D[IX(i0, j0, k0)];
            for (int q = 0; q < 3; q++) {
                if (lo) {
                    const double acc = eval_taps(line, s, 0, &TL[q]);
                    out[(3 + q) * s] = kind == ORC_D1 ? acc * idx_by_12
                                     : kind == ORC_D2 ? acc * idx_sqrd_by_12 : acc / smr[q];
                }
                if (hi) {
                    const double acc = eval_taps(line, s, n - 3, &TH[q]);
                    out[(n - 6 + q) * s] = kind == ORC_D1 ? acc * idx_by_12
                                         : kind == ORC_D2 ? acc * idx_sqrd_by_12 : acc / smr[2 - q];
                }
            }
        }
}

/* dir 0: i in [3,nx-3), j,k full (derivs.cpp:2151-2156)
 * dir 1: i,j in [3,n-3), k full;  dir 2: interior.  Values outside the
 * computed range are left untouched, as in the reference. */
void orc_deriv64(int dir, double *D, const double *u, double h, const unsigned *sz,
                 unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double c60 = (1.0 / h) / 60.0;
    const int jb = dir == 0 ? 0 : 3, je = dir == 0 ? ny : ny - 3;
    const int kb = dir == 2 ? 3 : 0, ke = dir == 2 ? nz - 3 : nz;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    for (int k = kb; k < ke; k++)
        for (int j = jb; j < je; j++)
            for (int i = 3; i < nx - 3; i++) D[IX(i, j, k)] = d1_6(&u[IX(i, j, k)], s, c60);
    /* closure loops run over the other two axes with the main loop's ranges */
    if (dir == 0) apply_closures(ORC_D1, 0, D, u, h, sz, bflag, 0, ny, 0, nz);
    else if (dir == 1) apply_closures(ORC_D1, 1, D, u, h, sz, bflag, 3, nx - 3, 0, nz);
    else apply_closures(ORC_D1, 2, D, u, h, sz, bflag, 3, nx - 3, 3, ny - 3);
}

void orc_deriv64_2(int dir, double *D, const double *u, double h, const unsigned *sz,
                   unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double c180 = (1.0 / (h * h)) / 180.0;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    for (int k = 3; k < nz - 3; k++)
        for (int j = 3; j < ny - 3; j++)
            for (int i = 3; i < nx - 3; i++) D[IX(i, j, k)] = d2_6(&u[IX(i, j, k)], s, c180);
    if (dir == 0) apply_closures(ORC_D2, 0, D, u, h, sz, bflag, 3, ny - 3, 3, nz - 3);
    else if (dir == 1) apply_closures(ORC_D2, 1, D, u, h, sz, bflag, 3, nx - 3, 3, nz - 3);
    else apply_closures(ORC_D2, 2, D, u, h, sz, bflag, 3, nx - 3, 3, ny - 3);
}

void orc_ko42(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double pre = -1.0 / 64.0 / h;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    for (int k = 3; k < nz - 3; k++)
        for (int j = 3; j < ny - 3; j++)
            for (int i = 3; i < nx - 3; i++) D[IX(i, j, k)] = ko_4(&u[IX(i, j, k)], s, pre);
    if (dir == 0) apply_closures(ORC_KO, 0, D, u, h, sz, bflag, 3, ny - 3, 3, nz - 3);
    else if (dir == 1) apply_closures(ORC_KO, 1, D, u, h, sz, bflag, 3, nx - 3, 3, nz - 3);
    else apply_closures(ORC_KO, 2, D, u, h, sz, bflag, 3, nx - 3, 3, ny - 3);
}

/* Outgoing-radiation condition on the flagged faces' boundary layer
 * (BSSN_GR/src/rhs.cpp:838-982):
 * rhs = -(1/r) (x f_x + y f_y + z f_z + falloff (f - asymptotic)). */
void orc_bssn_bcs(double *f_rhs, const double *f, const double *dxf, const double *dyf,
                  const double *dzf, const double *pmin, const double *pmax,
                  double falloff, double asym, const unsigned *sz, unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double hx = (pmax[0] - pmin[0]) / (nx - 1), hy = (pmax[1] - pmin[1]) / (ny - 1),
                 hz = (pmax[2] - pmin[2]) / (nz - 1);
    const int ib = 3, jb = 3, kb = 3, ie = nx - 3, je = ny - 3, ke = nz - 3;
    for (int face = 0; face < 6; face++) {
        if (!(bflag & (1u << face))) continue;
        const int dir = face / 2, hi = face & 1;
        const int fixed = dir == 0 ? (hi ? ie - 1 : ib) : dir == 1 ? (hi ? je - 1 : jb) : (hi ? ke - 1 : kb);
        const int na = dir == 0 ? jb : ib, ea = dir == 0 ? je : ie;   /* first free axis */
        const int nb = dir == 2 ? jb : kb, eb = dir == 2 ? je : ke;   /* second free axis */
        for (int b = nb; b < eb; b++)
            for (int a = na; a < ea; a++) {
                const int i = dir == 0 ? fixed : a;
                const int j = dir == 1 ? fixed : (dir == 0 ? a : b);
                const int k = dir == 2 ? fixed : b;
                const double x = pmin[0] + i * hx, y = pmin[1] + j * hy, z = pmin[2] + k * hz;
                const size_t pp = IX(i, j, k);
                const double inv_r = 1.0 / sqrt(x * x + y * y + z * z);
                f_rhs[pp] = -inv_r * (x * dxf[pp] + y * dyf[pp] + z * dzf[pp]
                                      + falloff * (f[pp] - asym));
            }
    }
}

/* ---------------- point algebra (CodeGen/bssn.py, dendro.py) ---------------- */
typedef struct {
    double a, chi, K, Gt[3], b[3], B[3], gt[3][3], At[3][3];
    double da[3], dchi[3], dK[3], dGt[3][3], db[3][3], dB[3][3];  /* [component][dir] */
    double dgt[3][3][3], dAt[3][3][3];                           /* [i][j][dir] */
    double ddgt[3][3][3][3], ddchi[3][3], dda[3][3], ddb[3][3][3]; /* [..][l][m] */
    /* upwind != 0: the advection terms beta^j d_j f of every field f are
     * adv[f] (VAR order), from the upwinded derivatives of the 4th-order
     * binding; otherwise they use the centred first derivatives above */
    int upwind;
    double adv[24];
} orc_point;

/* out[] in variable order (grDef.h:31). */
void orc_bssn_point(const orc_point *P, const double *prm, double eta, double *out)
{
    const double l1 = prm[0], l2 = prm[1], l3 = prm[2], l4 = prm[3];
    const double lf0 = prm[4], lf1 = prm[5];
    const double a = P->a, chi = P->chi, K = P->K;
    double g[3][3], ig[3][3];
    memcpy(g, P->gt, sizeof g);

    /* inverse conformal metric: adjugate over determinant (dendro.py:351) */
    const double det = g[0][0] * (g[1][1] * g[2][2] - g[1][2] * g[1][2])
                     - g[0][1] * g[0][1] * g[2][2] + 2.0 * g[0][1] * g[0][2] * g[1][2]
                     - g[0][2] * g[0][2] * g[1][1];
    ig[0][0] = (g[1][1] * g[2][2] - g[1][2] * g[1][2]) / det;
    ig[0][1] = (g[0][2] * g[1][2] - g[0][1] * g[2][2]) / det;
    ig[0][2] = (g[0][1] * g[1][2] - g[0][2] * g[1][1]) / det;
    ig[1][1] = (g[0][0] * g[2][2] - g[0][2] * g[0][2]) / det;
    ig[1][2] = (g[0][1] * g[0][2] - g[0][0] * g[1][2]) / det;
    ig[2][2] = (g[0][0] * g[1][1] - g[0][1] * g[0][1]) / det;
    ig[1][0] = ig[0][1]; ig[2][0] = ig[0][2]; ig[2][1] = ig[1][2];

    /* Christoffels (dendro.py:368-440) */
    double C1[3][3][3], C2[3][3][3], C3[3][3][3], igdchi[3], CalGt[3];
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                C1[k][i][j] = 0.5 * (P->dgt[k][i][j] + P->dgt[k][j][i] - P->dgt[i][j][k]);
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double s = 0.0;
                for (int l = 0; l < 3; l++) s += ig[k][l] * C1[l][i][j];
                C2[k][i][j] = s;
            }
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int m = 0; m < 3; m++) s += ig[i][m] * P->dchi[m];
        igdchi[i] = s;
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                C3[i][j][k] = C2[i][j][k] - 0.5 / chi * ((i == j ? P->dchi[k] : 0.0)
                              + (i == k ? P->dchi[j] : 0.0) - g[j][k] * igdchi[i]);
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) s += ig[k][l] * C2[i][k][l];
        CalGt[i] = s;
    }

    /* Ricci tensor (dendro.py:443-527) */
    double R[3][3];
    double trchi = 0.0, CalGtdchi = 0.0;
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++)
            trchi += ig[k][l] * (P->ddchi[k][l] - 3.0 / (2.0 * chi) * P->dchi[k] * P->dchi[l]);
    for (int m = 0; m < 3; m++) CalGtdchi += CalGt[m] * P->dchi[m];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double t1 = 0.0, t2 = 0.0, t3 = 0.0, t4 = 0.0;
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++) t1 += ig[l][m] * P->ddgt[i][j][l][m];
            for (int k = 0; k < 3; k++)
                t2 += g[k][i] * P->dGt[k][j] + g[k][j] * P->dGt[k][i];
            for (int k = 0; k < 3; k++) t3 += CalGt[k] * (C1[i][j][k] + C1[j][i][k]);
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++)
                    for (int m = 0; m < 3; m++)
                        t4 += ig[l][m] * (C2[k][l][i] * C1[j][k][m] + C2[k][l][j] * C1[i][k][m]
                                          + C2[k][i][m] * C1[k][l][j]);
            const double Rt = -0.5 * t1 + 0.5 * t2 + 0.5 * t3 + t4;
            double c2d = 0.0;
            for (int k = 0; k < 3; k++) c2d += C2[k][j][i] * P->dchi[k];
            const double xR = 1.0 / (2.0 * chi) * (P->ddchi[i][j] - c2d)
                            - 1.0 / (4.0 * chi * chi) * P->dchi[i] * P->dchi[j];
            const double Rphi = xR + 1.0 / (2.0 * chi) * g[i][j] * (trchi - CalGtdchi);
            R[i][j] = Rt + Rphi;
        }

    /* second covariant derivative of the lapse (dendro.py:160) */
    double DDa[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int l = 0; l < 3; l++) s += C3[l][i][j] * P->da[l];
            DDa[i][j] = P->dda[i][j] - s;
        }

    double divb = 0.0;
    for (int k = 0; k < 3; k++) divb += P->db[k][k];

    /* lapse, shift (bssn.py:65-72) */
    double adva = 0.0;
    if (P->upwind) adva = P->adv[A_];
    else for (int i = 0; i < 3; i++) adva += P->b[i] * P->da[i];
    const double a_rhs = l1 * adva - 2.0 * a * K;
    double b_rhs[3];
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        if (P->upwind) s = P->adv[BETA0_ + i];
        else for (int j = 0; j < 3; j++) s += P->b[j] * P->db[i][j];
        b_rhs[i] = 3.0 / 4.0 * (lf0 + lf1 * a) * P->B[i] + l2 * s;
    }

    /* Lie derivatives of weight -2/3 (dendro.py:211) */
    const double w = -2.0 / 3.0;
    double gt_rhs[3][3], At_rhs[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double sg = 0.0, sa = 0.0;
            if (P->upwind) {
                sg = P->adv[SGT0_ + SYM[i][j]];
                sa = P->adv[SAT0_ + SYM[i][j]];
                for (int k = 0; k < 3; k++) {
                    sg += g[i][k] * P->db[k][j] + g[k][j] * P->db[k][i] + w * g[i][j] * P->db[k][k];
                    sa += P->At[i][k] * P->db[k][j] + P->At[k][j] * P->db[k][i]
                        + w * P->At[i][j] * P->db[k][k];
                }
            } else {
                for (int k = 0; k < 3; k++) {
                    sg += P->b[k] * P->dgt[i][j][k] + g[i][k] * P->db[k][j] + g[k][j] * P->db[k][i]
                        + w * g[i][j] * P->db[k][k];
                    sa += P->b[k] * P->dAt[i][j][k] + P->At[i][k] * P->db[k][j]
                        + P->At[k][j] * P->db[k][i] + w * P->At[i][j] * P->db[k][k];
                }
            }
            gt_rhs[i][j] = sg - 2.0 * a * P->At[i][j];
            At_rhs[i][j] = sa;
        }
    double advchi = 0.0;
    if (P->upwind) advchi = P->adv[CHI_];
    else for (int i = 0; i < 3; i++) advchi += P->b[i] * P->dchi[i];
    const double chi_rhs = advchi + w * chi * divb + 2.0 / 3.0 * (chi * a * K);

    /* At: chi * TF(a R - DiDj a) + a (K At - 2 At_ik At^k_j)  (bssn.py:78-80) */
    double X[3][3], trX = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) X[i][j] = a * R[i][j] - DDa[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) trX += ig[i][j] * X[i][j];
    double AUd[3][3]; /* At^k_j = ig^kl At_lj */
    for (int k = 0; k < 3; k++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int l = 0; l < 3; l++) s += ig[k][l] * P->At[l][j];
            AUd[k][j] = s;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double AA = 0.0;
            for (int k = 0; k < 3; k++) AA += P->At[i][k] * AUd[k][j];
            At_rhs[i][j] += chi * (X[i][j] - g[i][j] * trX / 3.0)
                          + a * (K * P->At[i][j] - 2.0 * AA);
        }

    /* K (bssn.py:82) */
    double AUU[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) s += ig[i][k] * ig[j][l] * P->At[k][l];
            AUU[i][j] = s;
        }
    double lap = 0.0, sqrA = 0.0, advK = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            lap += chi * ig[i][j] * DDa[i][j];
            sqrA += P->At[i][j] * AUU[i][j];
        }
    if (P->upwind) advK = P->adv[K_];
    else for (int i = 0; i < 3; i++) advK += P->b[i] * P->dK[i];
    const double K_rhs = advK - lap + a * (K * K / 3.0 + sqrA);

    /* Gt, B (bssn.py:86-104) */
    double Gt_rhs[3], B_rhs[3];
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        if (P->upwind) s = P->adv[GT0_ + i];
        else for (int j = 0; j < 3; j++) s += P->b[j] * P->dGt[i][j];
        for (int j = 0; j < 3; j++) s -= CalGt[j] * P->db[i][j];
        s += 2.0 / 3.0 * CalGt[i] * divb;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                s += ig[j][k] * P->ddb[i][j][k] + ig[i][j] * P->ddb[k][j][k] / 3.0;
        for (int j = 0; j < 3; j++) s -= 2.0 * AUU[i][j] * P->da[j];
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) s += 2.0 * a * C2[i][j][k] * AUU[j][k];
        for (int j = 0; j < 3; j++)
            s -= a * (3.0 / chi * AUU[i][j] * P->dchi[j] + 4.0 / 3.0 * ig[i][j] * P->dK[j]);
        Gt_rhs[i] = s;
    }
    for (int i = 0; i < 3; i++) {
        double sB = 0.0, sG = 0.0;
        if (P->upwind) {
            sB = P->adv[B0_ + i];
            sG = P->adv[GT0_ + i];
        } else {
            for (int j = 0; j < 3; j++) {
                sB += P->b[j] * P->dB[i][j];
                sG += P->b[j] * P->dGt[i][j];
            }
        }
        B_rhs[i] = Gt_rhs[i] - eta * P->B[i] + l3 * sB - l4 * sG;
    }

    out[A_] = a_rhs; out[CHI_] = chi_rhs; out[K_] = K_rhs;
    for (int i = 0; i < 3; i++) {
        out[GT0_ + i] = Gt_rhs[i];
        out[BETA0_ + i] = b_rhs[i];
        out[B0_ + i] = B_rhs[i];
    }
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            out[SGT0_ + SYM[i][j]] = gt_rhs[i][j];
            out[SAT0_ + SYM[i][j]] = At_rhs[i][j];
        }
}

/* ---------------- per-block driver (BSSN_GR/src/rhs.cpp:86-392) ---------------- */
/* 11 fields carry second derivatives (BSSN_GR/scripts/bssnrhs_derivs.h). */
static const int HAS_D2[NV] = {1, 1, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0,
                               1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0};

/* Returns 0 on success, -1 for a domain-boundary block, -2 on allocation
 * failure.  Writes only interior points of each rhs[v] + offset. */
/* bssn_bcs falloff / asymptotic value per variable, VAR order
 * (BSSN_GR/src/rhs.cpp:269-321). */
static const double BC_FALLOFF[NV] = {1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1,
                                      1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2};
static const double BC_ASYM[NV] = {1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                   1, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0, 0};

void orc_deriv42(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag);
void orc_deriv42_2(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag);
void orc_bssn_adv42(int dir, double *D, const double *u, double h, const unsigned *sz,
                    const double *beta, unsigned bflag);

/* apply_bcs = 0 skips bssn_bcs.  order 6: the QuadGrav binding
 * (QuadGrav/include/derivs.h:80-97: deriv64 first and second derivatives,
 * the centred deriv64adv as advective derivative, ko_deriv42); order 4: the
 * BSSN_GR solver's own binding (BSSN_GR/include/rhs.h:23-37: deriv42,
 * upwinded deriv42adv, ko_deriv42). */
int orc_bssnrhs_ex2(double **rhs, const double **uz, unsigned long offset,
                    const double *pmin, const double *pmax, const unsigned *sz,
                    unsigned bflag, const double *prm, int apply_bcs, int order)
{
    if (bflag != 0 && (sz[0] < 13 || sz[1] < 13 || sz[2] < 13)) return -1;
    if (order != 4 && order != 6) return -3;
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const size_t n = (size_t)nx * ny * nz;
    const double h[3] = {(pmax[0] - pmin[0]) / (nx - 1), (pmax[1] - pmin[1]) / (ny - 1),
                         (pmax[2] - pmin[2]) / (nz - 1)};
    /* grad[v][d] and, for HAS_D2 fields, grad2[v][0..5] = xx,xy,xz,yy,yz,zz;
     * at order 4 also the upwinded agrad[v][d] */
    double *grad[NV][3], *grad2[NV][6], *agrad[NV][3];
    const size_t narr = NV * 3 + 11 * 6 + (order == 4 ? NV * 3 : 0);
    double *pool = (double *)malloc(sizeof(double) * n * narr);
    if (!pool) return -2;
    double *p = pool;
    for (int v = 0; v < NV; v++) {
        for (int d = 0; d < 3; d++) { grad[v][d] = p; p += n; }
        for (int q = 0; q < 6; q++) grad2[v][q] = NULL;
        if (HAS_D2[v]) for (int q = 0; q < 6; q++) { grad2[v][q] = p; p += n; }
        for (int d = 0; d < 3; d++) {
            agrad[v][d] = order == 4 ? p : NULL;
            if (order == 4) p += n;
        }
    }
    for (int v = 0; v < NV; v++) {
        const double *u = uz[v] + offset;
        if (order == 6) {
            for (int d = 0; d < 3; d++) orc_deriv64(d, grad[v][d], u, h[d], sz, bflag);
            if (HAS_D2[v]) {
                orc_deriv64_2(0, grad2[v][0], u, h[0], sz, bflag);
                orc_deriv64_2(1, grad2[v][3], u, h[1], sz, bflag);
                orc_deriv64_2(2, grad2[v][5], u, h[2], sz, bflag);
                orc_deriv64(1, grad2[v][1], grad[v][0], h[1], sz, bflag); /* d_y(d_x u) */
                orc_deriv64(2, grad2[v][2], grad[v][0], h[2], sz, bflag); /* d_z(d_x u) */
                orc_deriv64(2, grad2[v][4], grad[v][1], h[2], sz, bflag); /* d_z(d_y u) */
            }
        } else {
            for (int d = 0; d < 3; d++) {
                orc_deriv42(d, grad[v][d], u, h[d], sz, bflag);
                orc_bssn_adv42(d, agrad[v][d], u, h[d], sz, uz[BETA0_ + d] + offset, bflag);
            }
            if (HAS_D2[v]) {
                orc_deriv42_2(0, grad2[v][0], u, h[0], sz, bflag);
                orc_deriv42_2(1, grad2[v][3], u, h[1], sz, bflag);
                orc_deriv42_2(2, grad2[v][5], u, h[2], sz, bflag);
                orc_deriv42(1, grad2[v][1], grad[v][0], h[1], sz, bflag);
                orc_deriv42(2, grad2[v][2], grad[v][0], h[2], sz, bflag);
                orc_deriv42(2, grad2[v][4], grad[v][1], h[2], sz, bflag);
            }
        }
    }
    static const int Q[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    const double eta_const = prm[6], eta_r0 = prm[7], eta_exp = prm[8];
    for (int k = 3; k < nz - 3; k++) {
        const double z = pmin[2] + k * h[2];
        for (int j = 3; j < ny - 3; j++) {
            const double y = pmin[1] + j * h[1];
            for (int i = 3; i < nx - 3; i++) {
                const double x = pmin[0] + i * h[0];
                const size_t pp = IX(i, j, k);
                const double r = sqrt(x * x + y * y + z * z);
                double eta = eta_const;
                if (r >= eta_r0) eta *= pow(eta_r0 / r, eta_exp);
                orc_point P;
#define F(v) (uz[v][offset + pp])
                P.a = F(A_); P.chi = F(CHI_); P.K = F(K_);
                for (int c = 0; c < 3; c++) {
                    P.Gt[c] = F(GT0_ + c); P.b[c] = F(BETA0_ + c); P.B[c] = F(B0_ + c);
                }
                for (int a2 = 0; a2 < 3; a2++)
                    for (int b2 = 0; b2 < 3; b2++) {
                        P.gt[a2][b2] = F(SGT0_ + SYM[a2][b2]);
                        P.At[a2][b2] = F(SAT0_ + SYM[a2][b2]);
                    }
#undef F
                for (int d = 0; d < 3; d++) {
                    P.da[d] = grad[A_][d][pp]; P.dchi[d] = grad[CHI_][d][pp];
                    P.dK[d] = grad[K_][d][pp];
                    for (int c = 0; c < 3; c++) {
                        P.dGt[c][d] = grad[GT0_ + c][d][pp];
                        P.db[c][d] = grad[BETA0_ + c][d][pp];
                        P.dB[c][d] = grad[B0_ + c][d][pp];
                    }
                    for (int a2 = 0; a2 < 3; a2++)
                        for (int b2 = 0; b2 < 3; b2++) {
                            P.dgt[a2][b2][d] = grad[SGT0_ + SYM[a2][b2]][d][pp];
                            P.dAt[a2][b2][d] = grad[SAT0_ + SYM[a2][b2]][d][pp];
                        }
                }
                for (int l = 0; l < 3; l++)
                    for (int m = 0; m < 3; m++) {
                        const int q = Q[l][m];
                        P.ddchi[l][m] = grad2[CHI_][q][pp];
                        P.dda[l][m] = grad2[A_][q][pp];
                        for (int c = 0; c < 3; c++) P.ddb[c][l][m] = grad2[BETA0_ + c][q][pp];
                        for (int a2 = 0; a2 < 3; a2++)
                            for (int b2 = 0; b2 < 3; b2++)
                                P.ddgt[a2][b2][l][m] = grad2[SGT0_ + SYM[a2][b2]][q][pp];
                    }
                P.upwind = order == 4;
                if (P.upwind)
                    for (int v = 0; v < NV; v++) {
                        double t = 0.0;
                        for (int d = 0; d < 3; d++) t += P.b[d] * agrad[v][d][pp];
                        P.adv[v] = t;
                    }
                double out[NV];
                orc_bssn_point(&P, prm, eta, out);
                for (int v = 0; v < NV; v++) rhs[v][offset + pp] = out[v];
            }
        }
    }
    if (bflag != 0 && apply_bcs)
        for (int v = 0; v < NV; v++)
            orc_bssn_bcs(rhs[v] + offset, uz[v] + offset, grad[v][0], grad[v][1], grad[v][2],
                         pmin, pmax, BC_FALLOFF[v], BC_ASYM[v], sz, bflag);
    /* KO dissipation reuses the first-derivative scratch (bssnrhs_ko_derivs.h) */
    const double sigma = prm[9];
    for (int v = 0; v < NV; v++) {
        const double *u = uz[v] + offset;
        for (int d = 0; d < 3; d++) orc_ko42(d, grad[v][d], u, h[d], sz, bflag);
        double *o = rhs[v] + offset;
        for (int k = 3; k < nz - 3; k++)
            for (int j = 3; j < ny - 3; j++)
                for (int i = 3; i < nx - 3; i++) {
                    const size_t pp = IX(i, j, k);
                    o[pp] += sigma * (grad[v][0][pp] + grad[v][1][pp] + grad[v][2][pp]);
                }
    }
    free(pool);
    return 0;
}

int orc_bssnrhs_ex(double **rhs, const double **uz, unsigned long offset,
                   const double *pmin, const double *pmax, const unsigned *sz,
                   unsigned bflag, const double *prm, int apply_bcs)
{
    return orc_bssnrhs_ex2(rhs, uz, offset, pmin, pmax, sz, bflag, prm, apply_bcs, 6);
}

int orc_bssnrhs(double **rhs, const double **uz, unsigned long offset, const double *pmin,
                const double *pmax, const unsigned *sz, unsigned bflag, const double *prm)
{
    return orc_bssnrhs_ex2(rhs, uz, offset, pmin, pmax, sz, bflag, prm, 1, 6);
}

/* bssnRHS over a block list (BSSN_GR/src/rhs.cpp:9-76), OpenMP over blocks
 * as the reference test bed does (BSSN_GR/src/rhsTestBed.cpp:181-215).
 * blk[] rows: offset, sz0, sz1, sz2, bflag (as doubles are avoided: ulong). */
int orc_bssnrhs_blocks_ex(double **rhs, const double **uz, long nblk,
                          const unsigned long *offsets, const unsigned *sizes /*3 per block*/,
                          const unsigned *bflags, const double *pmins, const double *pmaxs,
                          const double *prm, int nthreads, int order)
{
    int err = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic) reduction(|:err)
#endif
    for (long b = 0; b < nblk; b++)
        err |= -orc_bssnrhs_ex2(rhs, uz, offsets[b], pmins + 3 * b, pmaxs + 3 * b,
                                sizes + 3 * b, bflags[b], prm, 1, order);
    (void)nthreads;
    return -err;
}

int orc_bssnrhs_blocks(double **rhs, const double **uz, long nblk,
                       const unsigned long *offsets, const unsigned *sizes /*3 per block*/,
                       const unsigned *bflags, const double *pmins, const double *pmaxs,
                       const double *prm, int nthreads)
{
    return orc_bssnrhs_blocks_ex(rhs, uz, nblk, offsets, sizes, bflags, pmins, pmaxs, prm,
                                 nthreads, 6);
}

/* ---------------- RK4 stage update + constraints ---------------- */
/* BSSN_GR/src/bssn_constraints.cpp:12-172 on one node of SoA vectors. */
void orc_enforce_bssn_constraints(double **v, size_t node, double chi_floor)
{
    const double one_third = 1.0 / 3.0;
    double g[3][3], A[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            g[i][j] = v[SGT0_ + SYM[i][j]][node];
            A[i][j] = v[SAT0_ + SYM[i][j]][node];
        }
    double det = g[0][0] * (g[1][1] * g[2][2] - g[1][2] * g[1][2]) - g[0][1] * g[0][1] * g[2][2]
               + 2.0 * g[0][1] * g[0][2] * g[1][2] - g[0][2] * g[0][2] * g[1][1];
    const double s = 1.0 / pow(det, one_third);
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) g[i][j] *= s;
    det = g[0][0] * (g[1][1] * g[2][2] - g[1][2] * g[1][2]) - g[0][1] * g[0][1] * g[2][2]
        + 2.0 * g[0][1] * g[0][2] * g[1][2] - g[0][2] * g[0][2] * g[1][1];
    const double idet = 1.0 / det;
    double gu[3][3];
    gu[0][0] = idet * (g[1][1] * g[2][2] - g[1][2] * g[1][2]);
    gu[0][1] = idet * (-g[0][1] * g[2][2] + g[0][2] * g[1][2]);
    gu[0][2] = idet * (g[0][1] * g[1][2] - g[0][2] * g[1][1]);
    gu[1][1] = idet * (g[0][0] * g[2][2] - g[0][2] * g[0][2]);
    gu[1][2] = idet * (-g[0][0] * g[1][2] + g[0][1] * g[0][2]);
    gu[2][2] = idet * (g[0][0] * g[1][1] - g[0][1] * g[0][1]);
    const double tr3 = one_third * (A[0][0] * gu[0][0] + A[1][1] * gu[1][1] + A[2][2] * gu[2][2]
                                    + 2.0 * (A[0][1] * gu[0][1] + A[0][2] * gu[0][2] + A[1][2] * gu[1][2]));
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            v[SAT0_ + SYM[i][j]][node] = A[i][j] - tr3 * g[i][j];
            v[SGT0_ + SYM[i][j]][node] = g[i][j];
        }
    if (v[CHI_][node] < chi_floor) v[CHI_][node] = chi_floor;
    v[A_][node] = (v[A_][node] < chi_floor) ? chi_floor : v[A_][node]; /* std::max */
}

/* Stage s in 0..2: im = prev + U[s+1] dt k_s, then enforce (rkBSSN.cpp:895-905).
 * Final (s == 3): var = prev + sum_s C[s] dt k_s in stage order, then enforce
 * (rkBSSN.cpp:996-1011).  k[s][v] are the zipped stage vectors. */
void orc_rk4_stage(int s, double **dst, const double **prev, const double ***k,
                   size_t nnodes, double dt, double chi_floor)
{
    static const double RK4_C[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    static const double RK4_U[4] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0};
    for (size_t node = 0; node < nnodes; node++) {
        for (int v = 0; v < NV; v++) {
            double x = prev[v][node];
            if (s < 3) {
                x += RK4_U[s + 1] * dt * k[s][v][node];
            } else {
                for (int q = 0; q < 4; q++) x += RK4_C[q] * dt * k[q][v][node];
            }
            dst[v][node] = x;
        }
        orc_enforce_bssn_constraints(dst, node, chi_floor);
    }
}

/* ---------------- Mesh::unzip / Mesh::zip from the operator ---------------- */
/* The restatement of include/mesh.tcc:7436-8690 used by the checker and the
 * CPU baseline: source elements' nodal values level by level (hanging nodes
 * interpolated from coarser sources, getElementNodalValues mesh.tcc:2467),
 * then copies and separable degree-6 interpolations of the padded points
 * (parent2ChildInterpolation, FEM/include/refel.h:249-296).  Reference word:
 * bit 63 clear = zipped node (low 32 bits); set = source (bits 12..42) at
 * codes 2*xi (bits 0..11). */
static double orc_lag[6][7];
static void orc_lag_init(void)
{
    for (int r = 0; r < 6; r++)
        for (int i = 0; i < 7; i++) {
            double num = 1.0, den = 1.0;
            for (int m = 0; m < 7; m++)
                if (m != i) { num *= (r + 0.5) - m; den *= (double)(i - m); }
            orc_lag[r][i] = num / den;
        }
}

static double orc_ref_value(unsigned long long ref, const double *z, const double *dg)
{
    if (!(ref >> 63)) return z[(unsigned)(ref & 0xFFFFFFFFull)];
    const unsigned long long src = (ref >> 12) & 0x7FFFFFFFull;
    double w[3][7];
    int idx[3][7], n[3];
    for (int a = 0; a < 3; a++) {
        const int code = (int)((ref >> (4 * a)) & 0xF);
        if ((code & 1) == 0) { n[a] = 1; w[a][0] = 1.0; idx[a][0] = code >> 1; }
        else { n[a] = 7; for (int i = 0; i < 7; i++) { w[a][i] = orc_lag[code >> 1][i]; idx[a][i] = i; } }
    }
    const double *e = dg + src * 343;
    double acc = 0.0;
    for (int c = 0; c < n[2]; c++) {
        double accy = 0.0;
        for (int b = 0; b < n[1]; b++) {
            double accx = 0.0;
            for (int q = 0; q < n[0]; q++) accx += w[0][q] * e[idx[0][q] + 7 * (idx[1][b] + 7 * idx[2][c])];
            accy += w[1][b] * accx;
        }
        acc += w[2][c] * accy;
    }
    return acc;
}

/* zipped -> unzipped for one field; dg is scratch of nsrc*343 doubles.
 * Padded points that are neither copies nor interpolation rows are left
 * untouched. */
void orc_unzip(const double *z, double *u, unsigned long long nunz, const unsigned *copy_src,
               unsigned long long ninterp, const unsigned long long *interp_dst,
               const unsigned long long *interp_ref, unsigned long long nlevels,
               const unsigned long long *level_ptr, const unsigned long long *src_refs,
               double *dg, int nthreads)
{
    static int init = 0;
    if (!init) { orc_lag_init(); init = 1; }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    (void)nthreads;
    for (unsigned long long l = 0; l < nlevels; l++) {
        const long long a = (long long)(level_ptr[l] * 343), b = (long long)(level_ptr[l + 1] * 343);
#pragma omp parallel for schedule(static)
        for (long long t = a; t < b; t++) dg[t] = orc_ref_value(src_refs[t], z, dg);
    }
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < (long long)nunz; p++)
        if (copy_src[p] != 0xFFFFFFFFu) u[p] = z[copy_src[p]];
#pragma omp parallel for schedule(static)
    for (long long r = 0; r < (long long)ninterp; r++)
        u[interp_dst[r]] = orc_ref_value(interp_ref[r], z, dg);
}

void orc_zip(const double *u, double *z, unsigned long long ndof, const unsigned long long *zip_src)
{
#pragma omp parallel for schedule(static)
    for (long long d = 0; d < (long long)ndof; d++) z[d] = u[zip_src[d]];
}
