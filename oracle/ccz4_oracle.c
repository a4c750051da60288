/*
 * ORACLE — test infrastructure only.  C restatement of the reference's CCZ4
 * right-hand side ccz4rhs (CCZ4_GR/src/rhs.cpp:12-298), the function its
 * RK4 solver calls (CCZ4_GR/src/rk4CCZ4.cpp:498):
 *   stencils   the 4th-order family CCZ4_GR/include/rhs.h:14-28 binds, from
 *              the CCZ4 solver's own CCZ4_GR/src/derivs.cpp: deriv42_*
 *              (same as orc_deriv42*), the upwind deriv42adv_* (:495-915)
 *              and ko_deriv42_* (:917-1347), with their closures;
 *   algebra    CodeGen for CCZ4, GR/rhs_scripts/ccz4/ccz4.py:52-117 with
 *              the tensor helpers of GR/rhs_scripts/ccz4/dendro_ccz4.py
 *              (lie :263, DiDj :182, laplacian :309, trace_free :373,
 *              Christoffels :447-536, compute_ricci :539-589), as index loops;
 *   BCs        ccz4_bcs (CCZ4_GR/src/rhs.cpp, the same operator as bssn_bcs)
 *              with the per-variable falloff / asymptotic values of
 *              rhs.cpp:168-231, theta_z4 excluded;
 *   KO         rhs += sigma (kx + ky + kz) for every variable but theta_z4
 *              (rhs.cpp:241-283).
 * Variable order (CCZ4_GR/include/grUtils.h:46): alpha, psi, K, Gh0-2,
 * beta0-2, B0-2, gt0-5, At0-5, theta_z4.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define IX(i, j, k) ((i) + nx * ((j) + ny * (k)))
#define NV4 25
enum { C_A = 0, C_PSI, C_K, C_GH0, C_GH1, C_GH2, C_B0_, C_B1_, C_B2_, C_BB0, C_BB1, C_BB2,
       C_G0, C_G1, C_G2, C_G3, C_G4, C_G5, C_A0, C_A1, C_A2, C_A3, C_A4, C_A5, C_TH };
static const int SYM4[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};

void orc_deriv42(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag);
void orc_deriv42_2(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag);
void orc_bssn_bcs(double *f_rhs, const double *f, const double *dxf, const double *dyf,
                  const double *dzf, const double *pmin, const double *pmax,
                  double falloff, double asym, const unsigned *sz, unsigned bflag);

/* Upwind advective derivative along dir (CCZ4_GR/src/derivs.cpp:495-915;
 * BSSN_GR/src/derivs.cpp:494-913 and its copy in QuadGrav/src/derivs.cpp):
 * interior points of the block, biased by the sign of beta_dir.  The two
 * solvers' files differ in one test only, at the point ie-3 of a flagged high
 * face: the CCZ4 file takes the one-sided forward form where beta < 0
 * (ccz4_hi != 0), the BSSN file where beta > 0. */
static void adv42(int dir, double *D, const double *u, double h, const unsigned *sz,
                  const double *beta, unsigned bflag, int ccz4_hi)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double idx = 1.0 / h, half = 0.50 * idx, c12 = idx / 12.0;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    const int n = dir == 0 ? nx : dir == 1 ? ny : nz;
    for (int k = 3; k < nz - 3; k++)
        for (int j = 3; j < ny - 3; j++)
            for (int i = 3; i < nx - 3; i++) {
                const size_t pp = IX(i, j, k);
                const double *c = &u[pp];
                if (beta[pp] > 0.0)
                    D[pp] = (-3.0 * c[-s] - 10.0 * c[0] + 18.0 * c[s] - 6.0 * c[2 * s] + c[3 * s]) * c12;
                else
                    D[pp] = (-c[-3 * s] + 6.0 * c[-2 * s] - 18.0 * c[-s] + 10.0 * c[0] + 3.0 * c[s]) * c12;
            }
    const int lo = (bflag >> (2 * dir)) & 1u, hi = (bflag >> (2 * dir + 1)) & 1u;
    if (!lo && !hi) return;
    const int ar1 = dir == 0 ? ny - 3 : nx - 3, br1 = dir == 2 ? ny - 3 : nz - 3;
    const int ie = n - 3;
    for (int b = 3; b < br1; b++)
        for (int a = 3; a < ar1; a++) {
            int i0, j0, k0;
            if (dir == 0) { i0 = 0; j0 = a; k0 = b; }
            else if (dir == 1) { i0 = a; j0 = 0; k0 = b; }
            else { i0 = a; j0 = b; k0 = 0; }
            const size_t base = IX(i0, j0, k0);
            const double *L = &u[base];
            const double *B = &beta[base];
            double *O = &D[base];
#define U(q) L[(q) * s]
            if (lo) {
                O[3 * s] = (-3.0 * U(3) + 4.0 * U(4) - U(5)) * half;
                O[4 * s] = B[4 * s] > 0.0 ? (-3.0 * U(4) + 4.0 * U(5) - U(6)) * half
                                          : (-U(3) + U(5)) * half;
                O[5 * s] = B[5 * s] > 0.0
                    ? (-3.0 * U(4) - 10.0 * U(5) + 18.0 * U(6) - 6.0 * U(7) + U(8)) * c12
                    : (U(3) - 4.0 * U(4) + 3.0 * U(5)) * half;
            }
            if (hi) {
                O[(ie - 3) * s] = (ccz4_hi ? B[(ie - 3) * s] < 0.0 : B[(ie - 3) * s] > 0.0)
                    ? (-3.0 * U(ie - 3) + 4.0 * U(ie - 2) - U(ie - 1)) * half
                    : (-U(ie - 6) + 6.0 * U(ie - 5) - 18.0 * U(ie - 4) + 10.0 * U(ie - 3)
                       + 3.0 * U(ie - 2)) * c12;
                O[(ie - 2) * s] = B[(ie - 2) * s] > 0.0 ? (-U(ie - 3) + U(ie - 1)) * half
                                                        : (U(ie - 4) - 4.0 * U(ie - 3) + 3.0 * U(ie - 2)) * half;
                O[(ie - 1) * s] = (U(ie - 3) - 4.0 * U(ie - 2) + 3.0 * U(ie - 1)) * half;
            }
#undef U
        }
}

void orc_ccz4_adv42(int dir, double *D, const double *u, double h, const unsigned *sz,
                    const double *beta, unsigned bflag)
{
    adv42(dir, D, u, h, sz, beta, bflag, 1);
}

void orc_bssn_adv42(int dir, double *D, const double *u, double h, const unsigned *sz,
                    const double *beta, unsigned bflag)
{
    adv42(dir, D, u, h, sz, beta, bflag, 0);
}

/* Kreiss-Oliger dissipation of the CCZ4 solver (CCZ4_GR/src/derivs.cpp:917-1347):
 * at the first and last interior point of each line the centred stencil
 * of the neighbouring point is used; one-sided closures on flagged faces. */
void orc_ccz4_ko42(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double pre = -1.0 / 64.0 / h;
    const double smr3 = 59.0 / 48.0 * 64 * h, smr2 = 43.0 / 48.0 * 64 * h, smr1 = 49.0 / 48.0 * 64 * h;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    const int n = dir == 0 ? nx : dir == 1 ? ny : nz;
    const int ie = n - 3;
    const int lo = (bflag >> (2 * dir)) & 1u, hi = (bflag >> (2 * dir + 1)) & 1u;
    const int ar1 = dir == 0 ? ny - 3 : nx - 3, br1 = dir == 2 ? ny - 3 : nz - 3;
    for (int b = 3; b < br1; b++)
        for (int a = 3; a < ar1; a++) {
            int i0, j0, k0;
            if (dir == 0) { i0 = 0; j0 = a; k0 = b; }
            else if (dir == 1) { i0 = a; j0 = 0; k0 = b; }
            else { i0 = a; j0 = b; k0 = 0; }
            const double *L = &u[IX(i0, j0, k0)];
            double *O = &D[IX(i0, j0, k0)];
#define U(q) L[(q) * s]
            O[3 * s] = pre * (-U(7) + 6.0 * U(6) - 15.0 * U(5) + 20.0 * U(4) - 15.0 * U(3)
                              + 6.0 * U(2) - U(1));
            for (int p = 4; p < ie - 1; p++)
                O[p * s] = pre * (-U(p - 3) + 6.0 * U(p - 2) - 15.0 * U(p - 1) + 20.0 * U(p)
                                  - 15.0 * U(p + 1) + 6.0 * U(p + 2) - U(p + 3));
            O[(ie - 1) * s] = pre * (-U(ie + 1) + 6.0 * U(ie) - 15.0 * U(ie - 1) + 20.0 * U(ie - 2)
                                     - 15.0 * U(ie - 3) + 6.0 * U(ie - 4) - U(ie - 5));
            if (lo) {
                O[3 * s] = (U(6) - 3.0 * U(5) + 3.0 * U(4) - U(3)) / smr3;
                O[4 * s] = (U(7) - 6.0 * U(6) + 12.0 * U(5) - 10.0 * U(4) + 3.0 * U(3)) / smr2;
                O[5 * s] = (U(8) - 6.0 * U(7) + 15.0 * U(6) - 19.0 * U(5) + 12.0 * U(4) - 3.0 * U(3)) / smr1;
            }
            if (hi) {
                O[(ie - 3) * s] = (U(ie - 6) - 6.0 * U(ie - 5) + 15.0 * U(ie - 4) - 19.0 * U(ie - 3)
                                   + 12.0 * U(ie - 2) - 3.0 * U(ie - 1)) / smr1;
                O[(ie - 2) * s] = (U(ie - 5) - 6.0 * U(ie - 4) + 12.0 * U(ie - 3) - 10.0 * U(ie - 2)
                                   + 3.0 * U(ie - 1)) / smr2;
                O[(ie - 1) * s] = (U(ie - 4) - 3.0 * U(ie - 3) + 3.0 * U(ie - 2) - U(ie - 1)) / smr3;
            }
#undef U
        }
}

/* ---------------- point algebra ---------------- */
typedef struct {
    double a, psi, K, th, Gh[3], b[3], B[3], gt[3][3], At[3][3];
    double da[3], dpsi[3], dK[3], dth[3], dGh[3][3], db[3][3], dgt[3][3][3]; /* [c][dir], [i][j][dir] */
    double ada[3], adpsi[3], adK[3], adth[3], adGh[3][3], adb[3][3], adB[3][3];
    double adgt[3][3][3], adAt[3][3][3];
    double dda[3][3], ddpsi[3][3], ddb[3][3][3], ddgt[3][3][3][3]; /* [..][l][m] */
} orc_cpt4;

/* prm: lambda[4], lambda_f[2], kappa[2], p_expo, ...; out in CCZ4 variable order */
void orc_ccz4_point(const orc_cpt4 *P, const double *prm, double eta, double *out)
{
    const double l1 = prm[0], l2 = prm[1], l3 = prm[2], l4 = prm[3], lf0 = prm[4], lf1 = prm[5];
    const double k1 = prm[6], k2 = prm[7], p = prm[8];
    const double a = P->a, psi = P->psi, K = P->K, th = P->th;
    const double (*g)[3] = P->gt, (*A)[3] = P->At;
    const double *b = P->b, *Gh = P->Gh;
    double ig[3][3];
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

    double C1[3][3][3], C2[3][3][3], C3[3][3][3], CalGt[3];
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
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) s += ig[k][l] * C2[i][k][l];
        CalGt[i] = s;
    }
    double igdpsi[3];
    for (int i = 0; i < 3; i++) igdpsi[i] = ig[i][0] * P->dpsi[0] + ig[i][1] * P->dpsi[1] + ig[i][2] * P->dpsi[2];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                C3[i][j][k] = C2[i][j][k] + 0.5 * p / psi * ((i == j ? P->dpsi[k] : 0.0)
                                                            + (i == k ? P->dpsi[j] : 0.0)
                                                            - g[j][k] * igdpsi[i]);

    /* Ricci pieces (dendro_ccz4.py:539-589) */
    double RDZ[3][3], RDZTF[3][3];
    double Rtemp = 0.0;
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++)
            Rtemp += ig[k][l] * (P->ddpsi[k][l] + 0.5 * (p - 2.0) / psi * P->dpsi[k] * P->dpsi[l]);
    for (int m = 0; m < 3; m++) Rtemp -= Gh[m] * P->dpsi[m];
    Rtemp *= 0.5 * p / psi;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double t1 = 0.0, t2 = 0.0, t3 = 0.0, t4 = 0.0, c2p = 0.0, gg = 0.0;
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++) t1 += ig[l][m] * P->ddgt[i][j][l][m];
            for (int k = 0; k < 3; k++) t2 += g[k][i] * P->dGh[k][j] + g[k][j] * P->dGh[k][i];
            for (int k = 0; k < 3; k++) t3 += Gh[k] * (C1[i][j][k] + C1[j][i][k]);
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++)
                    for (int m = 0; m < 3; m++)
                        t4 += ig[l][m] * (C2[k][l][i] * C1[j][k][m] + C2[k][l][j] * C1[i][k][m]
                                          + C2[k][i][m] * C1[k][l][j]);
            const double Rt = -0.5 * t1 + 0.5 * t2 + 0.5 * t3 + t4;
            for (int k = 0; k < 3; k++) c2p += C2[k][i][j] * P->dpsi[k];
            const double RpsiTF = -0.5 * p / psi * (P->ddpsi[i][j] - c2p)
                                + 0.25 * p * (p + 2.0) / (psi * psi) * P->dpsi[i] * P->dpsi[j];
            for (int k = 0; k < 3; k++)
                gg += (Gh[k] - CalGt[k]) * (g[k][i] * P->dpsi[j] + g[k][j] * P->dpsi[i]);
            const double RDZpsiTF = RpsiTF - 0.5 * p / psi * gg;
            RDZTF[i][j] = RDZpsiTF + Rt;
            RDZ[i][j] = RDZpsiTF - g[i][j] * Rtemp + Rt;
        }

    double divb = P->db[0][0] + P->db[1][1] + P->db[2][2];
    const double psimp = pow(psi, -p);
    const double w = -2.0 / 3.0;

    /* lapse, shift (ccz4.py:59-64) */
    out[C_A] = l1 * (b[0] * P->ada[0] + b[1] * P->ada[1] + b[2] * P->ada[2]) - 2.0 * a * (K - 2.0 * th);
    for (int i = 0; i < 3; i++)
        out[C_B0_ + i] = 0.75 * (lf0 + lf1 * a) * P->B[i]
                       + l2 * (b[0] * P->adb[i][0] + b[1] * P->adb[i][1] + b[2] * P->adb[i][2]);
    /* conformal metric: Lie derivative of weight -2/3 (ccz4.py:67) */
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++)
                s += b[k] * P->adgt[i][j][k] + g[i][k] * P->db[k][j] + g[k][j] * P->db[k][i]
                   + w * g[i][j] * P->db[k][k];
            out[C_G0 + SYM4[i][j]] = s - 2.0 * a * A[i][j];
        }
    /* psi (ccz4.py:70) */
    out[C_PSI] = b[0] * P->adpsi[0] + b[1] * P->adpsi[1] + b[2] * P->adpsi[2]
               + 2.0 / 3.0 * psi * (divb - a * K) / p;
    /* At (ccz4.py:77) */
    double AikAkj[3][3], AUU[3][3], X[3][3], trX = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0, u2 = 0.0;
            for (int k = 0; k < 3; k++) {
                double t = 0.0;
                for (int l = 0; l < 3; l++) t += ig[k][l] * A[l][j];
                s += A[i][k] * t;
            }
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) u2 += ig[i][k] * ig[j][l] * A[k][l];
            AikAkj[i][j] = s;
            AUU[i][j] = u2;
            double c3a = 0.0;
            for (int l = 0; l < 3; l++) c3a += C3[l][i][j] * P->da[l];
            X[i][j] = a * RDZTF[i][j] - (P->dda[i][j] - c3a);
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) trX += ig[i][j] * X[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++)
                s += b[k] * P->adAt[i][j][k] + A[i][k] * P->db[k][j] + A[k][j] * P->db[k][i]
                   + w * A[i][j] * P->db[k][k];
            out[C_A0 + SYM4[i][j]] = s + psimp * (X[i][j] - g[i][j] * trX / 3.0)
                                   + a * ((K - 2.0 * th) * A[i][j] - 2.0 * AikAkj[i][j]);
        }
    /* K (ccz4.py:81).  The Laplacian of alpha carries psi^p, as the compiled
     * CCZ4_GR/src/ccz4eqs.cpp does (its factor is 1/psi at p = -1,
     * ccz4eqs.cpp:65 and :1041); the generator in the tree,
     * GR/rhs_scripts/ccz4/dendro_ccz4.py:318, writes psi^-p.  The compiled
     * code is what the solver runs, so it is the behaviour reproduced. */
    double lap = 0.0, trRDZ = 0.0;
    const double psip = pow(psi, p);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double c3a = 0.0;
            for (int k = 0; k < 3; k++) c3a += C3[k][i][j] * P->da[k];
            lap += psip * ig[i][j] * (P->dda[i][j] - c3a);
            trRDZ += ig[i][j] * RDZ[i][j];
        }
    out[C_K] = b[0] * P->adK[0] + b[1] * P->adK[1] + b[2] * P->adK[2] - lap
             + a * (psimp * trRDZ + K * (K - 2.0 * th) - 3.0 * k1 * (1.0 + k2) * th);
    /* Gh (ccz4.py:88-95) and B (:99-102) */
    double Ghr[3];
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int j = 0; j < 3; j++) s += b[j] * P->adGh[i][j];
        for (int j = 0; j < 3; j++) s -= Gh[j] * P->db[i][j];
        s += 2.0 / 3.0 * Gh[i] * divb;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                s += ig[j][k] * P->ddb[i][j][k] + ig[i][j] * P->ddb[k][j][k] / 3.0;
        for (int j = 0; j < 3; j++) s -= 2.0 * AUU[i][j] * P->da[j];
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) s += 2.0 * a * C2[i][j][k] * AUU[j][k];
        double t = 0.0;
        for (int j = 0; j < 3; j++)
            t += 3.0 * p / psi * AUU[i][j] * P->dpsi[j] - 4.0 / 3.0 * ig[i][j] * P->dK[j];
        s += a * t;
        double u = 0.0;
        for (int j = 0; j < 3; j++) u += ig[i][j] * (a * P->dth[j] - th * P->da[j]);
        s += 2.0 * (u - 0.5 * a * (k1 + 2.0 / 3.0 * K) * (Gh[i] - CalGt[i]));
        Ghr[i] = s;
        out[C_GH0 + i] = s;
    }
    for (int i = 0; i < 3; i++) {
        double aB = 0.0, aG = 0.0;
        for (int j = 0; j < 3; j++) {
            aB += b[j] * P->adB[i][j];
            aG += b[j] * P->adGh[i][j];
        }
        out[C_BB0 + i] = Ghr[i] - eta * P->B[i] + l3 * aB - l4 * aG;
    }
    /* theta_z4 (ccz4.py:104) */
    double sqrA = 0.0, GdA = 0.0;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) sqrA += A[i][j] * AUU[i][j];
        GdA += (Gh[i] - CalGt[i]) * P->da[i];
    }
    out[C_TH] = b[0] * P->adth[0] + b[1] * P->adth[1] + b[2] * P->adth[2]
              + 0.5 * a * (psimp * trRDZ + 2.0 * K * K / 3.0 - sqrA - 2.0 * th * K)
              - 0.5 * psimp * GdA - a * (k1 * (2.0 + k2) * th);
}

/* ---------------- block driver ---------------- */
/* second-derivative fields (CCZ4_GR/scripts/ccz4rhs_derivs.h, those the
 * algebra reads): alpha, psi, beta0-2, gt0-5 */
static const int D2F[11] = {C_A, C_PSI, C_B0_, C_B1_, C_B2_, C_G0, C_G1, C_G2, C_G3, C_G4, C_G5};
static const double FALL4[NV4] = {1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1,
                                  1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 0};
static const double ASYM4[NV4] = {1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                  1, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0};

/* prm: lambda[4], lambda_f[2], kappa[2], p_expo, eta_const, eta_r0,
 * eta_damping_exp, ko_sigma.  Returns -2 on allocation failure. */
int orc_ccz4rhs_ex(double **rhs, const double **uz, unsigned long offset, const double *pmin,
                   const double *pmax, const unsigned *sz, unsigned bflag, const double *prm,
                   int apply_bcs)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const size_t n = (size_t)nx * ny * nz;
    const double h[3] = {(pmax[0] - pmin[0]) / (nx - 1), (pmax[1] - pmin[1]) / (ny - 1),
                         (pmax[2] - pmin[2]) / (nz - 1)};
    double *pool = (double *)malloc(sizeof(double) * n * (NV4 * 3 * 2 + 11 * 6 + 3));
    if (!pool) return -2;
    double *grad[NV4][3], *adv[NV4][3], *d2[NV4][6];
    memset(d2, 0, sizeof d2);
    double *q = pool;
    for (int v = 0; v < NV4; v++)
        for (int d = 0; d < 3; d++) {
            grad[v][d] = q; q += n;
            adv[v][d] = q; q += n;
        }
    for (int f = 0; f < 11; f++)
        for (int m = 0; m < 6; m++) { d2[D2F[f]][m] = q; q += n; }
    double *kob = q;  /* 3 KO scratch lines */
    const double *u[NV4];
    for (int v = 0; v < NV4; v++) u[v] = uz[v] + offset;
    for (int v = 0; v < NV4; v++) {
        for (int d = 0; d < 3; d++) {
            orc_deriv42(d, grad[v][d], u[v], h[d], sz, bflag);
            orc_ccz4_adv42(d, adv[v][d], u[v], h[d], sz, u[C_B0_ + d], bflag);
        }
        if (d2[v][0]) {
            orc_deriv42_2(0, d2[v][0], u[v], h[0], sz, bflag);
            orc_deriv42_2(1, d2[v][3], u[v], h[1], sz, bflag);
            orc_deriv42_2(2, d2[v][5], u[v], h[2], sz, bflag);
            orc_deriv42(1, d2[v][1], grad[v][0], h[1], sz, bflag);
            orc_deriv42(2, d2[v][2], grad[v][0], h[2], sz, bflag);
            orc_deriv42(2, d2[v][4], grad[v][1], h[2], sz, bflag);
        }
    }
    const double ETA_CONST = prm[9], ETA_R0 = prm[10], ETA_EXP = prm[11], sigma = prm[12];
    static const int Q[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int k = 3; k < nz - 3; k++) {
        const double z = pmin[2] + k * h[2];
        for (int j = 3; j < ny - 3; j++) {
            const double y = pmin[1] + j * h[1];
            for (int i = 3; i < nx - 3; i++) {
                const double x = pmin[0] + i * h[0];
                const size_t pp = IX(i, j, k);
                const double r = sqrt(x * x + y * y + z * z);
                double eta = ETA_CONST;
                if (r >= ETA_R0) eta *= pow(ETA_R0 / r, ETA_EXP);
                orc_cpt4 P;
                P.a = u[C_A][pp]; P.psi = u[C_PSI][pp]; P.K = u[C_K][pp]; P.th = u[C_TH][pp];
                for (int c = 0; c < 3; c++) {
                    P.Gh[c] = u[C_GH0 + c][pp];
                    P.b[c] = u[C_B0_ + c][pp];
                    P.B[c] = u[C_BB0 + c][pp];
                }
                for (int aa = 0; aa < 3; aa++)
                    for (int bb = 0; bb < 3; bb++) {
                        P.gt[aa][bb] = u[C_G0 + SYM4[aa][bb]][pp];
                        P.At[aa][bb] = u[C_A0 + SYM4[aa][bb]][pp];
                    }
                for (int d = 0; d < 3; d++) {
                    P.da[d] = grad[C_A][d][pp];
                    P.dpsi[d] = grad[C_PSI][d][pp];
                    P.dK[d] = grad[C_K][d][pp];
                    P.dth[d] = grad[C_TH][d][pp];
                    P.ada[d] = adv[C_A][d][pp];
                    P.adpsi[d] = adv[C_PSI][d][pp];
                    P.adK[d] = adv[C_K][d][pp];
                    P.adth[d] = adv[C_TH][d][pp];
                    for (int c = 0; c < 3; c++) {
                        P.dGh[c][d] = grad[C_GH0 + c][d][pp];
                        P.db[c][d] = grad[C_B0_ + c][d][pp];
                        P.adGh[c][d] = adv[C_GH0 + c][d][pp];
                        P.adb[c][d] = adv[C_B0_ + c][d][pp];
                        P.adB[c][d] = adv[C_BB0 + c][d][pp];
                    }
                    for (int aa = 0; aa < 3; aa++)
                        for (int bb = 0; bb < 3; bb++) {
                            P.dgt[aa][bb][d] = grad[C_G0 + SYM4[aa][bb]][d][pp];
                            P.adgt[aa][bb][d] = adv[C_G0 + SYM4[aa][bb]][d][pp];
                            P.adAt[aa][bb][d] = adv[C_A0 + SYM4[aa][bb]][d][pp];
                        }
                }
                for (int l = 0; l < 3; l++)
                    for (int m = 0; m < 3; m++) {
                        const int qq = Q[l][m];
                        P.dda[l][m] = d2[C_A][qq][pp];
                        P.ddpsi[l][m] = d2[C_PSI][qq][pp];
                        for (int c = 0; c < 3; c++) P.ddb[c][l][m] = d2[C_B0_ + c][qq][pp];
                        for (int aa = 0; aa < 3; aa++)
                            for (int bb = 0; bb < 3; bb++)
                                P.ddgt[aa][bb][l][m] = d2[C_G0 + SYM4[aa][bb]][qq][pp];
                    }
                double out[NV4];
                orc_ccz4_point(&P, prm, eta, out);
                for (int v = 0; v < NV4; v++) rhs[v][offset + pp] = out[v];
            }
        }
    }
    if (bflag != 0 && apply_bcs)
        for (int v = 0; v < NV4 - 1; v++)
            orc_bssn_bcs(rhs[v] + offset, u[v], grad[v][0], grad[v][1], grad[v][2], pmin, pmax,
                         FALL4[v], ASYM4[v], sz, bflag);
    /* KO for every variable but theta_z4 */
    double *kx = kob, *ky = kob + n, *kz = kob + 2 * n;
    for (int v = 0; v < NV4 - 1; v++) {
        orc_ccz4_ko42(0, kx, u[v], h[0], sz, bflag);
        orc_ccz4_ko42(1, ky, u[v], h[1], sz, bflag);
        orc_ccz4_ko42(2, kz, u[v], h[2], sz, bflag);
        for (int k = 3; k < nz - 3; k++)
            for (int j = 3; j < ny - 3; j++)
                for (int i = 3; i < nx - 3; i++) {
                    const size_t pp = IX(i, j, k);
                    rhs[v][offset + pp] += sigma * (kx[pp] + ky[pp] + kz[pp]);
                }
    }
    free(pool);
    return 0;
}

int orc_ccz4rhs_blocks(double **rhs, const double **uz, long nblk, const unsigned long *off,
                       const unsigned *sz, const unsigned *bflag, const double *pmin,
                       const double *pmax, const double *prm, int apply_bcs, int nthreads)
{
    int err = 0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
    for (long b = 0; b < nblk; b++)
        err |= orc_ccz4rhs_ex(rhs, uz, off[b], pmin + 3 * b, pmax + 3 * b, sz + 3 * b, bflag[b], prm,
                              apply_bcs);
    return err;
}
