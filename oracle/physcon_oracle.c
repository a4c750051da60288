/*
 * ORACLE — test infrastructure only.  C restatement of the reference's
 * constraint diagnostics physical_constraints (BSSN_GR/src/physcon.cpp:12-96):
 * 4th-order stencils (BSSN_GR/include/physcon.h:9-15 binds deriv42_*,
 * BSSN_GR/src/derivs.cpp:11-490, with their one-sided closures), the
 * derivative set of BSSN_GR/scripts/constraint_derivs.h, and the
 * Hamiltonian, momentum and Psi4 expressions of CodeGen/constraints.py
 * (tetrad :52-100, Psi4 :102-152, constraints :158-172) written as index
 * loops, reusing the Ricci tensor of CodeGen/dendro.py:443-527.
 * Output order: ham, mom0, mom1, mom2, psi4_real, psi4_img
 * (bssn::VAR_CONSTRAINT, BSSN_GR/include/grDef.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define IX(i, j, k) ((i) + nx * ((j) + ny * (k)))
enum { A_ = 0, CHI_, K_, GT0_, GT1_, GT2_, BETA0_, BETA1_, BETA2_, B0_, B1_, B2_,
       SGT0_, SGT1_, SGT2_, SGT3_, SGT4_, SGT5_, SAT0_, SAT1_, SAT2_, SAT3_, SAT4_, SAT5_ };
static const int SYM3[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};

/* deriv42 along dir; loop ranges of the reference: dir 0: i in [3,n-3),
 * j,k in [1,n-1); dir 1: i,j in [3,n-3), k in [1,n-1); dir 2: interior. */
void orc_deriv42(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double idx = 1.0 / h, idx_by_2 = 0.5 * idx, idx_by_12 = idx / 12.0;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    const int n = dir == 0 ? nx : dir == 1 ? ny : nz;
    const int jb = dir == 0 ? 1 : 3, je = dir == 0 ? ny - 1 : ny - 3;
    const int kb = dir == 2 ? 3 : 1, ke = dir == 2 ? nz - 3 : nz - 1;
    for (int k = kb; k < ke; k++)
        for (int j = jb; j < je; j++)
            for (int i = 3; i < nx - 3; i++) {
                const double *c = &u[IX(i, j, k)];
                D[IX(i, j, k)] = (c[-2 * s] - 8.0 * c[-s] + 8.0 * c[s] - c[2 * s]) * idx_by_12;
            }
    const int lo = (bflag >> (2 * dir)) & 1u, hi = (bflag >> (2 * dir + 1)) & 1u;
    if (!lo && !hi) return;
    /* closures: (a, b) over the other axes with the main loop's ranges */
    const int ar0 = dir == 0 ? jb : 3, ar1 = dir == 0 ? je : nx - 3;
    const int br0 = dir == 2 ? 3 : kb, br1 = dir == 2 ? ny - 3 : ke;
    for (int b = br0; b < br1; b++)
        for (int a = ar0; a < ar1; a++) {
            int i0, j0, k0;
            if (dir == 0) { i0 = 0; j0 = a; k0 = b; }
            else if (dir == 1) { i0 = a; j0 = 0; k0 = b; }
            else { i0 = a; j0 = b; k0 = 0; }
            const double *L = &u[IX(i0, j0, k0)];
            double *O = &D[IX(i0, j0, k0)];
            if (lo) {
                O[3 * s] = (-3.0 * L[3 * s] + 4.0 * L[4 * s] - L[5 * s]) * idx_by_2;
                O[4 * s] = (-L[3 * s] + L[5 * s]) * idx_by_2;
            }
            if (hi) {
                const int ie = n - 3;
                O[(ie - 2) * s] = (-L[(ie - 3) * s] + L[(ie - 1) * s]) * idx_by_2;
                O[(ie - 1) * s] = (L[(ie - 3) * s] - 4.0 * L[(ie - 2) * s] + 3.0 * L[(ie - 1) * s]) * idx_by_2;
            }
        }
}

void orc_deriv42_2(int dir, double *D, const double *u, double h, const unsigned *sz, unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const double idx_sqrd = 1.0 / (h * h), idx_sqrd_by_12 = idx_sqrd / 12.0;
    const long s = dir == 0 ? 1 : dir == 1 ? nx : (long)nx * ny;
    const int n = dir == 0 ? nx : dir == 1 ? ny : nz;
    for (int k = 3; k < nz - 3; k++)
        for (int j = 3; j < ny - 3; j++)
            for (int i = 3; i < nx - 3; i++) {
                const double *c = &u[IX(i, j, k)];
                D[IX(i, j, k)] = (-c[-2 * s] + 16.0 * c[-s] - 30.0 * c[0] + 16.0 * c[s] - c[2 * s])
                               * idx_sqrd_by_12;
            }
    const int lo = (bflag >> (2 * dir)) & 1u, hi = (bflag >> (2 * dir + 1)) & 1u;
    if (!lo && !hi) return;
    const int ar1 = dir == 0 ? ny - 3 : nx - 3, br1 = dir == 2 ? ny - 3 : nz - 3;
    for (int b = 3; b < br1; b++)
        for (int a = 3; a < ar1; a++) {
            int i0, j0, k0;
            if (dir == 0) { i0 = 0; j0 = a; k0 = b; }
            else if (dir == 1) { i0 = a; j0 = 0; k0 = b; }
            else { i0 = a; j0 = b; k0 = 0; }
            const double *L = &u[IX(i0, j0, k0)];
            double *O = &D[IX(i0, j0, k0)];
            if (lo) {
                O[3 * s] = (2.0 * L[3 * s] - 5.0 * L[4 * s] + 4.0 * L[5 * s] - L[6 * s]) * idx_sqrd;
                O[4 * s] = (L[3 * s] - 2.0 * L[4 * s] + L[5 * s]) * idx_sqrd;
            }
            if (hi) {
                const int ie = n - 3;
                O[(ie - 2) * s] = (L[(ie - 3) * s] - 2.0 * L[(ie - 2) * s] + L[(ie - 1) * s]) * idx_sqrd;
                O[(ie - 1) * s] = (-L[(ie - 4) * s] + 4.0 * L[(ie - 3) * s] - 5.0 * L[(ie - 2) * s]
                                   + 2.0 * L[(ie - 1) * s]) * idx_sqrd;
            }
        }
}

/* ---------------- constraint point algebra ---------------- */
typedef struct {
    double chi, K, Gt[3], gt[3][3], At[3][3];
    double dchi[3], dK[3], dGt[3][3], dgt[3][3][3], dAt[3][3][3]; /* [..][dir] */
    double ddgt[3][3][3][3], ddchi[3][3];
} orc_cpoint;

void orc_constraint_point(const orc_cpoint *P, double x, double y, double z, double *out)
{
    const double chi = P->chi, K = P->K;
    const double (*g)[3] = P->gt;
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

    double C1[3][3][3], C2[3][3][3], CalGt[3];
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
    /* Ricci (dendro.py:443-527), as in the RHS */
    double R[3][3];
    double trchi = 0.0, CalGtdchi = 0.0;
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++)
            trchi += ig[k][l] * (P->ddchi[k][l] - 3.0 / (2.0 * chi) * P->dchi[k] * P->dchi[l]);
    for (int m = 0; m < 3; m++) CalGtdchi += CalGt[m] * P->dchi[m];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double t1 = 0.0, t2 = 0.0, t3 = 0.0, t4 = 0.0, c2d = 0.0;
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++) t1 += ig[l][m] * P->ddgt[i][j][l][m];
            for (int k = 0; k < 3; k++) t2 += g[k][i] * P->dGt[k][j] + g[k][j] * P->dGt[k][i];
            for (int k = 0; k < 3; k++) t3 += CalGt[k] * (C1[i][j][k] + C1[j][i][k]);
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++)
                    for (int m = 0; m < 3; m++)
                        t4 += ig[l][m] * (C2[k][l][i] * C1[j][k][m] + C2[k][l][j] * C1[i][k][m]
                                          + C2[k][i][m] * C1[k][l][j]);
            for (int k = 0; k < 3; k++) c2d += C2[k][j][i] * P->dchi[k];
            const double xR = 1.0 / (2.0 * chi) * (P->ddchi[i][j] - c2d)
                            - 1.0 / (4.0 * chi * chi) * P->dchi[i] * P->dchi[j];
            R[i][j] = -0.5 * t1 + 0.5 * t2 + 0.5 * t3 + t4 + xR
                    + 1.0 / (2.0 * chi) * g[i][j] * (trchi - CalGtdchi);
        }

    /* Hamiltonian and momentum constraints (constraints.py:158-172) */
    double sqrA = 0.0, chiR = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) s += ig[i][k] * ig[j][l] * P->At[k][l];
            sqrA += P->At[i][j] * s;
            chiR += chi * ig[i][j] * R[i][j];
        }
    out[0] = chiR - sqrA + 2.0 / 3.0 * K * K;
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                double c = 0.0;
                for (int m = 0; m < 3; m++) c += C2[m][k][i] * P->At[j][m];
                s += ig[j][k] * (P->dAt[i][j][k] - c);
            }
        for (int j = 0; j < 3; j++) s -= P->Gt[j] * P->At[i][j];
        double t = 0.0;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) t += ig[j][k] * P->At[k][i] * P->dchi[j] / chi;
        s -= 3.0 / 2.0 * t;
        s -= 2.0 / 3.0 * P->dK[i];
        out[1 + i] = s;
    }

    /* Psi4 (constraints.py:52-152); zero on the z axis, where the tetrad is
     * undefined (the guard of BSSN_GR/src/physconeqs.cpp:1039-1044) */
    if (fabs(x) <= 1e-7 && fabs(y) <= 1e-7) {
        out[4] = out[5] = 0.0;
        return;
    }
    const double invsqrt2 = 0.7071067811865475244;
    const double inv_chi = 1.0 / chi;
    double gd[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) gd[i][j] = g[i][j] * inv_chi;
    double rv[3] = {x, y, z}, th[3] = {x * z, y * z, -(x * x + y * y)}, ph[3] = {-y, x, 0.0};
    double ip = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) ip += gd[i][j] * rv[i] * rv[j];
    for (int i = 0; i < 3; i++) rv[i] /= sqrt(ip);
    double ip1 = 0.0, ip2 = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            ip1 += gd[i][j] * th[i] * th[j];
            ip2 += gd[i][j] * rv[i] * th[j];
        }
    for (int i = 0; i < 3; i++) th[i] -= ip2 * rv[i];
    for (int i = 0; i < 3; i++) th[i] /= sqrt(ip1 - ip2 * ip2);
    double ip3 = 0.0;
    ip1 = ip2 = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            ip1 += gd[i][j] * ph[i] * ph[j];
            ip2 += gd[i][j] * rv[i] * ph[j];
            ip3 += gd[i][j] * th[i] * ph[j];
        }
    for (int i = 0; i < 3; i++) ph[i] -= ip2 * rv[i] + ip3 * th[i];
    for (int i = 0; i < 3; i++) ph[i] /= sqrt(ip1 - ip2 * ip2 - ip3 * ip3);
    double mre[3], mim[3];
    for (int i = 0; i < 3; i++) { mre[i] = th[i] * invsqrt2; mim[i] = ph[i] * invsqrt2; }
    double MM[3][3], NN[3][3], MR[3][3], NR[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            MM[i][j] = mre[i] * mre[j] - mim[i] * mim[j];
            NN[i][j] = mre[i] * mim[j] + mre[j] * mim[i];
            MR[i][j] = mre[i] * rv[j] - mre[j] * rv[i];
            NR[i][j] = mim[i] * rv[j] - mim[j] * rv[i];
        }
    double Av[3];
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int j = 0; j < 3; j++) s += P->At[i][j] * rv[j];
        Av[i] = s;
    }
    double Uu[3][3], Vv[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double su = 0.0, sv = 0.0;
            for (int k = 0; k < 3; k++) {
                double c = P->dAt[k][i][j];
                for (int m = 0; m < 3; m++) c += C2[m][k][i] * P->At[m][j];
                su += mre[k] * c;
                sv += mim[k] * c;
            }
            Uu[i][j] = su;
            Vv[i][j] = sv;
        }
    double rdchi = 0.0, mredchi = 0.0, mimdchi = 0.0, mreA = 0.0, mimA = 0.0, Ar = 0.0;
    for (int i = 0; i < 3; i++) {
        rdchi += rv[i] * P->dchi[i];
        mredchi += mre[i] * P->dchi[i];
        mimdchi += mim[i] * P->dchi[i];
        mreA += mre[i] * Av[i];
        mimA += mim[i] * Av[i];
        Ar += Av[i] * rv[i];
    }
    const double Atemp = inv_chi * inv_chi * (Ar + K * chi / 3.0 + 0.5 * rdchi);
    double p1r = 0.0, p1i = 0.0, p2r = 0.0, p2i = 0.0;
    for (int i = 0; i < 3; i++) {
        p1r += R[i][i] * MM[i][i];
        p1i += R[i][i] * NN[i][i];
        p2r += P->At[i][i] * MM[i][i];
        p2i += P->At[i][i] * NN[i][i];
    }
    for (int i = 0; i < 2; i++)
        for (int j = i + 1; j < 3; j++) {
            p1r += 2.0 * R[i][j] * MM[i][j];
            p1i += 2.0 * R[i][j] * NN[i][j];
            p2r += 2.0 * P->At[i][j] * MM[i][j];
            p2i += 2.0 * P->At[i][j] * NN[i][j];
        }
    p2r *= Atemp;
    p2i *= Atemp;
    double p3r = 0.0, p3i = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            p3r += MR[i][j] * Uu[i][j] - NR[i][j] * Vv[i][j];
            p3i += NR[i][j] * Uu[i][j] + MR[i][j] * Vv[i][j];
        }
    p3r *= inv_chi;
    p3i *= inv_chi;
    const double p4r = inv_chi * inv_chi * (mreA * (mreA + 0.5 * mredchi) - mimA * (mimA + 0.5 * mimdchi));
    const double p4i = inv_chi * inv_chi * (mreA * (mimA - 0.5 * mimdchi) + mimA * (mreA - 0.5 * mredchi));
    out[4] = p1r + p2r - p3r - p4r;
    out[5] = -(p1i + p2i - p3i - p4i);
}

/* physical_constraints for one block; cons[c] + offset written at interior
 * points.  Returns -2 on allocation failure. */
static const int CFIELDS[17] = {CHI_, GT0_, GT1_, GT2_, K_, SGT0_, SGT1_, SGT2_, SGT3_, SGT4_,
                                SGT5_, SAT0_, SAT1_, SAT2_, SAT3_, SAT4_, SAT5_};

int orc_physcon_block(double **cons, const double **uz, unsigned long offset, const double *pmin,
                      const double *pmax, const unsigned *sz, unsigned bflag)
{
    const int nx = sz[0], ny = sz[1], nz = sz[2];
    const size_t n = (size_t)nx * ny * nz;
    const double h[3] = {(pmax[0] - pmin[0]) / (nx - 1), (pmax[1] - pmin[1]) / (ny - 1),
                         (pmax[2] - pmin[2]) / (nz - 1)};
    /* first derivatives of 17 fields, second (incl. mixed) of gt and chi */
    double *pool = (double *)malloc(sizeof(double) * n * (17 * 3 + 7 * 6));
    if (!pool) return -2;
    double *grad[24][3], *grad2[24][6];
    memset(grad, 0, sizeof grad);
    memset(grad2, 0, sizeof grad2);
    double *p = pool;
    for (int q = 0; q < 17; q++) {
        const int v = CFIELDS[q];
        for (int d = 0; d < 3; d++) { grad[v][d] = p; p += n; }
        if (v == CHI_ || (v >= SGT0_ && v <= SGT5_))
            for (int m = 0; m < 6; m++) { grad2[v][m] = p; p += n; }
    }
    for (int q = 0; q < 17; q++) {
        const int v = CFIELDS[q];
        const double *u = uz[v] + offset;
        for (int d = 0; d < 3; d++) orc_deriv42(d, grad[v][d], u, h[d], sz, bflag);
        if (grad2[v][0]) {
            orc_deriv42_2(0, grad2[v][0], u, h[0], sz, bflag);
            orc_deriv42_2(1, grad2[v][3], u, h[1], sz, bflag);
            orc_deriv42_2(2, grad2[v][5], u, h[2], sz, bflag);
            orc_deriv42(1, grad2[v][1], grad[v][0], h[1], sz, bflag);
            orc_deriv42(2, grad2[v][2], grad[v][0], h[2], sz, bflag);
            orc_deriv42(2, grad2[v][4], grad[v][1], h[2], sz, bflag);
        }
    }
    static const int Q[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int k = 3; k < nz - 3; k++) {
        const double z = pmin[2] + k * h[2];
        for (int j = 3; j < ny - 3; j++) {
            const double y = pmin[1] + j * h[1];
            for (int i = 3; i < nx - 3; i++) {
                const double x = pmin[0] + i * h[0];
                const size_t pp = IX(i, j, k);
                orc_cpoint P;
#define F(v) (uz[v][offset + pp])
                P.chi = F(CHI_); P.K = F(K_);
                for (int c = 0; c < 3; c++) P.Gt[c] = F(GT0_ + c);
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) {
                        P.gt[a][b] = F(SGT0_ + SYM3[a][b]);
                        P.At[a][b] = F(SAT0_ + SYM3[a][b]);
                    }
#undef F
                for (int d = 0; d < 3; d++) {
                    P.dchi[d] = grad[CHI_][d][pp];
                    P.dK[d] = grad[K_][d][pp];
                    for (int c = 0; c < 3; c++) P.dGt[c][d] = grad[GT0_ + c][d][pp];
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++) {
                            P.dgt[a][b][d] = grad[SGT0_ + SYM3[a][b]][d][pp];
                            P.dAt[a][b][d] = grad[SAT0_ + SYM3[a][b]][d][pp];
                        }
                }
                for (int l = 0; l < 3; l++)
                    for (int m = 0; m < 3; m++) {
                        P.ddchi[l][m] = grad2[CHI_][Q[l][m]][pp];
                        for (int a = 0; a < 3; a++)
                            for (int b = 0; b < 3; b++)
                                P.ddgt[a][b][l][m] = grad2[SGT0_ + SYM3[a][b]][Q[l][m]][pp];
                    }
                double out[6];
                orc_constraint_point(&P, x, y, z, out);
                for (int c = 0; c < 6; c++) cons[c][offset + pp] = out[c];
            }
        }
    }
    free(pool);
    return 0;
}

/* physical_constraints over a block list (the per-block loop of
 * BSSN_GR/src/gr.cpp's constraint output), blocks in parallel. */
int orc_physcon_blocks(double **cons, const double **uz, long nblk, const unsigned long *off,
                       const unsigned *sz, const unsigned *bflag, const double *pmin,
                       const double *pmax, int nthreads)
{
    int err = 0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
    for (long b = 0; b < nblk; b++)
        err |= orc_physcon_block(cons, uz, off[b], pmin + 3 * b, pmax + 3 * b, sz + 3 * b, bflag[b]);
    return err;
}
