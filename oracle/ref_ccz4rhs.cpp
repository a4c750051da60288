/*
 * Test infrastructure only: a C-callable harness around the reference's OWN
 * per-block CCZ4 right-hand-side arithmetic, compiled from the reference
 * sources where they lie (see oracle/Makefile.ref).  Nothing here ships.
 *
 * It has the shape of ccz4rhs() (CCZ4_GR/src/rhs.cpp:12-298), the function
 * the RK4 solver calls (CCZ4_GR/src/rk4CCZ4.cpp:498): the 25 field pointers
 * at `offset`, h = (pmax - pmin)/(n - 1), the generated derivative drivers
 * CCZ4_GR/scripts/ccz4rhs_{derivs,derivs_adv}.h with the 4th-order stencils
 * of CCZ4_GR/src/derivs.cpp (the binding of CCZ4_GR/include/rhs.h:14-28),
 * the generated point algebra CCZ4_GR/src/ccz4eqs.cpp inside the interior
 * loop with eta(r), the KO drivers and the KO accumulate loop (which leaves
 * theta_z4 out, rhs.cpp:241-283).  Domain-boundary blocks get the one-sided
 * stencils and the outgoing-radiation condition ccz4_bcs, extracted verbatim
 * from CCZ4_GR/src/rhs.cpp at build time (oracle/Makefile.ref), called for
 * every variable but theta_z4 with the falloff and asymptotic values of the
 * solver's ccz4rhs (rhs.cpp:170-228).
 */
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "derivs.h"

#include "ccz4_bcs.inc"

#define deriv_x deriv42_x
#define deriv_y deriv42_y
#define deriv_z deriv42_z
#define deriv_xx deriv42_xx
#define deriv_yy deriv42_yy
#define deriv_zz deriv42_zz
#define adv_deriv_x deriv42adv_x
#define adv_deriv_y deriv42adv_y
#define adv_deriv_z deriv42adv_z
#define ko_deriv_x ko_deriv42_x
#define ko_deriv_y ko_deriv42_y
#define ko_deriv_z ko_deriv42_z

using std::pow;
using std::sqrt;

namespace {
enum { V_ALPHA = 0, V_PSI, V_K, V_GH0, V_GH1, V_GH2, V_BETA0, V_BETA1, V_BETA2, V_B0, V_B1,
       V_B2, V_SYMGT0, V_SYMGT1, V_SYMGT2, V_SYMGT3, V_SYMGT4, V_SYMGT5, V_SYMAT0, V_SYMAT1,
       V_SYMAT2, V_SYMAT3, V_SYMAT4, V_SYMAT5, V_THETA_Z4 };
}

/* prm layout: lambda[4], lambda_f[2], kappa[2], p_expo, eta_const, eta_r0,
 * eta_damping_exp, ko_sigma */
extern "C" int ref_ccz4rhs(double **unzipVarsRHS, const double **uZipVars, unsigned int offset,
                           const double *pmin, const double *pmax, const unsigned int *sz,
                           unsigned int bflag, const double *prm)
{
    const unsigned int lambda[4] = {(unsigned)prm[0], (unsigned)prm[1], (unsigned)prm[2],
                                    (unsigned)prm[3]};
    const double lambda_f[2] = {prm[4], prm[5]};
    const double kappa[2] = {prm[6], prm[7]};
    const double p_expo = prm[8];
    const double ETA_CONST = prm[9], ETA_R0 = prm[10], ETA_DAMPING_EXP = prm[11];
    const double KO_DISS_SIGMA = prm[12];
    (void)p_expo;

#define IN_(name, v) const double *name = &uZipVars[v][offset]
#define OUT_(name, v) double *name = &unzipVarsRHS[v][offset]
    IN_(alpha, V_ALPHA); IN_(psi, V_PSI); IN_(theta_z4, V_THETA_Z4); IN_(K, V_K);
    IN_(gt0, V_SYMGT0); IN_(gt1, V_SYMGT1); IN_(gt2, V_SYMGT2);
    IN_(gt3, V_SYMGT3); IN_(gt4, V_SYMGT4); IN_(gt5, V_SYMGT5);
    IN_(beta0, V_BETA0); IN_(beta1, V_BETA1); IN_(beta2, V_BETA2);
    IN_(At0, V_SYMAT0); IN_(At1, V_SYMAT1); IN_(At2, V_SYMAT2);
    IN_(At3, V_SYMAT3); IN_(At4, V_SYMAT4); IN_(At5, V_SYMAT5);
    IN_(Gh0, V_GH0); IN_(Gh1, V_GH1); IN_(Gh2, V_GH2);
    IN_(B0, V_B0); IN_(B1, V_B1); IN_(B2, V_B2);
    OUT_(a_rhs, V_ALPHA); OUT_(psi_rhs, V_PSI); OUT_(K_rhs, V_K);
    OUT_(gt_rhs00, V_SYMGT0); OUT_(gt_rhs01, V_SYMGT1); OUT_(gt_rhs02, V_SYMGT2);
    OUT_(gt_rhs11, V_SYMGT3); OUT_(gt_rhs12, V_SYMGT4); OUT_(gt_rhs22, V_SYMGT5);
    OUT_(b_rhs0, V_BETA0); OUT_(b_rhs1, V_BETA1); OUT_(b_rhs2, V_BETA2);
    OUT_(At_rhs00, V_SYMAT0); OUT_(At_rhs01, V_SYMAT1); OUT_(At_rhs02, V_SYMAT2);
    OUT_(At_rhs11, V_SYMAT3); OUT_(At_rhs12, V_SYMAT4); OUT_(At_rhs22, V_SYMAT5);
    OUT_(Gh_rhs0, V_GH0); OUT_(Gh_rhs1, V_GH1); OUT_(Gh_rhs2, V_GH2);
    OUT_(B_rhs0, V_B0); OUT_(B_rhs1, V_B1); OUT_(B_rhs2, V_B2);
    OUT_(theta_z4_rhs, V_THETA_Z4);
#undef IN_
#undef OUT_

    const unsigned int nx = sz[0], ny = sz[1], nz = sz[2];
    const double hx = (pmax[0] - pmin[0]) / (nx - 1);
    const double hy = (pmax[1] - pmin[1]) / (ny - 1);
    const double hz = (pmax[2] - pmin[2]) / (nz - 1);
    const unsigned int n = nx * ny * nz;

#include "ccz4rhs_memalloc.h"
#include "ccz4rhs_memalloc_adv.h"
#include "ccz4rhs_derivs.h"
#include "ccz4rhs_derivs_adv.h"

    for (unsigned int k = 3; k < nz - 3; k++) {
        const double z = pmin[2] + k * hz;
        for (unsigned int j = 3; j < ny - 3; j++) {
            const double y = pmin[1] + j * hy;
            for (unsigned int i = 3; i < nx - 3; i++) {
                const double x = pmin[0] + i * hx;
                const unsigned int pp = i + nx * (j + ny * k);
                const double r_coord = sqrt(x * x + y * y + z * z);
                double eta = ETA_CONST;
                if (r_coord >= ETA_R0) eta *= pow((ETA_R0 / r_coord), ETA_DAMPING_EXP);
#include "ccz4eqs.cpp"
            }
        }
    }

    if (bflag != 0) {
        struct Bc {
            double *rhs;
            const double *f, *dx, *dy, *dz;
            double falloff, asymptotic;
        };
        const Bc bcs[24] = {
            {a_rhs, alpha, grad_0_alpha, grad_1_alpha, grad_2_alpha, 1.0, 1.0},
            {psi_rhs, psi, grad_0_psi, grad_1_psi, grad_2_psi, 1.0, 1.0},
            {K_rhs, K, grad_0_K, grad_1_K, grad_2_K, 1.0, 0.0},
            {b_rhs0, beta0, grad_0_beta0, grad_1_beta0, grad_2_beta0, 1.0, 0.0},
            {b_rhs1, beta1, grad_0_beta1, grad_1_beta1, grad_2_beta1, 1.0, 0.0},
            {b_rhs2, beta2, grad_0_beta2, grad_1_beta2, grad_2_beta2, 1.0, 0.0},
            {Gh_rhs0, Gh0, grad_0_Gh0, grad_1_Gh0, grad_2_Gh0, 2.0, 0.0},
            {Gh_rhs1, Gh1, grad_0_Gh1, grad_1_Gh1, grad_2_Gh1, 2.0, 0.0},
            {Gh_rhs2, Gh2, grad_0_Gh2, grad_1_Gh2, grad_2_Gh2, 2.0, 0.0},
            {B_rhs0, B0, grad_0_B0, grad_1_B0, grad_2_B0, 1.0, 0.0},
            {B_rhs1, B1, grad_0_B1, grad_1_B1, grad_2_B1, 1.0, 0.0},
            {B_rhs2, B2, grad_0_B2, grad_1_B2, grad_2_B2, 1.0, 0.0},
            {At_rhs00, At0, grad_0_At0, grad_1_At0, grad_2_At0, 2.0, 0.0},
            {At_rhs01, At1, grad_0_At1, grad_1_At1, grad_2_At1, 2.0, 0.0},
            {At_rhs02, At2, grad_0_At2, grad_1_At2, grad_2_At2, 2.0, 0.0},
            {At_rhs11, At3, grad_0_At3, grad_1_At3, grad_2_At3, 2.0, 0.0},
            {At_rhs12, At4, grad_0_At4, grad_1_At4, grad_2_At4, 2.0, 0.0},
            {At_rhs22, At5, grad_0_At5, grad_1_At5, grad_2_At5, 2.0, 0.0},
            {gt_rhs00, gt0, grad_0_gt0, grad_1_gt0, grad_2_gt0, 1.0, 1.0},
            {gt_rhs01, gt1, grad_0_gt1, grad_1_gt1, grad_2_gt1, 1.0, 0.0},
            {gt_rhs02, gt2, grad_0_gt2, grad_1_gt2, grad_2_gt2, 1.0, 0.0},
            {gt_rhs11, gt3, grad_0_gt3, grad_1_gt3, grad_2_gt3, 1.0, 1.0},
            {gt_rhs12, gt4, grad_0_gt4, grad_1_gt4, grad_2_gt4, 1.0, 0.0},
            {gt_rhs22, gt5, grad_0_gt5, grad_1_gt5, grad_2_gt5, 1.0, 1.0}};
        for (const Bc &c : bcs)
            ccz4_bcs(c.rhs, c.f, c.dx, c.dy, c.dz, pmin, pmax, c.falloff, c.asymptotic, sz, bflag);
    }

#include "ccz4rhs_ko_derivs.h"

    const double sigma = KO_DISS_SIGMA;
    for (unsigned int k = 3; k < nz - 3; k++)
        for (unsigned int j = 3; j < ny - 3; j++)
            for (unsigned int i = 3; i < nx - 3; i++) {
                const unsigned int pp = i + nx * (j + ny * k);
                a_rhs[pp] += sigma * (grad_0_alpha[pp] + grad_1_alpha[pp] + grad_2_alpha[pp]);
                b_rhs0[pp] += sigma * (grad_0_beta0[pp] + grad_1_beta0[pp] + grad_2_beta0[pp]);
                b_rhs1[pp] += sigma * (grad_0_beta1[pp] + grad_1_beta1[pp] + grad_2_beta1[pp]);
                b_rhs2[pp] += sigma * (grad_0_beta2[pp] + grad_1_beta2[pp] + grad_2_beta2[pp]);
                gt_rhs00[pp] += sigma * (grad_0_gt0[pp] + grad_1_gt0[pp] + grad_2_gt0[pp]);
                gt_rhs01[pp] += sigma * (grad_0_gt1[pp] + grad_1_gt1[pp] + grad_2_gt1[pp]);
                gt_rhs02[pp] += sigma * (grad_0_gt2[pp] + grad_1_gt2[pp] + grad_2_gt2[pp]);
                gt_rhs11[pp] += sigma * (grad_0_gt3[pp] + grad_1_gt3[pp] + grad_2_gt3[pp]);
                gt_rhs12[pp] += sigma * (grad_0_gt4[pp] + grad_1_gt4[pp] + grad_2_gt4[pp]);
                gt_rhs22[pp] += sigma * (grad_0_gt5[pp] + grad_1_gt5[pp] + grad_2_gt5[pp]);
                psi_rhs[pp] += sigma * (grad_0_psi[pp] + grad_1_psi[pp] + grad_2_psi[pp]);
                At_rhs00[pp] += sigma * (grad_0_At0[pp] + grad_1_At0[pp] + grad_2_At0[pp]);
                At_rhs01[pp] += sigma * (grad_0_At1[pp] + grad_1_At1[pp] + grad_2_At1[pp]);
                At_rhs02[pp] += sigma * (grad_0_At2[pp] + grad_1_At2[pp] + grad_2_At2[pp]);
                At_rhs11[pp] += sigma * (grad_0_At3[pp] + grad_1_At3[pp] + grad_2_At3[pp]);
                At_rhs12[pp] += sigma * (grad_0_At4[pp] + grad_1_At4[pp] + grad_2_At4[pp]);
                At_rhs22[pp] += sigma * (grad_0_At5[pp] + grad_1_At5[pp] + grad_2_At5[pp]);
                K_rhs[pp] += sigma * (grad_0_K[pp] + grad_1_K[pp] + grad_2_K[pp]);
                Gh_rhs0[pp] += sigma * (grad_0_Gh0[pp] + grad_1_Gh0[pp] + grad_2_Gh0[pp]);
                Gh_rhs1[pp] += sigma * (grad_0_Gh1[pp] + grad_1_Gh1[pp] + grad_2_Gh1[pp]);
                Gh_rhs2[pp] += sigma * (grad_0_Gh2[pp] + grad_1_Gh2[pp] + grad_2_Gh2[pp]);
                B_rhs0[pp] += sigma * (grad_0_B0[pp] + grad_1_B0[pp] + grad_2_B0[pp]);
                B_rhs1[pp] += sigma * (grad_0_B1[pp] + grad_1_B1[pp] + grad_2_B1[pp]);
                B_rhs2[pp] += sigma * (grad_0_B2[pp] + grad_1_B2[pp] + grad_2_B2[pp]);
            }

#include "ccz4rhs_dealloc.h"
#include "ccz4rhs_dealloc_adv.h"
    return 0;
}

#define REF_STENCIL(name, fn) \
    extern "C" void name(double *D, const double *u, double h, const unsigned *sz, unsigned bflag) \
    { fn(D, u, h, sz, bflag); }
#define REF_ADV(name, fn) \
    extern "C" void name(double *D, const double *u, double h, const unsigned *sz, \
                         const double *beta, unsigned bflag) \
    { fn(D, u, h, sz, beta, bflag); }
REF_STENCIL(ccz4_deriv42_x, deriv42_x)
REF_STENCIL(ccz4_deriv42_y, deriv42_y)
REF_STENCIL(ccz4_deriv42_z, deriv42_z)
REF_STENCIL(ccz4_deriv42_xx, deriv42_xx)
REF_STENCIL(ccz4_deriv42_yy, deriv42_yy)
REF_STENCIL(ccz4_deriv42_zz, deriv42_zz)
REF_STENCIL(ccz4_ko_deriv42_x, ko_deriv42_x)
REF_STENCIL(ccz4_ko_deriv42_y, ko_deriv42_y)
REF_STENCIL(ccz4_ko_deriv42_z, ko_deriv42_z)
REF_ADV(ccz4_deriv42adv_x, deriv42adv_x)
REF_ADV(ccz4_deriv42adv_y, deriv42adv_y)
REF_ADV(ccz4_deriv42adv_z, deriv42adv_z)
