/*
 * Test infrastructure only: a C-callable harness around the reference's OWN
 * per-block BSSN right-hand-side arithmetic, compiled from the reference
 * sources where they lie (see oracle/Makefile.ref).  Nothing here ships.
 *
 * It has the shape of bssnrhs() (BSSN_GR/src/rhs.cpp:86-392): the 24 field
 * pointers at `offset`, h = (pmax - pmin)/(n - 1) (rhs.cpp:148-150), the
 * generated derivative drivers (BSSN_GR/scripts/bssnrhs_*.h), the generated
 * point algebra BSSN_GR/src/bssneqs_eta_const_standard_gauge.cpp inside the
 * interior loop with eta(r) (rhs.cpp:210-262), the generated KO drivers and
 * the KO accumulate loop (rhs.cpp:328-373).  The stencils are bound to the
 * 6th-order family through QuadGrav/include/derivs.h
 * (QUADGRAV_USE_6TH_ORDER_DERIVS), i.e. QuadGrav/src/derivs.cpp.
 * Domain-boundary blocks (bflag != 0) get the reference's one-sided
 * closures (they live in derivs.cpp) and its outgoing-radiation condition
 * bssn_bcs, extracted verbatim from BSSN_GR/src/rhs.cpp at build time
 * (oracle/Makefile.ref), called with the reference's falloff and asymptotic
 * values per variable (rhs.cpp:265-324).
 */
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "derivs.h"

#include "bssn_bcs.inc"

namespace {
enum { V_ALPHA = 0, V_CHI, V_K, V_GT0, V_GT1, V_GT2, V_BETA0, V_BETA1, V_BETA2,
       V_B0, V_B1, V_B2, V_SYMGT0, V_SYMGT1, V_SYMGT2, V_SYMGT3, V_SYMGT4,
       V_SYMGT5, V_SYMAT0, V_SYMAT1, V_SYMAT2, V_SYMAT3, V_SYMAT4, V_SYMAT5 };
}

/* prm layout: lambda[4], lambda_f[2], eta_const, eta_r0, eta_damping_exp, ko_sigma */
extern "C" int ref_bssnrhs(double **unzipVarsRHS, const double **uZipVars,
                           unsigned int offset, const double *pmin,
                           const double *pmax, const unsigned int *sz,
                           unsigned int bflag, const double *prm)
{
    const unsigned int lambda[4] = {(unsigned)prm[0], (unsigned)prm[1],
                                    (unsigned)prm[2], (unsigned)prm[3]};
    const double lambda_f[2] = {prm[4], prm[5]};
    const double ETA_CONST = prm[6], ETA_R0 = prm[7], ETA_DAMPING_EXP = prm[8];
    const double KO_DISS_SIGMA = prm[9];

#define IN_(name, v) const double *name = &uZipVars[v][offset]
#define OUT_(name, v) double *name = &unzipVarsRHS[v][offset]
    IN_(alpha, V_ALPHA); IN_(chi, V_CHI); IN_(K, V_K);
    IN_(gt0, V_SYMGT0); IN_(gt1, V_SYMGT1); IN_(gt2, V_SYMGT2);
    IN_(gt3, V_SYMGT3); IN_(gt4, V_SYMGT4); IN_(gt5, V_SYMGT5);
    IN_(beta0, V_BETA0); IN_(beta1, V_BETA1); IN_(beta2, V_BETA2);
    IN_(At0, V_SYMAT0); IN_(At1, V_SYMAT1); IN_(At2, V_SYMAT2);
    IN_(At3, V_SYMAT3); IN_(At4, V_SYMAT4); IN_(At5, V_SYMAT5);
    IN_(Gt0, V_GT0); IN_(Gt1, V_GT1); IN_(Gt2, V_GT2);
    IN_(B0, V_B0); IN_(B1, V_B1); IN_(B2, V_B2);
    OUT_(a_rhs, V_ALPHA); OUT_(chi_rhs, V_CHI); OUT_(K_rhs, V_K);
    OUT_(gt_rhs00, V_SYMGT0); OUT_(gt_rhs01, V_SYMGT1); OUT_(gt_rhs02, V_SYMGT2);
    OUT_(gt_rhs11, V_SYMGT3); OUT_(gt_rhs12, V_SYMGT4); OUT_(gt_rhs22, V_SYMGT5);
    OUT_(b_rhs0, V_BETA0); OUT_(b_rhs1, V_BETA1); OUT_(b_rhs2, V_BETA2);
    OUT_(At_rhs00, V_SYMAT0); OUT_(At_rhs01, V_SYMAT1); OUT_(At_rhs02, V_SYMAT2);
    OUT_(At_rhs11, V_SYMAT3); OUT_(At_rhs12, V_SYMAT4); OUT_(At_rhs22, V_SYMAT5);
    OUT_(Gt_rhs0, V_GT0); OUT_(Gt_rhs1, V_GT1); OUT_(Gt_rhs2, V_GT2);
    OUT_(B_rhs0, V_B0); OUT_(B_rhs1, V_B1); OUT_(B_rhs2, V_B2);
#undef IN_
#undef OUT_

    const unsigned int nx = sz[0], ny = sz[1], nz = sz[2];
    const double hx = (pmax[0] - pmin[0]) / (nx - 1);
    const double hy = (pmax[1] - pmin[1]) / (ny - 1);
    const double hz = (pmax[2] - pmin[2]) / (nz - 1);
    const unsigned int n = nx * ny * nz;

#include "bssnrhs_memalloc.h"
#include "bssnrhs_memalloc_adv.h"
#include "bssnrhs_derivs.h"
#include "bssnrhs_derivs_adv.h"

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
#include "bssneqs_eta_const_standard_gauge.cpp"
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
            {chi_rhs, chi, grad_0_chi, grad_1_chi, grad_2_chi, 1.0, 1.0},
            {K_rhs, K, grad_0_K, grad_1_K, grad_2_K, 1.0, 0.0},
            {b_rhs0, beta0, grad_0_beta0, grad_1_beta0, grad_2_beta0, 1.0, 0.0},
            {b_rhs1, beta1, grad_0_beta1, grad_1_beta1, grad_2_beta1, 1.0, 0.0},
            {b_rhs2, beta2, grad_0_beta2, grad_1_beta2, grad_2_beta2, 1.0, 0.0},
            {Gt_rhs0, Gt0, grad_0_Gt0, grad_1_Gt0, grad_2_Gt0, 2.0, 0.0},
            {Gt_rhs1, Gt1, grad_0_Gt1, grad_1_Gt1, grad_2_Gt1, 2.0, 0.0},
            {Gt_rhs2, Gt2, grad_0_Gt2, grad_1_Gt2, grad_2_Gt2, 2.0, 0.0},
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
            bssn_bcs(c.rhs, c.f, c.dx, c.dy, c.dz, pmin, pmax, c.falloff, c.asymptotic, sz, bflag);
    }

#include "bssnrhs_ko_derivs.h"

    const double sigma = KO_DISS_SIGMA;
    double *const outs[24] = {a_rhs, chi_rhs, K_rhs, Gt_rhs0, Gt_rhs1, Gt_rhs2,
                              b_rhs0, b_rhs1, b_rhs2, B_rhs0, B_rhs1, B_rhs2,
                              gt_rhs00, gt_rhs01, gt_rhs02, gt_rhs11, gt_rhs12, gt_rhs22,
                              At_rhs00, At_rhs01, At_rhs02, At_rhs11, At_rhs12, At_rhs22};
    const double *const ko[24][3] = {
        {grad_0_alpha, grad_1_alpha, grad_2_alpha}, {grad_0_chi, grad_1_chi, grad_2_chi},
        {grad_0_K, grad_1_K, grad_2_K}, {grad_0_Gt0, grad_1_Gt0, grad_2_Gt0},
        {grad_0_Gt1, grad_1_Gt1, grad_2_Gt1}, {grad_0_Gt2, grad_1_Gt2, grad_2_Gt2},
        {grad_0_beta0, grad_1_beta0, grad_2_beta0}, {grad_0_beta1, grad_1_beta1, grad_2_beta1},
        {grad_0_beta2, grad_1_beta2, grad_2_beta2}, {grad_0_B0, grad_1_B0, grad_2_B0},
        {grad_0_B1, grad_1_B1, grad_2_B1}, {grad_0_B2, grad_1_B2, grad_2_B2},
        {grad_0_gt0, grad_1_gt0, grad_2_gt0}, {grad_0_gt1, grad_1_gt1, grad_2_gt1},
        {grad_0_gt2, grad_1_gt2, grad_2_gt2}, {grad_0_gt3, grad_1_gt3, grad_2_gt3},
        {grad_0_gt4, grad_1_gt4, grad_2_gt4}, {grad_0_gt5, grad_1_gt5, grad_2_gt5},
        {grad_0_At0, grad_1_At0, grad_2_At0}, {grad_0_At1, grad_1_At1, grad_2_At1},
        {grad_0_At2, grad_1_At2, grad_2_At2}, {grad_0_At3, grad_1_At3, grad_2_At3},
        {grad_0_At4, grad_1_At4, grad_2_At4}, {grad_0_At5, grad_1_At5, grad_2_At5}};
    for (unsigned int k = 3; k < nz - 3; k++)
        for (unsigned int j = 3; j < ny - 3; j++)
            for (unsigned int i = 3; i < nx - 3; i++) {
                const unsigned int pp = i + nx * (j + ny * k);
                for (int v = 0; v < 24; v++)
                    outs[v][pp] += sigma * (ko[v][0][pp] + ko[v][1][pp] + ko[v][2][pp]);
            }

#include "bssnrhs_dealloc.h"
#include "bssnrhs_dealloc_adv.h"
    return 0;
}

/* bssnRHS over a block list with OpenMP over blocks, the loop the
 * reference's test bed times (BSSN_GR/src/rhsTestBed.cpp:181-215); each
 * call allocates and frees its 210 scratch arrays as bssnrhs does. */
extern "C" int ref_bssnrhs_blocks(double **rhs, const double **uz, long nblk,
                                  const unsigned long *offsets, const unsigned *sizes,
                                  const unsigned *bflags, const double *pmins, const double *pmaxs,
                                  const double *prm, int nthreads)
{
    int err = 0;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads > 0 ? nthreads : 1) reduction(| : err)
    for (long b = 0; b < nblk; b++)
        err |= ref_bssnrhs(rhs, uz, (unsigned)offsets[b], pmins + 3 * b, pmaxs + 3 * b, sizes + 3 * b,
                           bflags[b], prm);
    return err;
}

/* The reference's per-node RK update closure (BSSN_GR/src/bssn_constraints.cpp). */
namespace bssn { double CHI_FLOOR = 1e-4; }
void enforce_bssn_constraints(double **uiVar, const unsigned int offset);
extern "C" void ref_enforce_bssn_constraints(double **uiVar, unsigned int node, double chi_floor)
{
    bssn::CHI_FLOOR = chi_floor;
    enforce_bssn_constraints(uiVar, node);
}

/* The reference stencils themselves (with their boundary closures when
 * bflag is set), exported for per-stencil pins. */
#define REF_STENCIL(name, fn) \
    extern "C" void name(double *D, const double *u, double h, const unsigned *sz, unsigned bflag) \
    { fn(D, u, h, sz, bflag); }
REF_STENCIL(ref_deriv64_x, deriv64_x)
REF_STENCIL(ref_deriv64_y, deriv64_y)
REF_STENCIL(ref_deriv64_z, deriv64_z)
REF_STENCIL(ref_deriv64_xx, deriv64_xx)
REF_STENCIL(ref_deriv64_yy, deriv64_yy)
REF_STENCIL(ref_deriv64_zz, deriv64_zz)
REF_STENCIL(ref_ko_deriv42_x, ko_deriv42_x)
REF_STENCIL(ref_ko_deriv42_y, ko_deriv42_y)
REF_STENCIL(ref_ko_deriv42_z, ko_deriv42_z)
