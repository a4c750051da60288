/*
 * Test infrastructure only: the bssnrhs harness with the BSSN_GR solver's
 * own stencil binding (BSSN_GR/include/rhs.h:23-37): deriv42_* first and
 * second derivatives, the upwinded deriv42adv_* as advective derivatives and
 * ko_deriv42_*.  Those functions are taken from QuadGrav/src/derivs.cpp,
 * whose 4th-order part (lines 1-2140) is the text of BSSN_GR/src/derivs.cpp
 * (the two differ in one unused variable and a comment), bound through
 * QuadGrav/include/derivs.h's QUADGRAV_USE_4TH_ORDER_DERIVS macros, which
 * name the same functions as BSSN_GR/include/rhs.h.  bssn_bcs is the one
 * extracted from BSSN_GR/src/rhs.cpp (oracle/Makefile.ref), renamed here so
 * that it does not clash with the 6th-order harness's copy.
 */
#include <cmath>
#include <cstdlib>
#include <cstring>

#undef QUADGRAV_USE_6TH_ORDER_DERIVS
#define QUADGRAV_USE_4TH_ORDER_DERIVS
#include "derivs.h"

#define bssn_bcs ref42_bssn_bcs
#include "bssn_bcs.inc"

namespace {
enum { V_ALPHA = 0, V_CHI, V_K, V_GT0, V_GT1, V_GT2, V_BETA0, V_BETA1, V_BETA2,
       V_B0, V_B1, V_B2, V_SYMGT0, V_SYMGT1, V_SYMGT2, V_SYMGT3, V_SYMGT4,
       V_SYMGT5, V_SYMAT0, V_SYMAT1, V_SYMAT2, V_SYMAT3, V_SYMAT4, V_SYMAT5 };
}

#define REF_BSSNRHS ref_bssnrhs42
#include "ref_bssnrhs_body.inc"
#undef REF_BSSNRHS

/* the 4th-order stencils themselves, for per-stencil pins */
extern "C" void ref_deriv42adv(int dir, double *D, const double *u, double h, const unsigned *sz,
                               const double *beta, unsigned bflag)
{
    if (dir == 0) deriv42adv_x(D, u, h, sz, beta, bflag);
    else if (dir == 1) deriv42adv_y(D, u, h, sz, beta, bflag);
    else deriv42adv_z(D, u, h, sz, beta, bflag);
}
