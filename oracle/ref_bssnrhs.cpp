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

#define REF_BSSNRHS ref_bssnrhs
#include "ref_bssnrhs_body.inc"
#undef REF_BSSNRHS

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
