/*
 * Test infrastructure only: a C-callable harness around the reference's OWN
 * constraint diagnostics, compiled from the reference sources where they lie
 * (see oracle/Makefile.ref).  Nothing here ships.
 *
 * It has the shape of physical_constraints() (BSSN_GR/src/physcon.cpp:12-96):
 * the field pointers at `offset`, h = (pmax - pmin)/(n - 1), the generated
 * derivative driver BSSN_GR/scripts/constraint_derivs.h with the 4th-order
 * stencils that BSSN_GR/include/physcon.h binds (deriv42_*, identical in
 * QuadGrav/src/derivs.cpp, which the same library already compiles), and the
 * generated point algebra BSSN_GR/src/physconeqs.cpp inside the interior
 * loop.  Output order: ham, mom0, mom1, mom2, psi4_real, psi4_img.
 */
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "derivs.h"

#undef deriv_x
#undef deriv_y
#undef deriv_z
#undef deriv_xx
#undef deriv_yy
#undef deriv_zz
#define deriv_x deriv42_x
#define deriv_y deriv42_y
#define deriv_z deriv42_z
#define deriv_xx deriv42_xx
#define deriv_yy deriv42_yy
#define deriv_zz deriv42_zz

using std::pow;
using std::sqrt;
using std::fabs;

namespace {
enum { V_ALPHA = 0, V_CHI, V_K, V_GT0, V_GT1, V_GT2, V_BETA0, V_BETA1, V_BETA2,
       V_B0, V_B1, V_B2, V_SYMGT0, V_SYMGT1, V_SYMGT2, V_SYMGT3, V_SYMGT4,
       V_SYMGT5, V_SYMAT0, V_SYMAT1, V_SYMAT2, V_SYMAT3, V_SYMAT4, V_SYMAT5 };
}

extern "C" int ref_physical_constraints(double **cons, const double **uZipVars,
                                        unsigned int offset, const double *pmin,
                                        const double *pmax, const unsigned int *sz,
                                        unsigned int bflag)
{
#define IN_(name, v) const double *name = &uZipVars[v][offset]
    IN_(chi, V_CHI); IN_(K, V_K);
    IN_(gt0, V_SYMGT0); IN_(gt1, V_SYMGT1); IN_(gt2, V_SYMGT2);
    IN_(gt3, V_SYMGT3); IN_(gt4, V_SYMGT4); IN_(gt5, V_SYMGT5);
    IN_(At0, V_SYMAT0); IN_(At1, V_SYMAT1); IN_(At2, V_SYMAT2);
    IN_(At3, V_SYMAT3); IN_(At4, V_SYMAT4); IN_(At5, V_SYMAT5);
    IN_(Gt0, V_GT0); IN_(Gt1, V_GT1); IN_(Gt2, V_GT2);
#undef IN_
    double *ham = &cons[0][offset];
    double *mom0 = &cons[1][offset];
    double *mom1 = &cons[2][offset];
    double *mom2 = &cons[3][offset];
    double *psi4_real = &cons[4][offset];
    double *psi4_img = &cons[5][offset];

    const unsigned int nx = sz[0], ny = sz[1], nz = sz[2];
    const double hx = (pmax[0] - pmin[0]) / (nx - 1);
    const double hy = (pmax[1] - pmin[1]) / (ny - 1);
    const double hz = (pmax[2] - pmin[2]) / (nz - 1);
    const unsigned int n = nx * ny * nz;

#include "constraint_memalloc.h"
#include "constraint_derivs.h"

    for (unsigned int k = 3; k < nz - 3; k++) {
        const double z = pmin[2] + k * hz;
        for (unsigned int j = 3; j < ny - 3; j++) {
            const double y = pmin[1] + j * hy;
            for (unsigned int i = 3; i < nx - 3; i++) {
                const double x = pmin[0] + i * hx;
                const unsigned int pp = i + nx * (j + ny * k);
#include "physconeqs.cpp"
            }
        }
    }

#include "constraint_dealloc.h"
    return 0;
}

#define REF_STENCIL42(name, fn) \
    extern "C" void name(double *D, const double *u, double h, const unsigned *sz, unsigned bflag) \
    { fn(D, u, h, sz, bflag); }
REF_STENCIL42(ref_deriv42_x, deriv42_x)
REF_STENCIL42(ref_deriv42_y, deriv42_y)
REF_STENCIL42(ref_deriv42_z, deriv42_z)
REF_STENCIL42(ref_deriv42_xx, deriv42_xx)
REF_STENCIL42(ref_deriv42_yy, deriv42_yy)
REF_STENCIL42(ref_deriv42_zz, deriv42_zz)
