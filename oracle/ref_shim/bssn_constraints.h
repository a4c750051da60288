/* Build shim for compiling BSSN_GR/src/bssn_constraints.cpp standalone.
 * The reference header pulls in the mesh and MPI; the function only needs
 * the evolved-variable order (BSSN_GR/include/grDef.h:31) and CHI_FLOOR. */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <iostream>
namespace bssn {
enum VAR { U_ALPHA = 0, U_CHI, U_K, U_GT0, U_GT1, U_GT2, U_BETA0, U_BETA1,
           U_BETA2, U_B0, U_B1, U_B2, U_SYMGT0, U_SYMGT1, U_SYMGT2, U_SYMGT3,
           U_SYMGT4, U_SYMGT5, U_SYMAT0, U_SYMAT1, U_SYMAT2, U_SYMAT3,
           U_SYMAT4, U_SYMAT5 };
extern double CHI_FLOOR;
}
void enforce_bssn_constraints(double **uiVar, const unsigned int offset);
