/* dgesv_ for the oracle build of the reference's octree mesh.  The
 * reference's RefElement (FEM/src/refel.cpp:165-172, through
 * FEM/include/lapac.h:22) solves its Vandermonde systems with LAPACK's
 * dgesv_; no LAPACK is installed here, so this file gives the same entry
 * point: Gaussian elimination with partial pivoting (the row of largest
 * magnitude, first on ties), on column-major A (n x n, leading dimension lda)
 * and B (n x nrhs, leading dimension ldb), solution in B, A overwritten by
 * its LU factors, ipiv 1-based as LAPACK returns it, info = k > 0 when the
 * k-th pivot is exactly zero.  Its rounding differs from LAPACK's blocked
 * factorisation by a few units in the last place.  Test infrastructure only. */
#include <math.h>

void dgesv_(int *n_, int *nrhs_, double *a, int *lda_, int *ipiv, double *b, int *ldb_, int *info)
{
    const int n = *n_, nrhs = *nrhs_, lda = *lda_, ldb = *ldb_;
    *info = 0;
#define A(i, j) a[(long)(j) * lda + (i)]
#define B(i, j) b[(long)(j) * ldb + (i)]
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = fabs(A(k, k));
        for (int i = k + 1; i < n; i++)
            if (fabs(A(i, k)) > best) { best = fabs(A(i, k)); p = i; }
        ipiv[k] = p + 1;
        if (A(p, k) == 0.0) { if (*info == 0) *info = k + 1; continue; }
        if (p != k) {
            for (int j = 0; j < n; j++) { double t = A(k, j); A(k, j) = A(p, j); A(p, j) = t; }
            for (int j = 0; j < nrhs; j++) { double t = B(k, j); B(k, j) = B(p, j); B(p, j) = t; }
        }
        for (int i = k + 1; i < n; i++) {
            const double l = A(i, k) / A(k, k);
            A(i, k) = l;
            for (int j = k + 1; j < n; j++) A(i, j) -= l * A(k, j);
            for (int j = 0; j < nrhs; j++) B(i, j) -= l * B(k, j);
        }
    }
    if (*info) return;
    for (int j = 0; j < nrhs; j++)
        for (int i = n - 1; i >= 0; i--) {
            double s = B(i, j);
            for (int m = i + 1; m < n; m++) s -= A(i, m) * B(m, j);
            B(i, j) = s / A(i, i);
        }
#undef A
#undef B
}

/* dsyev_ (jobz "V", upper or lower triangle) for the same build: the
 * reference's Gauss-Jacobi quadrature (FEM/src/basis.cpp:147, through
 * FEM/include/lapac.h:114-131) takes the eigenvalues of a symmetric
 * tridiagonal matrix and the squares of its eigenvectors' first components.
 * Cyclic Jacobi rotations until the off-diagonal part vanishes; eigenvalues
 * ascending in w, eigenvectors in the columns of a (column-major), as LAPACK
 * returns them (an eigenvector's sign is not fixed, and the caller squares
 * it).  A workspace query (lwork = -1) returns 1. */
void dsyev_(char *jobz, char *uplo, int *n_, double *a, int *lda_, double *w, double *work, int *lwork, int *info)
{
    const int n = *n_, lda = *lda_;
    (void)jobz;
    *info = 0;
    if (*lwork == -1) { work[0] = 1.0; return; }
#define M(i, j) a[(long)(j) * lda + (i)]
    double s[64 * 64], v[64 * 64];
    if (n > 64) { *info = -3; return; }
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            const int up = (uplo[0] == 'U' || uplo[0] == 'u');
            const double x = (up ? (i <= j) : (i >= j)) ? M(i, j) : M(j, i);
            s[j * n + i] = x;
            v[j * n + i] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += s[q * n + p] * s[q * n + p];
        if (off == 0.0) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = s[q * n + p];
                if (apq == 0.0) continue;
                const double app = s[p * n + p], aqq = s[q * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; k++) {
                    const double skp = s[p * n + k], skq = s[q * n + k];
                    s[p * n + k] = c * skp - sn * skq;
                    s[q * n + k] = sn * skp + c * skq;
                }
                for (int k = 0; k < n; k++) {
                    const double spk = s[k * n + p], sqk = s[k * n + q];
                    s[k * n + p] = c * spk - sn * sqk;
                    s[k * n + q] = sn * spk + c * sqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vkp = v[p * n + k], vkq = v[q * n + k];
                    v[p * n + k] = c * vkp - sn * vkq;
                    v[q * n + k] = sn * vkp + c * vkq;
                }
            }
    }
    int order[64];
    for (int i = 0; i < n; i++) order[i] = i;
    for (int i = 1; i < n; i++)
        for (int j = i; j > 0 && s[order[j] * n + order[j]] < s[order[j - 1] * n + order[j - 1]]; j--) {
            const int t = order[j]; order[j] = order[j - 1]; order[j - 1] = t;
        }
    for (int j = 0; j < n; j++) {
        w[j] = s[order[j] * n + order[j]];
        for (int i = 0; i < n; i++) M(i, j) = v[order[j] * n + i];
    }
#undef M
}
