// Host check of the generated BSSN point algebra (csrc/bssn_algebra.cuh and,
// for the 4th-order binding, csrc/bssn_algebra42.cuh, compiled as plain C++)
// against the oracle's orc_bssn_point on random fields and derivative
// values; exits 1 when a field differs by more than 1e-12 of its largest
// value.  Built and run by tests/test_algebra_host.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#define __device__
#define __forceinline__ inline
#include "bssn_algebra.cuh"
#include "bssn_algebra42.cuh"
extern "C" {
typedef struct {
    double a, chi, K, Gt[3], b[3], B[3], gt[3][3], At[3][3];
    double da[3], dchi[3], dK[3], dGt[3][3], db[3][3], dB[3][3];
    double dgt[3][3][3], dAt[3][3][3];
    double ddgt[3][3][3][3], ddchi[3][3], dda[3][3], ddb[3][3][3];
    int upwind;
    double adv[24];
} orc_point;
void orc_bssn_point(const orc_point *P, const double *prm, double eta, double *out);
}
static const int SY[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
struct IO {
    double u_[24];
    double s[DGB_B42_NUM_SLOTS];
    double o[24];
    double u(int v) const { return u_[v]; }
    double d(int k) const { return s[k]; }
    void out(int v, double x) { o[v] = x; }
};
struct PRM {
    double l1, l2, l3, l4, lf0, lf1;
};
int main()
{
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(-1, 1);
    double mx = 0;
    for (int upwind = 0; upwind < 2; upwind++) {
        double worst[24] = {0}, scale[24] = {0};
        for (int t = 0; t < 2000; t++) {
            IO io;
            orc_point P;
            for (int v = 0; v < 24; v++) io.u_[v] = 0.3 * U(rng);
            io.u_[0] = 0.6 + 0.2 * U(rng);
            io.u_[1] = 0.5 + 0.2 * U(rng);
            io.u_[12] += 1.0;
            io.u_[15] += 1.0;
            io.u_[17] += 1.0;
            for (int k = 0; k < DGB_B42_NUM_SLOTS; k++) io.s[k] = U(rng);
            P.a = io.u_[0];
            P.chi = io.u_[1];
            P.K = io.u_[2];
            for (int c = 0; c < 3; c++) {
                P.Gt[c] = io.u_[3 + c];
                P.b[c] = io.u_[6 + c];
                P.B[c] = io.u_[9 + c];
            }
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    P.gt[i][j] = io.u_[12 + SY[i][j]];
                    P.At[i][j] = io.u_[18 + SY[i][j]];
                }
            auto G = [&](int v, int d) { return io.s[3 * v + d]; };
            const int d2v[11] = {0, 1, 6, 7, 8, 12, 13, 14, 15, 16, 17};
            auto D2 = [&](int v, int l, int m) {
                int q = -1;
                for (int r = 0; r < 11; r++)
                    if (d2v[r] == v) q = r;
                return io.s[DGB_NUM_GRAD + 6 * q + SY[l][m]];
            };
            for (int d = 0; d < 3; d++) {
                P.da[d] = G(0, d);
                P.dchi[d] = G(1, d);
                P.dK[d] = G(2, d);
                for (int c = 0; c < 3; c++) {
                    P.dGt[c][d] = G(3 + c, d);
                    P.db[c][d] = G(6 + c, d);
                    P.dB[c][d] = G(9 + c, d);
                }
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        P.dgt[i][j][d] = G(12 + SY[i][j], d);
                        P.dAt[i][j][d] = G(18 + SY[i][j], d);
                    }
            }
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++) {
                    P.dda[l][m] = D2(0, l, m);
                    P.ddchi[l][m] = D2(1, l, m);
                    for (int c = 0; c < 3; c++) P.ddb[c][l][m] = D2(6 + c, l, m);
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++) P.ddgt[i][j][l][m] = D2(12 + SY[i][j], l, m);
                }
            P.upwind = upwind;
            for (int v = 0; v < 24; v++) P.adv[v] = io.s[DGB_B42_ADV0 + v];
            const double prm[10] = {1, 1, 1, 1, 1, 0.3, 2.0, 30.0, 1.0, 0.4};
            const PRM pr{1, 1, 1, 1, 1, 0.3};
            double want[24];
            orc_bssn_point(&P, prm, 1.7, want);
            if (upwind)
                dgb_bssn_algebra_upwind(io, pr, 1.7);
            else
                dgb_bssn_algebra(io, pr, 1.7);
            for (int v = 0; v < 24; v++) {
                const double e = std::fabs(io.o[v] - want[v]);
                if (e > worst[v]) worst[v] = e;
                if (std::fabs(want[v]) > scale[v]) scale[v] = std::fabs(want[v]);
            }
        }
        printf("%s:", upwind ? "upwind" : "centred");
        for (int v = 0; v < 24; v++) {
            const double r = worst[v] / scale[v];
            printf(" %d:%.1e", v, r);
            if (r > mx) mx = r;
        }
        printf("\n");
    }
    printf("max %.2e\n", mx);
    return mx < 1e-12 ? 0 : 1;
}
