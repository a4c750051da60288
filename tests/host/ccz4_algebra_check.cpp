// Host check of the generated CCZ4 point algebra (csrc/ccz4_algebra.cuh,
// compiled as plain C++) against the oracle's orc_ccz4_point on random
// fields and derivative values; exits 1 when a field differs by more than
// 1e-12 of its largest value.  Built and run by tests/test_algebra_host.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#define __device__
#define __forceinline__ inline
#include "ccz4_algebra.cuh"
extern "C" {
typedef struct {
    double a, psi, K, th, Gh[3], b[3], B[3], gt[3][3], At[3][3];
    double da[3], dpsi[3], dK[3], dth[3], dGh[3][3], db[3][3], dgt[3][3][3];
    double ada[3], adpsi[3], adK[3], adth[3], adGh[3][3], adb[3][3], adB[3][3];
    double adgt[3][3][3], adAt[3][3][3];
    double dda[3][3], ddpsi[3][3], ddb[3][3][3], ddgt[3][3][3][3];
} orc_cpt4;
void orc_ccz4_point(const orc_cpt4 *P, const double *prm, double eta, double *out);
}
static const int SY[3][3] = {{0,1,2},{1,3,4},{2,4,5}};
struct IO { double u_[25]; double s[241]; double o[25];
  double u(int v) const { return u_[v]; } double d(int k) const { return s[k]; } void out(int v, double x) { o[v] = x; } };
struct PRM { double l1,l2,l3,l4,lf0,lf1,k1,k2,p; };
int main() {
  std::mt19937_64 rng(5); std::uniform_real_distribution<double> U(-1, 1);
  double worst[25] = {0}, scale[25] = {0};
  for (int t = 0; t < 2000; t++) {
    IO io; orc_cpt4 P;
    for (int v = 0; v < 25; v++) io.u_[v] = 0.3 * U(rng);
    io.u_[0] = 0.6 + 0.2*U(rng); io.u_[1] = 0.5 + 0.2*U(rng);
    io.u_[12] += 1.0; io.u_[15] += 1.0; io.u_[17] += 1.0;
    for (int k = 0; k < 241; k++) io.s[k] = U(rng);
    P.a = io.u_[0]; P.psi = io.u_[1]; P.K = io.u_[2]; P.th = io.u_[24];
    for (int c = 0; c < 3; c++) { P.Gh[c] = io.u_[3+c]; P.b[c] = io.u_[6+c]; P.B[c] = io.u_[9+c]; }
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) { P.gt[i][j] = io.u_[12+SY[i][j]]; P.At[i][j] = io.u_[18+SY[i][j]]; }
    auto G = [&](int v, int d) { return io.s[3*v+d]; };
    auto A = [&](int v, int d) { return io.s[75+3*v+d]; };
    const int d2v[11] = {0,1,6,7,8,12,13,14,15,16,17};
    auto D2 = [&](int v, int l, int m) { int q=-1; for (int r=0;r<11;r++) if (d2v[r]==v) q=r; return io.s[150+6*q+SY[l][m]]; };
    for (int d = 0; d < 3; d++) {
      P.da[d]=G(0,d); P.dpsi[d]=G(1,d); P.dK[d]=G(2,d); P.dth[d]=G(24,d);
      P.ada[d]=A(0,d); P.adpsi[d]=A(1,d); P.adK[d]=A(2,d); P.adth[d]=A(24,d);
      for (int c = 0; c < 3; c++) { P.dGh[c][d]=G(3+c,d); P.db[c][d]=G(6+c,d); P.adGh[c][d]=A(3+c,d); P.adb[c][d]=A(6+c,d); P.adB[c][d]=A(9+c,d); }
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) { P.dgt[i][j][d]=G(12+SY[i][j],d); P.adgt[i][j][d]=A(12+SY[i][j],d); P.adAt[i][j][d]=A(18+SY[i][j],d); }
    }
    for (int l = 0; l < 3; l++) for (int m = 0; m < 3; m++) {
      P.dda[l][m]=D2(0,l,m); P.ddpsi[l][m]=D2(1,l,m);
      for (int c = 0; c < 3; c++) P.ddb[c][l][m]=D2(6+c,l,m);
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) P.ddgt[i][j][l][m]=D2(12+SY[i][j],l,m);
    }
    double prm[13] = {1,1,1,1, 1,0.3, 0.1,0.05, -1, 2,30,1, 0.4};
    PRM pr{1,1,1,1,1,0.3,0.1,0.05,-1};
    double want[25];
    orc_ccz4_point(&P, prm, 1.7, want);
    dgb_ccz4_algebra(io, pr, 1.7);
    for (int v = 0; v < 25; v++) { double e = std::fabs(io.o[v]-want[v]); if (e > worst[v]) worst[v]=e; if (std::fabs(want[v])>scale[v]) scale[v]=std::fabs(want[v]); }
  }
  double mx = 0; for (int v = 0; v < 25; v++) { double r = worst[v]/scale[v]; printf("%d:%.1e ", v, r); if (r>mx) mx=r; } printf("\nmax %.2e\n", mx);
  return mx < 1e-12 ? 0 : 1;
}
