"""The C++ drop-in header on the GPU: a program built against a stand-in for
ot::Block calls dgb_bssn::bssnRHS (BSSN_GR/src/rhs.cpp:9-76) and
dgb_bssn::bssnrhs (rhs.cpp:86-392) the way a solver would, on host arrays,
for interior and domain-boundary blocks in both stencil bindings; the results
must equal, bit for bit, those of a plan built through the C ABI from the
same descriptors."""
import os
import subprocess
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = textwrap.dedent(r"""
    #include <cstdio>
    #include <cstring>
    #include <vector>
    #include "dendro_gb300_bssn.hpp"
    // stand-ins with the reference's accessor names (include/block.h, TreeNode.h);
    // one octant of order 6 per block, so the block spacing is the octant width / 6
    struct Point { double v[3]; double x() const {return v[0];} double y() const {return v[1];}
                   double z() const {return v[2];} };
    struct Node { unsigned mn[3], mx[3];
      unsigned minX() const {return mn[0];} unsigned minY() const {return mn[1];}
      unsigned minZ() const {return mn[2];} unsigned maxX() const {return mx[0];}
      unsigned maxY() const {return mx[1];} unsigned maxZ() const {return mx[2];} };
    struct Block {
      unsigned long off; unsigned flag; Node node; unsigned maxDepth;
      unsigned long getOffset() const {return off;}
      unsigned getAllocationSzX() const {return 13;} unsigned getAllocationSzY() const {return 13;}
      unsigned getAllocationSzZ() const {return 13;} unsigned getBlkNodeFlag() const {return flag;}
      const Node& getBlockNode() const {return node;}
      double h(double a, double b) const { return ((b - a) / (double)(1u << maxDepth)) * ((node.mx[0] - node.mn[0]) / 6.0); }
      double computeDx(const Point& a, const Point& b) const { return h(a.x(), b.x()); }
      double computeDy(const Point& a, const Point& b) const { return h(a.y(), b.y()); }
      double computeDz(const Point& a, const Point& b) const { return h(a.z(), b.z()); }
    };
    int main() {
      if (dgb_init(0) != DGB_OK) return 3;
      const unsigned maxDepth = 8;
      Point pmin{{-32, -32, -32}}, pmax{{32, 32, 32}};
      auto g2d = [](int, unsigned xg) { return (64.0 / 256.0) * (xg - 0.0) + (-32.0); };
      const unsigned n3 = 13 * 13 * 13;
      // two interior octants side by side, one on the low-x face, one on the high-z face
      std::vector<Block> bl = {{0 * n3, 0, Node{{64, 96, 128}, {72, 104, 136}}, maxDepth},
                               {1 * n3, 0, Node{{72, 96, 128}, {80, 104, 136}}, maxDepth},
                               {2 * n3, 1, Node{{0, 96, 128}, {8, 104, 136}}, maxDepth},
                               {3 * n3, 32, Node{{64, 96, 248}, {72, 104, 256}}, maxDepth}};
      const size_t n = 4 * n3;
      std::vector<dgb_block_desc> d;
      for (const Block& b : bl) d.push_back(dgb_bssn::describe_block(b, pmin, pmax, g2d));
      std::vector<std::vector<double>> U(24, std::vector<double>(n));
      double* u[24]; const double* uc[24];
      for (int v = 0; v < 24; v++) { u[v] = U[v].data(); uc[v] = u[v]; }
      if (dgb_synth_fill_host(d.data(), d.size(), u, 20261204, 1e-6, 1) != DGB_OK) return 4;
      unsigned lam[4] = {1, 1, 1, 1}; double lf[2] = {1, 0};
      int bad = 0;
      for (int order : {6, 4}) {
        const dgb_bssn_params p = dgb_bssn::params(lam, lf, 2.0, 30.0, 1.0, 0.1, 1e-4, order);
        std::vector<std::vector<double>> R1(24, std::vector<double>(n, 0.0)), R2 = R1, R3 = R1;
        double *r1[24], *r2[24], *r3[24];
        for (int v = 0; v < 24; v++) { r1[v] = R1[v].data(); r2[v] = R2[v].data(); r3[v] = R3[v].data(); }
        dgb_bssn::PlanCache cache;
        for (int call = 0; call < 2; call++)  // the second call reuses the cached plan
          if (dgb_bssn::bssnRHS(r1, uc, bl.data(), (unsigned)bl.size(), pmin, pmax, g2d, p, cache) != DGB_OK) return 5;
        dgb_plan* plan = nullptr;
        if (dgb_plan_create(d.data(), d.size(), &p, &plan) != DGB_OK) return 6;
        if (dgb_bssn_rhs_host(plan, r2, uc, DGB_PREC_FP64) != DGB_OK) return 7;
        dgb_plan_destroy(plan);
        for (const dgb_block_desc& x : d) {
          const unsigned off = (unsigned)x.offset, bf = x.bflag;
          const unsigned sz[3] = {x.sz[0], x.sz[1], x.sz[2]};
          if (dgb_bssn::bssnrhs(r3, uc, off, x.ptmin, x.ptmax, sz, bf, p) != DGB_OK) return 8;
        }
        for (int v = 0; v < 24; v++) {
          bad += std::memcmp(R1[v].data(), R2[v].data(), n * 8) != 0;
          bad += std::memcmp(R3[v].data(), R2[v].data(), n * 8) != 0;
        }
        double amax = 0;
        for (int v = 0; v < 24; v++) for (size_t i = 0; i < n; i++) amax = R2[v][i] > amax ? R2[v][i] : (-R2[v][i] > amax ? -R2[v][i] : amax);
        std::printf("order %d: max |rhs| %.6e, fields differing %d\n", order, amax, bad);
        bad += !(amax > 0);
      }
      return bad ? 1 : 0;
    }
""")


@pytest.mark.gpu
def test_shim_bssnRHS_on_gpu_equals_plan(dgb, gpu, tmp_path):
    src = tmp_path / "shim_gpu.cpp"
    src.write_text(SRC)
    exe = tmp_path / "shim_gpu"
    libdir = os.path.dirname(dgb.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT}/include", str(src), "-o", str(exe),
                    f"-L{libdir}", "-ldendro_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
