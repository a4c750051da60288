"""The C++ drop-in header (include/dendro_gb300_bssn.hpp) compiles against a
stand-in for ot::Block with the reference's accessor names and derives the
block descriptor exactly as bssnRHS does (BSSN_GR/src/rhs.cpp:45-62)."""
import os
import subprocess
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = textwrap.dedent(r"""
    #include <cstdio>
    #include <cmath>
    #include "dendro_gb300_bssn.hpp"
    // stand-ins with the reference's accessor names (include/block.h, TreeNode.h)
    struct Point { double v[3]; double x() const {return v[0];} double y() const {return v[1];}
                   double z() const {return v[2];} };
    struct Node { unsigned mn[3], mx[3];
      unsigned minX() const {return mn[0];} unsigned minY() const {return mn[1];}
      unsigned minZ() const {return mn[2];} unsigned maxX() const {return mx[0];}
      unsigned maxY() const {return mx[1];} unsigned maxZ() const {return mx[2];} };
    struct Block {
      unsigned long off; unsigned s; unsigned flag; Node node; unsigned eleOrder, lev, maxDepth;
      unsigned long getOffset() const {return off;}
      unsigned getAllocationSzX() const {return s;} unsigned getAllocationSzY() const {return s;}
      unsigned getAllocationSzZ() const {return s;} unsigned getBlkNodeFlag() const {return flag;}
      const Node& getBlockNode() const {return node;}
      // Block::computeDx (src/block.cpp:85-98)
      double gdx() const { return (double)(node.mx[0]-node.mn[0]) / (double)((1u<<(lev-lev))*eleOrder); }
      double computeDx(const Point& a, const Point& b) const { return ((b.x()-a.x())/(double)(1u<<maxDepth))*gdx(); }
      double computeDy(const Point& a, const Point& b) const { return ((b.y()-a.y())/(double)(1u<<maxDepth))*gdx(); }
      double computeDz(const Point& a, const Point& b) const { return ((b.z()-a.z())/(double)(1u<<maxDepth))*gdx(); }
    };
    int main() {
      const unsigned maxDepth = 8;
      Point pmin{{-32,-32,-32}}, pmax{{32,32,32}};
      // GRIDX_TO_X (BSSN_GR/include/grDef.h:13): octree [0, 2^maxDepth] -> [-32, 32]
      auto g2d = [&](int a, unsigned xg) { return (64.0 / 256.0) * (xg - 0.0) + (-32.0); };
      Block b{1234, 13, 0, Node{{64, 96, 128}, {72, 104, 136}}, 6, 5, maxDepth};
      dgb_block_desc d = dgb_bssn::describe_block(b, pmin, pmax, g2d);
      const double dx = b.computeDx(pmin, pmax);
      int bad = 0;
      bad += d.offset != 1234 || d.sz[0] != 13 || d.sz[2] != 13 || d.bflag != 0;
      bad += d.ptmin[0] != g2d(0, 64) - 3 * dx || d.ptmax[2] != g2d(2, 136) + 3 * dx;
      // the block spacing the RHS uses, (pmax - pmin)/(n - 1), equals dx
      bad += std::fabs((d.ptmax[0] - d.ptmin[0]) / 12.0 - dx) > 1e-15;
      // without a device the drop-in returns a status instead of exiting
      unsigned lam[4] = {1, 1, 1, 1}; double lf[2] = {1, 0};
      dgb_bssn_params p = dgb_bssn::params(lam, lf, 2.0, 30.0, 1.0, 0.1, 1e-4, 4);
      dgb_bssn::PlanCache cache;
      double* r[24]; const double* u[24];
      dgb_status s = dgb_bssn::bssnRHS(r, u, &b, 1, pmin, pmax, g2d, p, cache);
      std::printf("desc %.17g %.17g status %d\n", d.ptmin[0], d.ptmax[0], (int)s);
      return bad ? 1 : (s == DGB_ERR_NOT_INIT ? 0 : 2);
    }
""")


def test_shim_compiles_and_describes_blocks(dgb, tmp_path):
    """Runs with or without a GPU: the program never calls dgb_init, so the
    drop-in answers DGB_ERR_NOT_INIT instead of exiting."""
    src = tmp_path / "shim.cpp"
    src.write_text(SRC)
    exe = tmp_path / "shim"
    libdir = os.path.dirname(dgb.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT}/include", str(src), "-o", str(exe),
                    f"-L{libdir}", "-ldendro_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
