"""ORACLE binding — test infrastructure only (tests/, smoke(), bench.py's
CPU-baseline leg).  Loads oracle/_build/liboracle.so (the C restatement,
built by `make -f oracle/Makefile`) and, where it was built,
oracle/_ref/libdendro_ref.so (the reference's own sources,
`make -f oracle/Makefile.ref`)."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdendro_ref.so")

_D = C.POINTER(C.c_double)
_PP = C.POINTER(C.c_void_p)


def build_oracle():
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")], check=True)
    return ORACLE_SO


def build_ref(ref_root="/root/reference"):
    """Compile the reference's own sources (only where the tree exists)."""
    if not os.path.isdir(ref_root):
        return None
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), f"REF={ref_root}"],
                   check=True)
    return REF_SO


def _ptrs(arrays, offset=0):
    arr = (C.c_void_p * len(arrays))(*[a.ctypes.data + 8 * offset for a in arrays])
    return C.cast(arr, _PP), arr


class Oracle:
    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        L = C.CDLL(path)
        L.orc_bssnrhs.restype = C.c_int
        L.orc_bssnrhs.argtypes = [_PP, _PP, C.c_ulong, _D, _D, C.POINTER(C.c_uint), C.c_uint, _D]
        L.orc_bssnrhs_ex.restype = C.c_int
        L.orc_bssnrhs_ex.argtypes = [_PP, _PP, C.c_ulong, _D, _D, C.POINTER(C.c_uint), C.c_uint,
                                     _D, C.c_int]
        L.orc_bssnrhs_blocks.restype = C.c_int
        L.orc_bssnrhs_blocks.argtypes = [_PP, _PP, C.c_long, C.POINTER(C.c_ulong),
                                         C.POINTER(C.c_uint), C.POINTER(C.c_uint), _D, _D, _D,
                                         C.c_int]
        L.orc_rk4_stage.restype = None
        L.orc_rk4_stage.argtypes = [C.c_int, _PP, _PP, C.POINTER(_PP), C.c_size_t, C.c_double,
                                    C.c_double]
        L.orc_enforce_bssn_constraints.restype = None
        L.orc_enforce_bssn_constraints.argtypes = [_PP, C.c_size_t, C.c_double]
        for nm in ("orc_deriv64", "orc_deriv64_2", "orc_ko42"):
            f = getattr(L, nm)
            f.restype = None
            f.argtypes = [C.c_int, _D, _D, C.c_double, C.POINTER(C.c_uint), C.c_uint]
        self.L = L

    def bssnrhs_blocks(self, rhs, u, blocks, prm, nthreads=0):
        """bssnRHS over a block list (list of dgb BlockDesc)."""
        n = len(blocks)
        off = (C.c_ulong * n)(*[b.offset for b in blocks])
        sz = (C.c_uint * (3 * n))(*[s for b in blocks for s in b.sz])
        bf = (C.c_uint * n)(*[b.bflag for b in blocks])
        pmin = np.array([x for b in blocks for x in b.ptmin], dtype=np.float64)
        pmax = np.array([x for b in blocks for x in b.ptmax], dtype=np.float64)
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        return self.L.orc_bssnrhs_blocks(r, uu, n, off, sz, bf, pmin.ctypes.data_as(_D),
                                         pmax.ctypes.data_as(_D), p.ctypes.data_as(_D), nthreads)

    def stencil(self, kind, dirn, u3, h, bflag=0):
        """kind in {'d1','d2','ko'} on a 3-D array u3[z][y][x]; returns D (zeros
        where the reference leaves the output untouched)."""
        fn = {"d1": self.L.orc_deriv64, "d2": self.L.orc_deriv64_2, "ko": self.L.orc_ko42}[kind]
        u = np.ascontiguousarray(u3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        fn(dirn, D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz, bflag)
        return D

    def bssnrhs_block(self, rhs, u, block, prm, apply_bcs=True):
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        pmin = np.array(list(block.ptmin), dtype=np.float64)
        pmax = np.array(list(block.ptmax), dtype=np.float64)
        sz = (C.c_uint * 3)(*block.sz)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        return self.L.orc_bssnrhs_ex(r, uu, block.offset, pmin.ctypes.data_as(_D),
                                     pmax.ctypes.data_as(_D), sz, block.bflag,
                                     p.ctypes.data_as(_D), 1 if apply_bcs else 0)

    def rk4_stage(self, s, dst, prev, k, dt, chi_floor):
        n = dst[0].size
        d, k1 = _ptrs(dst)
        p, k2 = _ptrs(prev)
        rows = []
        keep = []
        for q in range(4):
            if q < len(k):
                pp, kk = _ptrs(k[q])
                keep.append(kk)
                rows.append(pp)
            else:
                rows.append(C.cast(None, _PP))
        karr = (_PP * 4)(*rows)
        self.L.orc_rk4_stage(s, d, p, karr, n, dt, chi_floor)


class Reference:
    """The reference's own compiled code (machines with the reference tree)."""

    def __init__(self, path=REF_SO):
        L = C.CDLL(path)
        L.ref_bssnrhs.restype = C.c_int
        L.ref_bssnrhs.argtypes = [_PP, _PP, C.c_uint, _D, _D, C.POINTER(C.c_uint), C.c_uint, _D]
        L.ref_enforce_bssn_constraints.restype = None
        L.ref_enforce_bssn_constraints.argtypes = [_PP, C.c_uint, C.c_double]
        for nm in ("ref_deriv64_x", "ref_deriv64_y", "ref_deriv64_z", "ref_deriv64_xx",
                   "ref_deriv64_yy", "ref_deriv64_zz", "ref_ko_deriv42_x", "ref_ko_deriv42_y",
                   "ref_ko_deriv42_z"):
            f = getattr(L, nm)
            f.restype = None
            f.argtypes = [_D, _D, C.c_double, C.POINTER(C.c_uint), C.c_uint]
        self.L = L

    def bssnrhs(self, rhs, u, block, prm):
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        pmin = np.array(list(block.ptmin), dtype=np.float64)
        pmax = np.array(list(block.ptmax), dtype=np.float64)
        sz = (C.c_uint * 3)(*block.sz)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        return self.L.ref_bssnrhs(r, uu, block.offset, pmin.ctypes.data_as(_D),
                                  pmax.ctypes.data_as(_D), sz, block.bflag, p.ctypes.data_as(_D))

    def stencil(self, kind, dirn, u3, h, bflag=0):
        nm = {"d1": ["ref_deriv64_x", "ref_deriv64_y", "ref_deriv64_z"],
              "d2": ["ref_deriv64_xx", "ref_deriv64_yy", "ref_deriv64_zz"],
              "ko": ["ref_ko_deriv42_x", "ref_ko_deriv42_y", "ref_ko_deriv42_z"]}[kind][dirn]
        u = np.ascontiguousarray(u3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        getattr(self.L, nm)(D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz, bflag)
        return D

    def enforce(self, fields, node, chi_floor):
        pp, k = _ptrs(fields)
        self.L.ref_enforce_bssn_constraints(pp, node, chi_floor)
