"""ORACLE binding — test infrastructure only (tests/, smoke(), bench.py's
CPU-baseline leg).  Loads oracle/_build/liboracle.so (the C restatement,
built by `make -f oracle/Makefile`) and, where they were built,
oracle/_ref/libdendro_ref.so, libccz4_ref.so and libmesh_ref.so (the
reference's own sources, `make -f oracle/Makefile.ref`)."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
# the same sources built -O3 for the host's own CPU: the CPU timing legs
ORACLE_BENCH_SO = os.path.join(HERE, "_build", "liboracle_bench.so")
REF_SO = os.path.join(HERE, "_ref", "libdendro_ref.so")
CCZ4_REF_SO = os.path.join(HERE, "_ref", "libccz4_ref.so")
MESH_REF_SO = os.path.join(HERE, "_ref", "libmesh_ref.so")
# where the reference tree lies (read-only); DENDRO_REF overrides the default
REF_ROOT = os.environ.get("DENDRO_REF", "/root/reference")

_D = C.POINTER(C.c_double)
_PP = C.POINTER(C.c_void_p)


def build_oracle():
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")], check=True)
    return ORACLE_SO


def build_ref(ref_root=None):
    """Compile the reference's own sources (only where the tree exists)."""
    ref_root = ref_root or REF_ROOT
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
        L.orc_bssnrhs_ex2.restype = C.c_int
        L.orc_bssnrhs_ex2.argtypes = [_PP, _PP, C.c_ulong, _D, _D, C.POINTER(C.c_uint), C.c_uint,
                                      _D, C.c_int, C.c_int]
        L.orc_bssnrhs_blocks_ex.restype = C.c_int
        L.orc_bssnrhs_blocks_ex.argtypes = [_PP, _PP, C.c_long, C.POINTER(C.c_ulong),
                                            C.POINTER(C.c_uint), C.POINTER(C.c_uint), _D, _D, _D,
                                            C.c_int, C.c_int]
        L.orc_bssnrhs_blocks.restype = C.c_int
        L.orc_bssnrhs_blocks.argtypes = [_PP, _PP, C.c_long, C.POINTER(C.c_ulong),
                                         C.POINTER(C.c_uint), C.POINTER(C.c_uint), _D, _D, _D,
                                         C.c_int]
        L.orc_rk4_stage.restype = None
        L.orc_rk4_stage.argtypes = [C.c_int, _PP, _PP, C.POINTER(_PP), C.c_size_t, C.c_double,
                                    C.c_double]
        L.orc_unzip.restype = None
        L.orc_unzip.argtypes = [C.c_void_p, C.c_void_p, C.c_ulonglong, C.c_void_p, C.c_ulonglong,
                                C.c_void_p, C.c_void_p, C.c_ulonglong, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_int]
        L.orc_zip.restype = None
        L.orc_zip.argtypes = [C.c_void_p, C.c_void_p, C.c_ulonglong, C.c_void_p]
        L.orc_enforce_bssn_constraints.restype = None
        L.orc_enforce_bssn_constraints.argtypes = [_PP, C.c_size_t, C.c_double]
        L.orc_physcon_block.restype = C.c_int
        L.orc_physcon_block.argtypes = [_PP, _PP, C.c_ulong, _D, _D, C.POINTER(C.c_uint), C.c_uint]
        L.orc_physcon_blocks.restype = C.c_int
        L.orc_physcon_blocks.argtypes = [_PP, _PP, C.c_long, C.POINTER(C.c_ulong),
                                         C.POINTER(C.c_uint), C.POINTER(C.c_uint), _D, _D, C.c_int]
        L.orc_ccz4rhs_ex.restype = C.c_int
        L.orc_ccz4rhs_ex.argtypes = [_PP, _PP, C.c_ulong, _D, _D, C.POINTER(C.c_uint), C.c_uint,
                                     _D, C.c_int]
        L.orc_ccz4rhs_blocks.restype = C.c_int
        L.orc_ccz4rhs_blocks.argtypes = [_PP, _PP, C.c_long, C.POINTER(C.c_ulong),
                                         C.POINTER(C.c_uint), C.POINTER(C.c_uint), _D, _D, _D,
                                         C.c_int, C.c_int]
        L.orc_ccz4_adv42.restype = None
        L.orc_ccz4_adv42.argtypes = [C.c_int, _D, _D, C.c_double, C.POINTER(C.c_uint), _D, C.c_uint]
        L.orc_wavelet_patch.restype = None
        L.orc_wavelet_patch.argtypes = [_D, C.c_int, _D]
        L.orc_wavelet_rms.restype = C.c_double
        L.orc_wavelet_rms.argtypes = [_D]
        L.orc_synth_blocks.restype = C.c_long
        L.orc_synth_blocks.argtypes = [C.c_int, C.c_uint64, C.c_void_p]
        L.orc_synth_fill.restype = None
        L.orc_synth_fill.argtypes = [C.c_void_p, C.c_long, _PP, C.c_int, C.c_uint64, C.c_double,
                                     C.c_int]
        L.orc_remesh_wavelets.restype = C.c_uint64
        L.orc_remesh_wavelets.argtypes = [_PP, C.POINTER(C.c_uint32), C.c_int, C.c_uint64,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_double, C.c_void_p, C.c_void_p, C.c_int]
        for nm in ("orc_deriv64", "orc_deriv64_2", "orc_ko42", "orc_deriv42", "orc_deriv42_2",
                   "orc_ccz4_ko42"):
            f = getattr(L, nm)
            f.restype = None
            f.argtypes = [C.c_int, _D, _D, C.c_double, C.POINTER(C.c_uint), C.c_uint]
        self.L = L

    def synth_blocks(self, which, seed, block_type):
        """The synthetic block list (which = 1: 512 uniform 13^3 blocks, 2: the
        uneven 20,000-block batch) as an array of block_type (a ctypes
        structure with the dgb_block_desc layout)."""
        n = self.L.orc_synth_blocks(which, seed, None)
        arr = (block_type * n)()
        self.L.orc_synth_blocks(which, seed, C.addressof(arr))
        return arr

    def synth_fill(self, blocks, fields, seed, noise=1e-6, nthreads=0):
        """Brill-Lindquist + seeded noise into fields (24 or 25 arrays)."""
        pp, keep = _ptrs(fields)
        self.L.orc_synth_fill(C.addressof(blocks), len(blocks), pp, len(fields), seed, noise,
                              nthreads or (os.cpu_count() or 1))

    def bssnrhs_blocks(self, rhs, u, blocks, prm, nthreads=0, order=6):
        """bssnRHS over a block list (list of dgb BlockDesc); order 6: the
        QuadGrav binding, 4: the BSSN_GR solver's (upwinded advection)."""
        n = len(blocks)
        off = (C.c_ulong * n)(*[b.offset for b in blocks])
        sz = (C.c_uint * (3 * n))(*[s for b in blocks for s in b.sz])
        bf = (C.c_uint * n)(*[b.bflag for b in blocks])
        pmin = np.array([x for b in blocks for x in b.ptmin], dtype=np.float64)
        pmax = np.array([x for b in blocks for x in b.ptmax], dtype=np.float64)
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        return self.L.orc_bssnrhs_blocks_ex(r, uu, n, off, sz, bf, pmin.ctypes.data_as(_D),
                                            pmax.ctypes.data_as(_D), p.ctypes.data_as(_D),
                                            nthreads, order)

    def stencil(self, kind, dirn, u3, h, bflag=0):
        """kind in {'d1','d2','ko'} on a 3-D array u3[z][y][x]; returns D (zeros
        where the reference leaves the output untouched)."""
        fn = {"d1": self.L.orc_deriv64, "d2": self.L.orc_deriv64_2, "ko": self.L.orc_ko42,
              "d1_4": self.L.orc_deriv42, "d2_4": self.L.orc_deriv42_2,
              "ko_ccz4": self.L.orc_ccz4_ko42}[kind]
        u = np.ascontiguousarray(u3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        fn(dirn, D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz, bflag)
        return D

    def adv_ccz4(self, dirn, u3, h, beta3, bflag=0):
        """CCZ4 upwind advective derivative on u3[z][y][x] with shift component beta3."""
        u = np.ascontiguousarray(u3, dtype=np.float64)
        b = np.ascontiguousarray(beta3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        self.L.orc_ccz4_adv42(dirn, D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz,
                              b.ctypes.data_as(_D), bflag)
        return D

    def ccz4rhs_blocks(self, rhs, u, blocks, prm, apply_bcs=True, nthreads=0):
        """ccz4rhs over a block list; rhs, u: 25 arrays in CCZ4 variable order."""
        n = len(blocks)
        off = (C.c_ulong * n)(*[b.offset for b in blocks])
        sz = (C.c_uint * (3 * n))(*[s for b in blocks for s in b.sz])
        bf = (C.c_uint * n)(*[b.bflag for b in blocks])
        pmin = np.array([x for b in blocks for x in b.ptmin], dtype=np.float64)
        pmax = np.array([x for b in blocks for x in b.ptmax], dtype=np.float64)
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        return self.L.orc_ccz4rhs_blocks(r, uu, n, off, sz, bf, pmin.ctypes.data_as(_D),
                                         pmax.ctypes.data_as(_D), p.ctypes.data_as(_D),
                                         1 if apply_bcs else 0, nthreads)

    def physcon_block(self, cons, u, block):
        """physical_constraints on one block: cons = 6 arrays (ham, mom0-2,
        psi4_real, psi4_img), written at the block's interior points."""
        c, k1 = _ptrs(cons)
        uu, k2 = _ptrs(u)
        pmin = np.array(list(block.ptmin), dtype=np.float64)
        pmax = np.array(list(block.ptmax), dtype=np.float64)
        sz = (C.c_uint * 3)(*block.sz)
        return self.L.orc_physcon_block(c, uu, block.offset, pmin.ctypes.data_as(_D),
                                        pmax.ctypes.data_as(_D), sz, block.bflag)

    def physcon_blocks(self, cons, u, blocks, nthreads=0):
        n = len(blocks)
        off = (C.c_ulong * n)(*[b.offset for b in blocks])
        sz = (C.c_uint * (3 * n))(*[s for b in blocks for s in b.sz])
        bf = (C.c_uint * n)(*[b.bflag for b in blocks])
        pmin = np.array([x for b in blocks for x in b.ptmin], dtype=np.float64)
        pmax = np.array([x for b in blocks for x in b.ptmax], dtype=np.float64)
        c, k1 = _ptrs(cons)
        uu, k2 = _ptrs(u)
        return self.L.orc_physcon_blocks(c, uu, n, off, sz, bf, pmin.ctypes.data_as(_D),
                                         pmax.ctypes.data_as(_D), nthreads)

    def wavelet_patch(self, patch, boundary):
        """compute_wavelets_3D on one 13^3 patch (x fastest): the 64 wavelet
        slots and their RMS."""
        p = np.ascontiguousarray(patch, dtype=np.float64).reshape(-1)
        assert p.size == 13 ** 3
        wc = np.zeros(64)
        self.L.orc_wavelet_patch(p.ctypes.data_as(_D), 1 if boundary else 0, wc.ctypes.data_as(_D))
        return wc, self.L.orc_wavelet_rms(wc.ctypes.data_as(_D))

    def remesh_wavelets(self, unzipped, var_ids, patch_base, block_side, boundary, tol,
                        coarse_fac, nthreads=0):
        """isReMeshUnzip's indicator over a leaf list: (wmax, flags, changed)."""
        n = len(patch_base)
        pb = np.ascontiguousarray(patch_base, dtype=np.uint64)
        bs = np.ascontiguousarray(block_side, dtype=np.uint32)
        bd = np.ascontiguousarray(boundary, dtype=np.uint8)
        tl = np.ascontiguousarray(tol, dtype=np.float64)
        wmax = np.zeros(n)
        flags = np.zeros(n, dtype=np.uint8)
        uu, k1 = _ptrs(unzipped)
        vid = (C.c_uint32 * len(var_ids))(*var_ids)
        changed = self.L.orc_remesh_wavelets(uu, vid, len(var_ids), n, pb.ctypes.data,
                                             bs.ctypes.data, bd.ctypes.data, tl.ctypes.data,
                                             coarse_fac, wmax.ctypes.data, flags.ctypes.data,
                                             nthreads or os.cpu_count())
        return wmax, flags, int(changed)

    def bssnrhs_block(self, rhs, u, block, prm, apply_bcs=True, order=6):
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        pmin = np.array(list(block.ptmin), dtype=np.float64)
        pmax = np.array(list(block.ptmax), dtype=np.float64)
        sz = (C.c_uint * 3)(*block.sz)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        return self.L.orc_bssnrhs_ex2(r, uu, block.offset, pmin.ctypes.data_as(_D),
                                      pmax.ctypes.data_as(_D), sz, block.bflag,
                                      p.ctypes.data_as(_D), 1 if apply_bcs else 0, order)

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


class CCZ4Reference:
    """The reference's own CCZ4 code (CCZ4_GR/src/derivs.cpp + the ccz4rhs
    harness), machines with the reference tree only."""

    def __init__(self, path=CCZ4_REF_SO):
        L = C.CDLL(path)
        L.ref_ccz4rhs.restype = C.c_int
        L.ref_ccz4rhs.argtypes = [_PP, _PP, C.c_uint, _D, _D, C.POINTER(C.c_uint), C.c_uint, _D]
        for nm in ("ccz4_deriv42_x", "ccz4_deriv42_y", "ccz4_deriv42_z", "ccz4_deriv42_xx",
                   "ccz4_deriv42_yy", "ccz4_deriv42_zz", "ccz4_ko_deriv42_x",
                   "ccz4_ko_deriv42_y", "ccz4_ko_deriv42_z"):
            f = getattr(L, nm)
            f.restype = None
            f.argtypes = [_D, _D, C.c_double, C.POINTER(C.c_uint), C.c_uint]
        for nm in ("ccz4_deriv42adv_x", "ccz4_deriv42adv_y", "ccz4_deriv42adv_z"):
            f = getattr(L, nm)
            f.restype = None
            f.argtypes = [_D, _D, C.c_double, C.POINTER(C.c_uint), _D, C.c_uint]
        self.L = L

    def ccz4rhs(self, rhs, u, block, prm):
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        pmin = np.array(list(block.ptmin), dtype=np.float64)
        pmax = np.array(list(block.ptmax), dtype=np.float64)
        sz = (C.c_uint * 3)(*block.sz)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        return self.L.ref_ccz4rhs(r, uu, block.offset, pmin.ctypes.data_as(_D),
                                  pmax.ctypes.data_as(_D), sz, block.bflag, p.ctypes.data_as(_D))

    def stencil(self, kind, dirn, u3, h, bflag=0):
        nm = {"d1_4": ["ccz4_deriv42_x", "ccz4_deriv42_y", "ccz4_deriv42_z"],
              "d2_4": ["ccz4_deriv42_xx", "ccz4_deriv42_yy", "ccz4_deriv42_zz"],
              "ko_ccz4": ["ccz4_ko_deriv42_x", "ccz4_ko_deriv42_y", "ccz4_ko_deriv42_z"]}[kind][dirn]
        u = np.ascontiguousarray(u3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        getattr(self.L, nm)(D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz, bflag)
        return D

    def adv(self, dirn, u3, h, beta3, bflag=0):
        nm = ["ccz4_deriv42adv_x", "ccz4_deriv42adv_y", "ccz4_deriv42adv_z"][dirn]
        u = np.ascontiguousarray(u3, dtype=np.float64)
        b = np.ascontiguousarray(beta3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        getattr(self.L, nm)(D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz,
                            b.ctypes.data_as(_D), bflag)
        return D


class Reference:
    """The reference's own compiled code (machines with the reference tree)."""

    def __init__(self, path=REF_SO):
        L = C.CDLL(path)
        L.ref_bssnrhs.restype = C.c_int
        L.ref_bssnrhs.argtypes = [_PP, _PP, C.c_uint, _D, _D, C.POINTER(C.c_uint), C.c_uint, _D]
        L.ref_bssnrhs42.restype = C.c_int
        L.ref_bssnrhs42.argtypes = [_PP, _PP, C.c_uint, _D, _D, C.POINTER(C.c_uint), C.c_uint, _D]
        L.ref_deriv42adv.restype = None
        L.ref_deriv42adv.argtypes = [C.c_int, _D, _D, C.c_double, C.POINTER(C.c_uint), _D, C.c_uint]
        L.ref_enforce_bssn_constraints.restype = None
        L.ref_enforce_bssn_constraints.argtypes = [_PP, C.c_uint, C.c_double]
        L.ref_physical_constraints.restype = C.c_int
        L.ref_physical_constraints.argtypes = [_PP, _PP, C.c_uint, _D, _D, C.POINTER(C.c_uint),
                                               C.c_uint]
        for nm in ("ref_deriv64_x", "ref_deriv64_y", "ref_deriv64_z", "ref_deriv64_xx",
                   "ref_deriv64_yy", "ref_deriv64_zz", "ref_ko_deriv42_x", "ref_ko_deriv42_y",
                   "ref_ko_deriv42_z", "ref_deriv42_x", "ref_deriv42_y", "ref_deriv42_z",
                   "ref_deriv42_xx", "ref_deriv42_yy", "ref_deriv42_zz"):
            f = getattr(L, nm)
            f.restype = None
            f.argtypes = [_D, _D, C.c_double, C.POINTER(C.c_uint), C.c_uint]
        self.L = L

    def bssnrhs(self, rhs, u, block, prm, order=6):
        """The reference's bssnrhs on one block; order 6: QuadGrav's binding,
        4: the BSSN_GR solver's (ref_bssnrhs42)."""
        r, k1 = _ptrs(rhs)
        uu, k2 = _ptrs(u)
        pmin = np.array(list(block.ptmin), dtype=np.float64)
        pmax = np.array(list(block.ptmax), dtype=np.float64)
        sz = (C.c_uint * 3)(*block.sz)
        p = np.ascontiguousarray(prm, dtype=np.float64)
        fn = self.L.ref_bssnrhs42 if order == 4 else self.L.ref_bssnrhs
        return fn(r, uu, block.offset, pmin.ctypes.data_as(_D), pmax.ctypes.data_as(_D), sz,
                  block.bflag, p.ctypes.data_as(_D))

    def adv42(self, dirn, u3, h, beta3, bflag=0):
        """The BSSN_GR solver's upwinded deriv42adv along dirn on u3[z][y][x]."""
        u = np.ascontiguousarray(u3, dtype=np.float64)
        b = np.ascontiguousarray(beta3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        self.L.ref_deriv42adv(dirn, D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz,
                              b.ctypes.data_as(_D), bflag)
        return D

    def stencil(self, kind, dirn, u3, h, bflag=0):
        nm = {"d1": ["ref_deriv64_x", "ref_deriv64_y", "ref_deriv64_z"],
              "d2": ["ref_deriv64_xx", "ref_deriv64_yy", "ref_deriv64_zz"],
              "ko": ["ref_ko_deriv42_x", "ref_ko_deriv42_y", "ref_ko_deriv42_z"],
              "d1_4": ["ref_deriv42_x", "ref_deriv42_y", "ref_deriv42_z"],
              "d2_4": ["ref_deriv42_xx", "ref_deriv42_yy", "ref_deriv42_zz"]}[kind][dirn]
        u = np.ascontiguousarray(u3, dtype=np.float64)
        D = np.zeros_like(u)
        sz = (C.c_uint * 3)(u.shape[2], u.shape[1], u.shape[0])
        getattr(self.L, nm)(D.ctypes.data_as(_D), u.ctypes.data_as(_D), h, sz, bflag)
        return D

    def physical_constraints(self, cons, u, block):
        c, k1 = _ptrs(cons)
        uu, k2 = _ptrs(u)
        pmin = np.array(list(block.ptmin), dtype=np.float64)
        pmax = np.array(list(block.ptmax), dtype=np.float64)
        sz = (C.c_uint * 3)(*block.sz)
        return self.L.ref_physical_constraints(c, uu, block.offset, pmin.ctypes.data_as(_D),
                                               pmax.ctypes.data_as(_D), sz, block.bflag)

    def enforce(self, fields, node, chi_floor):
        pp, k = _ptrs(fields)
        self.L.ref_enforce_bssn_constraints(pp, node, chi_floor)


# ----------------------------------------------------------------------------
# Host application of a mesh's unzip / zip operator and the RK4 step pipeline
# (RK_BSSN::performSingleIteration's RK4 branch, BSSN_GR/src/rkBSSN.cpp:803-1012):
# the checker for the GPU unzip, zip and graph-captured step.

def _lagrange_table():
    t = np.zeros((6, 7))
    for r in range(6):
        xi = r + 0.5
        for i in range(7):
            num = den = 1.0
            for m in range(7):
                if m != i:
                    num *= xi - m
                    den *= i - m
            t[r, i] = num / den
    return t


LAG = _lagrange_table()


def _ref_values(refs, z, dg, chunk=65536):
    """Values of 64-bit node references: bit 63 clear = copy of zipped node
    (low 32 bits); set = separable degree-6 interpolation of source element
    (bits 12..42) at codes 2*xi (bits 0..11, 4 per axis)."""
    out = np.empty(len(refs))
    interp = (refs >> np.uint64(63)) != 0
    out[~interp] = z[(refs[~interp] & np.uint64(0xFFFFFFFF)).astype(np.int64)]
    idx = np.nonzero(interp)[0]
    for c0 in range(0, len(idx), chunk):
        sel = idx[c0:c0 + chunk]
        r = refs[sel]
        src = ((r >> np.uint64(12)) & np.uint64(0x7FFFFFFF)).astype(np.int64)
        W = []
        for a in range(3):
            code = ((r >> np.uint64(4 * a)) & np.uint64(0xF)).astype(np.int64)
            w = np.zeros((len(r), 7))
            even = code % 2 == 0
            w[np.nonzero(even)[0], code[even] // 2] = 1.0
            w[~even] = LAG[code[~even] // 2]
            W.append(w)
        E = dg[src].reshape(len(r), 7, 7, 7)  # [k][j][i]
        out[sel] = np.einsum("nk,nj,ni,nkji->n", W[2], W[1], W[0], E)
    return out


_ORC = None


def _default_oracle():
    global _ORC
    if _ORC is None:
        _ORC = Oracle()
    return _ORC


def unzip_apply(op, z, n, oracle=None, nthreads=0):
    """Mesh::unzip on the host from the operator (oracle/bssn_oracle.c
    orc_unzip); NaN where nothing is written (padding beyond domain faces)."""
    ora = oracle or _default_oracle()
    out = np.full(n, np.nan)
    nsrc = len(op["src_refs"]) // 343
    dg = np.zeros(max(nsrc * 343, 1))
    nlev = max(len(op["level_ptr"]) - 1, 0)
    ora.L.orc_unzip(np.ascontiguousarray(z).ctypes.data, out.ctypes.data, n,
                    op["copy_src"].ctypes.data, len(op["interp_dst"]), op["interp_dst"].ctypes.data,
                    op["interp_ref"].ctypes.data, nlev, op["level_ptr"].ctypes.data,
                    op["src_refs"].ctypes.data, dg.ctypes.data, nthreads)
    return out


def unzip_apply_numpy(op, z, n):
    """Same operator applied with numpy (an independent second restatement)."""
    lp = op["level_ptr"].astype(np.int64)
    nsrc = len(op["src_refs"]) // 343
    dg = np.zeros((nsrc, 343))
    for l in range(len(lp) - 1):
        a, b = lp[l], lp[l + 1]
        dg[a:b] = _ref_values(op["src_refs"][a * 343:b * 343], z, dg).reshape(b - a, 343)
    out = np.full(n, np.nan)
    cp = op["copy_src"]
    m = cp != 0xFFFFFFFF
    out[m] = z[cp[m]]
    if len(op["interp_dst"]):
        out[op["interp_dst"].astype(np.int64)] = _ref_values(op["interp_ref"], z, dg)
    return out


def rk4_step_pipeline(oracle, blocks, op, nunzipped, state, dt, prm, chi_floor=1e-4, nthreads=0):
    """One RK4 step: for each stage unzip -> bssnrhs per block -> zip -> stage
    update with enforce_bssn_constraints.  Returns the new state."""
    prev = state
    ks, im = [], prev
    zs = op["zip_src"].astype(np.int64)
    ndof = len(state[0])
    for s in range(4):
        src = prev if s == 0 else im
        U = [np.nan_to_num(unzip_apply(op, src[v], nunzipped, oracle, nthreads), nan=0.0)
             for v in range(24)]
        R = [np.zeros(nunzipped) for _ in range(24)]
        assert oracle.bssnrhs_blocks(R, U, blocks, prm, nthreads) == 0
        ks.append([R[v][zs] for v in range(24)])
        dst = [np.zeros(ndof) for _ in range(24)]
        oracle.rk4_stage(s, dst, prev, ks, dt, chi_floor)
        im = dst
    return im


class MeshReference:
    """The reference's own ot::Mesh (oracle/ref_mesh.cpp over src/mesh.cpp,
    include/mesh.tcc, src/octUtils.cpp ... built by oracle/Makefile.ref with a
    single-rank MPI stand-in and an own dgesv_), built from a leaf list."""

    def __init__(self, path=MESH_REF_SO):
        L = C.CDLL(path)
        V = C.c_void_p
        L.refmesh_build.argtypes = [V, V, C.c_uint64, C.c_uint, C.c_uint]
        for nm in ("refmesh_sizes", "refmesh_blocks", "refmesh_elements", "refmesh_cg_coords",
                   "refmesh_zip_owner"):
            getattr(L, nm).argtypes = [V]
        L.refmesh_element_patches.argtypes = [V, V, V, V]
        L.refmesh_unzip.argtypes = [V, V]
        L.refmesh_zip.argtypes = [V, V]
        L.refmesh_wavelets.argtypes = [C.c_uint, V, V, C.c_int, V, V]
        L.refmesh_destroy.restype = None
        self.L = L

    def build(self, anchors, levels, max_depth, order=6):
        """anchors: (n, 3) in octree units of max_depth; levels: (n,)."""
        a = np.ascontiguousarray(anchors, dtype=np.uint32)
        lv = np.ascontiguousarray(levels, dtype=np.uint8)
        assert self.L.refmesh_build(a.ctypes.data, lv.ctypes.data, len(lv), max_depth, order) == 0
        s = (C.c_uint64 * 8)()
        self.L.refmesh_sizes(s)
        (self.nelem, self.nblocks, self.nunzipped, self.ncg, self.node_begin, self.node_end,
         self.elem_begin, self.elem_end) = [int(x) for x in s]
        return self

    def blocks(self):
        """(nblocks, 12): node x, y, z, level, regular level, sizes x, y, z,
        offset, face flags, element range."""
        b = np.zeros((self.nblocks, 12), dtype=np.int64)
        self.L.refmesh_blocks(b.ctypes.data)
        return b

    def elements(self):
        e = np.zeros((self.nelem, 4), dtype=np.uint32)
        self.L.refmesh_elements(e.ctypes.data)
        return e

    def cg_coords(self):
        """CG node coordinates in octree units (n, 3)."""
        x = np.zeros((self.ncg, 3))
        self.L.refmesh_cg_coords(x.ctypes.data)
        return x

    def zip_owner(self):
        o = np.zeros(self.ncg, dtype=np.int64)
        self.L.refmesh_zip_owner(o.ctypes.data)
        return o

    def unzip(self, cg):
        out = np.full(self.nunzipped, np.nan)
        c = np.ascontiguousarray(cg, dtype=np.float64)
        self.L.refmesh_unzip(c.ctypes.data, out.ctypes.data)
        return out

    def zip(self, uz):
        out = np.full(self.ncg, np.nan)
        u = np.ascontiguousarray(uz, dtype=np.float64)
        self.L.refmesh_zip(u.ctypes.data, out.ctypes.data)
        return out

    def element_patches(self, uz, with_patches=True):
        """Per local element in isReMeshUnzip's order: (element index, its
        13^3 padded patches of uz or None, isBoundaryOctant)."""
        n = self.elem_end - self.elem_begin
        e = np.zeros(n, dtype=np.int64)
        bd = np.zeros(n, dtype=np.uint8)
        pt = np.zeros((n, 13 ** 3)) if with_patches else None
        u = np.ascontiguousarray(uz, dtype=np.float64)
        self.L.refmesh_element_patches(u.ctypes.data, e.ctypes.data,
                                       pt.ctypes.data if with_patches else None, bd.ctypes.data)
        return e, pt, bd

    def wavelets(self, patch, shape, boundary, order=6):
        """WaveletEl::compute_wavelets_3D on one patch (shape x, y, z)."""
        p = np.ascontiguousarray(patch, dtype=np.float64)
        isz = np.array(shape, dtype=np.uint32)
        wc = np.zeros(4096)
        n = C.c_uint()
        self.L.refmesh_wavelets(order, p.ctypes.data, isz.ctypes.data, int(boundary), wc.ctypes.data,
                                C.addressof(n))
        return wc[:n.value].copy()

    def close(self):
        self.L.refmesh_destroy()
