"""ctypes binding of libdendro_gb300.so (include/dendro_gb300.h).

The library is the product: every compute call here goes to its CUDA
kernels.  Loading fails loudly when the shared object is missing; there is
no CPU fallback.  Device arrays are passed as raw pointers (e.g. torch
tensors' data_ptr()); host arrays as numpy arrays.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# DGB_LIB selects another build of the same library (build experiments)
LIB_PATH = os.environ.get("DGB_LIB") or os.path.join(HERE, "libdendro_gb300.so")
NUM_VARS = 24

VAR_NAMES = ["alpha", "chi", "K", "Gt0", "Gt1", "Gt2", "beta0", "beta1", "beta2",
             "B0", "B1", "B2", "gt0", "gt1", "gt2", "gt3", "gt4", "gt5",
             "At0", "At1", "At2", "At3", "At4", "At5"]

DGB_OK = 0
PREC_FP64 = 0
PREC_MIXED = 1
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "ALLOC", 4: "NOT_INIT", 5: "TIMEOUT",
                6: "NONFINITE", 7: "CONSTRAINT", 8: "UNSUPPORTED"}


class BlockDesc(C.Structure):
    _fields_ = [("offset", C.c_uint64), ("sz", C.c_uint32 * 3), ("bflag", C.c_uint32),
                ("ptmin", C.c_double * 3), ("ptmax", C.c_double * 3)]


class BssnParams(C.Structure):
    _fields_ = [("lambda_", C.c_double * 4), ("lambda_f", C.c_double * 2),
                ("eta_const", C.c_double), ("eta_r0", C.c_double),
                ("eta_damping_exp", C.c_double), ("ko_sigma", C.c_double),
                ("chi_floor", C.c_double)]


def default_params(ko_sigma=0.1):
    """lambda = {1,1,1,1}, lambda_f = {1,0}, eta = 2 (R0 = 30, exponent 1),
    chi_floor = 1e-4 (BSSN_GR/pars/bbh.par.json:103-129)."""
    p = BssnParams()
    p.lambda_[:] = [1.0, 1.0, 1.0, 1.0]
    p.lambda_f[:] = [1.0, 0.0]
    p.eta_const = 2.0
    p.eta_r0 = 30.0
    p.eta_damping_exp = 1.0
    p.ko_sigma = ko_sigma
    p.chi_floor = 1e-4
    return p


def params_vector(p):
    """The 10-double vector the oracle and the reference harness take."""
    return np.array(list(p.lambda_) + list(p.lambda_f)
                    + [p.eta_const, p.eta_r0, p.eta_damping_exp, p.ko_sigma], dtype=np.float64)


class DgbError(RuntimeError):
    pass


_lib = None

PtrArr = C.POINTER(C.c_void_p)

_SIGS = {
    "dgb_version": (C.c_int, []),
    "dgb_last_error": (C.c_char_p, []),
    "dgb_init": (C.c_int, [C.c_int]),
    "dgb_plan_create": (C.c_int, [C.POINTER(BlockDesc), C.c_size_t, C.POINTER(BssnParams),
                                  C.POINTER(C.c_void_p)]),
    "dgb_plan_destroy": (C.c_int, [C.c_void_p]),
    "dgb_plan_unzipped_size": (C.c_uint64, [C.c_void_p]),
    "dgb_plan_interior_points": (C.c_uint64, [C.c_void_p]),
    "dgb_bssn_rhs": (C.c_int, [C.c_void_p, PtrArr, PtrArr, C.c_int, C.c_void_p]),
    "dgb_bssn_rhs_host": (C.c_int, [C.c_void_p, PtrArr, PtrArr, C.c_int]),
    "dgb_bssnrhs_block_host": (C.c_int, [PtrArr, PtrArr, C.c_uint64, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_uint32),
                                         C.c_uint32, C.POINTER(BssnParams), C.c_int]),
    "dgb_bssnrhs_block_noalloc": (C.c_int, [PtrArr, PtrArr, C.c_uint64, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(C.c_uint32),
                                            C.c_uint32, C.POINTER(BssnParams), C.c_void_p]),
    "dgb_plan_autotune": (C.c_int, [C.c_void_p, PtrArr, PtrArr, C.c_int, C.c_void_p]),
    "dgb_plan_tile": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint32)]),
    "dgb_num_tile_variants": (C.c_int, []),
    "dgb_plan_set_tile_variant": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "dgb_rk4_stage": (C.c_int, [C.c_int, PtrArr, PtrArr, PtrArr, C.c_uint64, C.c_double,
                                C.c_double, C.c_void_p]),
    "dgb_synth_fill_host": (C.c_int, [C.POINTER(BlockDesc), C.c_size_t, PtrArr, C.c_uint64,
                                      C.c_double, C.c_int]),
    "dgb_synth_fill_device": (C.c_int, [C.c_void_p, PtrArr, C.c_uint64, C.c_double,
                                        C.c_void_p]),
    "dgb_synth_blocks": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(BlockDesc),
                                   C.POINTER(C.c_size_t)]),
    "dgb_measure_fp64_peak": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "dgb_selftest_exact_mul": (C.c_int, [C.c_int, C.c_uint64, C.c_uint64,
                                         C.POINTER(C.c_uint64)]),
}


def selftest_exact_mul(on_device, n, seed=1):
    bad = C.c_uint64()
    check(lib().dgb_selftest_exact_mul(on_device, n, seed, C.byref(bad)),
          "dgb_selftest_exact_mul")
    return bad.value


def measure_fp64_peak():
    g, ms = C.c_double(), C.c_double()
    check(lib().dgb_measure_fp64_peak(C.byref(g), C.byref(ms)), "dgb_measure_fp64_peak")
    return g.value, ms.value

EXPORTED = sorted(_SIGS)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise DgbError(f"{LIB_PATH} is missing: build it first (python build.py)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, what=""):
    if status != DGB_OK:
        msg = lib().dgb_last_error().decode(errors="replace")
        raise DgbError(f"{what}: {STATUS_NAMES.get(status, status)}: {msg}")


def ptr_array(ptrs):
    arr = (C.c_void_p * len(ptrs))(*[C.c_void_p(int(p)) for p in ptrs])
    return C.cast(arr, PtrArr), arr


def host_ptrs(arrays):
    return ptr_array([a.ctypes.data for a in arrays])


def synth_blocks(which, seed=0):
    n = C.c_size_t(0)
    check(lib().dgb_synth_blocks(which, seed, None, C.byref(n)), "dgb_synth_blocks")
    arr = (BlockDesc * n.value)()
    check(lib().dgb_synth_blocks(which, seed, arr, C.byref(n)), "dgb_synth_blocks")
    return arr


def blocks_array(rows):
    """rows: iterable of (offset, (sx,sy,sz), bflag, ptmin3, ptmax3)."""
    rows = list(rows)
    arr = (BlockDesc * len(rows))()
    for b, (off, sz, bflag, pmin, pmax) in enumerate(rows):
        arr[b].offset = off
        arr[b].sz[:] = list(sz)
        arr[b].bflag = bflag
        arr[b].ptmin[:] = list(pmin)
        arr[b].ptmax[:] = list(pmax)
    return arr


def unzipped_size(blocks):
    return max((b.offset + b.sz[0] * b.sz[1] * b.sz[2] for b in blocks), default=0)


def synth_fill_host(blocks, fields, seed, noise=1e-6, nthreads=0):
    pa, keep = host_ptrs(fields)
    check(lib().dgb_synth_fill_host(blocks, len(blocks), pa, seed, noise, nthreads),
          "dgb_synth_fill_host")


def init(device=0):
    check(lib().dgb_init(device), "dgb_init")


class Plan:
    def __init__(self, blocks, params):
        self.blocks = blocks
        self.params = params
        h = C.c_void_p()
        check(lib().dgb_plan_create(blocks, len(blocks), C.byref(params), C.byref(h)),
              "dgb_plan_create")
        self.h = h

    @property
    def unzipped(self):
        return lib().dgb_plan_unzipped_size(self.h)

    @property
    def interior(self):
        return lib().dgb_plan_interior_points(self.h)

    def rhs_device(self, rhs_ptrs, u_ptrs, precision=PREC_FP64, stream=0):
        r, k1 = ptr_array(rhs_ptrs)
        u, k2 = ptr_array(u_ptrs)
        check(lib().dgb_bssn_rhs(self.h, r, u, precision, C.c_void_p(stream)), "dgb_bssn_rhs")

    def rhs_host(self, rhs_arrays, u_arrays, precision=PREC_FP64):
        r, k1 = host_ptrs(rhs_arrays)
        u, k2 = host_ptrs(u_arrays)
        check(lib().dgb_bssn_rhs_host(self.h, r, u, precision), "dgb_bssn_rhs_host")

    def autotune(self, rhs_ptrs, u_ptrs, precision=PREC_FP64, stream=0):
        r, k1 = ptr_array(rhs_ptrs)
        u, k2 = ptr_array(u_ptrs)
        check(lib().dgb_plan_autotune(self.h, r, u, precision, C.c_void_p(stream)),
              "dgb_plan_autotune")

    def tile(self, precision=PREC_FP64):
        t = (C.c_uint32 * 3)()
        check(lib().dgb_plan_tile(self.h, precision, t), "dgb_plan_tile")
        return tuple(t)

    def set_tile_variant(self, variant, precision=PREC_FP64):
        check(lib().dgb_plan_set_tile_variant(self.h, precision, variant),
              "dgb_plan_set_tile_variant")

    def synth_fill_device(self, u_ptrs, seed, noise=1e-6, stream=0):
        u, k = ptr_array(u_ptrs)
        check(lib().dgb_synth_fill_device(self.h, u, seed, noise, C.c_void_p(stream)),
              "dgb_synth_fill_device")

    def close(self):
        if self.h:
            lib().dgb_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rk4_stage(stage, dst_ptrs, prev_ptrs, k_ptrs, nnodes, dt, chi_floor=1e-4, stream=0):
    d, k1 = ptr_array(dst_ptrs)
    p, k2 = ptr_array(prev_ptrs)
    kk, k3 = ptr_array(k_ptrs)
    check(lib().dgb_rk4_stage(stage, d, p, kk, nnodes, dt, chi_floor, C.c_void_p(stream)),
          "dgb_rk4_stage")
