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
                ("chi_floor", C.c_double), ("fd_order", C.c_int), ("gauge", C.c_int)]


GAUGE_ETA_CONST, GAUGE_ETA_FUNC, GAUGE_ROCHESTER_ETA_CONST, GAUGE_ROCHESTER_ETA_FUNC = 0, 1, 2, 3


def default_params(ko_sigma=0.1, fd_order=6):
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
    p.fd_order = fd_order
    p.gauge = GAUGE_ETA_CONST
    return p


CCZ4_VAR_NAMES = ["alpha", "psi", "K", "Gh0", "Gh1", "Gh2", "beta0", "beta1", "beta2",
                  "B0", "B1", "B2", "gt0", "gt1", "gt2", "gt3", "gt4", "gt5",
                  "At0", "At1", "At2", "At3", "At4", "At5", "theta_z4"]


class Ccz4Params(C.Structure):
    """The ccz4:: globals ccz4rhs reads (CCZ4_GR/include/parameters.h)."""
    _fields_ = [("lambda_", C.c_double * 4), ("lambda_f", C.c_double * 2),
                ("kappa", C.c_double * 2), ("p_expo", C.c_double), ("eta_const", C.c_double),
                ("eta_r0", C.c_double), ("eta_damping_exp", C.c_double),
                ("ko_sigma", C.c_double)]


def default_ccz4_params(ko_sigma=0.4, kappa=(0.1, 0.0)):
    """lambda = 1, lambda_f = (1, 0), p_expo = -1, eta = 2 within r0 = 30
    (CCZ4_GR/pars/ccz4.par.json:90-115), damping kappa."""
    p = Ccz4Params()
    p.lambda_[:] = [1.0, 1.0, 1.0, 1.0]
    p.lambda_f[:] = [1.0, 0.0]
    p.kappa[:] = list(kappa)
    p.p_expo = -1.0
    p.eta_const = 2.0
    p.eta_r0 = 30.0
    p.eta_damping_exp = 1.0
    p.ko_sigma = ko_sigma
    return p


def ccz4_params_vector(p):
    """The 13-double vector the CCZ4 oracle and reference harness take."""
    return np.array(list(p.lambda_) + list(p.lambda_f) + list(p.kappa)
                    + [p.p_expo, p.eta_const, p.eta_r0, p.eta_damping_exp, p.ko_sigma],
                    dtype=np.float64)


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
    "dgb_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "dgb_host_free": (C.c_int, [C.c_void_p]),
    "dgb_bssnrhs_block_host": (C.c_int, [PtrArr, PtrArr, C.c_uint64, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_uint32),
                                         C.c_uint32, C.POINTER(BssnParams), C.c_int]),
    "dgb_bssnrhs_block_noalloc": (C.c_int, [PtrArr, PtrArr, C.c_uint64, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(C.c_uint32),
                                            C.c_uint32, C.POINTER(BssnParams), C.c_void_p]),
    "dgb_plan_autotune": (C.c_int, [C.c_void_p, PtrArr, PtrArr, C.c_int, C.c_void_p]),
    "dgb_ccz4_rhs": (C.c_int, [C.c_void_p, C.c_void_p, PtrArr, PtrArr, C.c_int, C.c_void_p]),
    "dgb_ccz4_rhs_host": (C.c_int, [C.c_void_p, C.c_void_p, PtrArr, PtrArr, C.c_int]),
    "dgb_physical_constraints": (C.c_int, [C.c_void_p, PtrArr, PtrArr, C.c_void_p]),
    "dgb_physical_constraints_host": (C.c_int, [C.c_void_p, PtrArr, PtrArr]),
    "dgb_constraint_l2": (C.c_int, [PtrArr, C.c_int, C.c_void_p, C.c_double, C.c_uint64,
                                    C.POINTER(C.c_double), C.c_void_p]),
    "dgb_plan_tile": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint32)]),
    "dgb_plan_class_tiles": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t,
                                       C.POINTER(C.c_size_t)]),
    "dgb_num_tile_variants": (C.c_int, []),
    "dgb_plan_set_tile_variant": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "dgb_rk4_stage": (C.c_int, [C.c_int, PtrArr, PtrArr, PtrArr, C.c_uint64, C.c_double,
                                C.c_double, C.c_void_p]),
    "dgb_synth_fill_host": (C.c_int, [C.POINTER(BlockDesc), C.c_size_t, PtrArr, C.c_uint64,
                                      C.c_double, C.c_int]),
    "dgb_synth_fill_device": (C.c_int, [C.c_void_p, PtrArr, C.c_uint64, C.c_double,
                                        C.c_void_p]),
    "dgb_synth_fill_var_host": (C.c_int, [C.POINTER(BlockDesc), C.c_size_t, C.c_int,
                                          C.POINTER(C.c_double), C.c_uint64, C.c_double,
                                          C.c_int]),
    "dgb_synth_fill_var_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_uint64,
                                            C.c_double, C.c_void_p]),
    "dgb_synth_blocks": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(BlockDesc),
                                   C.POINTER(C.c_size_t)]),
    "dgb_mesh_create": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "dgb_mesh_destroy": (C.c_int, [C.c_void_p]),
    "dgb_mesh_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "dgb_mesh_blocks": (C.c_int, [C.c_void_p, C.POINTER(BlockDesc)]),
    "dgb_mesh_dof_coords": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dgb_mesh_leaf_levels": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "dgb_mesh_hilbert_tables": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "dgb_mesh_unzip_operator": (C.c_int, [C.c_void_p] + [C.c_void_p] * 6),
    "dgb_mesh_leaf_patches": (C.c_int, [C.c_void_p] + [C.c_void_p] * 5),
    "dgb_wavelet_tol_radial": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_int, C.c_void_p]),
    "dgb_remesh_wavelets": (C.c_int, [PtrArr, C.POINTER(C.c_uint32), C.c_int, C.c_uint64,
                                      C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]),
    "dgb_unzip_plan_create": (C.c_int, [C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint64,
                                        C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                        C.c_uint64, C.c_void_p, C.c_void_p,
                                        C.POINTER(C.c_void_p)]),
    "dgb_unzip_plan_destroy": (C.c_int, [C.c_void_p]),
    "dgb_unzip": (C.c_int, [C.c_void_p, PtrArr, PtrArr, C.c_int, C.c_void_p]),
    "dgb_zip": (C.c_int, [C.c_void_p, PtrArr, PtrArr, C.c_int, C.c_void_p]),
    "dgb_stepper_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "dgb_stepper_create_ex": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_uint,
                                        C.POINTER(C.c_void_p)]),
    "dgb_stepper_device_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "dgb_stepper_destroy": (C.c_int, [C.c_void_p]),
    "dgb_rk4_step": (C.c_int, [C.c_void_p, PtrArr, C.c_double, C.c_double, C.c_int,
                               C.c_void_p]),
    "dgb_synth_fill_points_host": (C.c_int, [C.c_void_p, C.c_uint64, PtrArr, C.c_uint64,
                                             C.c_double, C.c_int]),
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


def host_array(n, dtype=np.float64):
    """A zeroed numpy array of n elements in page-locked memory from
    dgb_host_alloc; the host-array entries upload such fields without the
    staging copy.  The memory is freed when the last view of it is gone."""
    import weakref
    dt = np.dtype(dtype)
    p = C.c_void_p()
    check(lib().dgb_host_alloc(max(1, n) * dt.itemsize, C.byref(p)), "dgb_host_alloc")
    buf = (C.c_char * (max(1, n) * dt.itemsize)).from_address(p.value)
    weakref.finalize(buf, lib().dgb_host_free, p.value)
    a = np.frombuffer(buf, dtype=dt, count=n)
    a[...] = 0
    return a


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
    if len(fields) > 24:  # the CCZ4 set: theta_z4 as variable 24
        check(lib().dgb_synth_fill_var_host(blocks, len(blocks), 24,
                                            fields[24].ctypes.data_as(C.POINTER(C.c_double)),
                                            seed, noise, nthreads), "dgb_synth_fill_var_host")


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

    def ccz4_rhs(self, params, rhs_ptrs, u_ptrs, precision=PREC_FP64, stream=0):
        """CCZ4 right-hand side (25 device arrays each) over the plan's blocks."""
        r, k1 = ptr_array(rhs_ptrs)
        u, k2 = ptr_array(u_ptrs)
        check(lib().dgb_ccz4_rhs(self.h, C.byref(params), r, u, precision, C.c_void_p(stream)),
              "dgb_ccz4_rhs")

    def ccz4_rhs_host(self, params, rhs_arrays, u_arrays, precision=PREC_FP64):
        """CCZ4 right-hand side on 25 host (numpy) arrays each way."""
        r, k1 = host_ptrs(rhs_arrays)
        u, k2 = host_ptrs(u_arrays)
        check(lib().dgb_ccz4_rhs_host(self.h, C.byref(params), r, u, precision),
              "dgb_ccz4_rhs_host")

    def physical_constraints_host(self, cons_arrays, u_arrays):
        """The constraint diagnostics on host (numpy) arrays: 6 out, 24 in."""
        c, k1 = host_ptrs(cons_arrays)
        u, k2 = host_ptrs(u_arrays)
        check(lib().dgb_physical_constraints_host(self.h, c, u),
              "dgb_physical_constraints_host")

    def physical_constraints(self, cons_ptrs, u_ptrs, stream=0):
        """ham, mom0-2, psi4_real, psi4_img at every block interior point."""
        c, k1 = ptr_array(cons_ptrs)
        u, k2 = ptr_array(u_ptrs)
        check(lib().dgb_physical_constraints(self.h, c, u, C.c_void_p(stream)),
              "dgb_physical_constraints")

    def autotune(self, rhs_ptrs, u_ptrs, precision=PREC_FP64, stream=0):
        r, k1 = ptr_array(rhs_ptrs)
        u, k2 = ptr_array(u_ptrs)
        check(lib().dgb_plan_autotune(self.h, r, u, precision, C.c_void_p(stream)),
              "dgb_plan_autotune")

    def tile(self, precision=PREC_FP64):
        t = (C.c_uint32 * 3)()
        check(lib().dgb_plan_tile(self.h, precision, t), "dgb_plan_tile")
        return tuple(t)

    def class_tiles(self, precision=PREC_FP64):
        """The autotuner's per-class caps: list of ((sx, sy, sz), face, (cx, cy, cz))."""
        n = C.c_size_t(0)
        check(lib().dgb_plan_class_tiles(self.h, precision, None, 0, C.byref(n)),
              "dgb_plan_class_tiles")
        rows = (C.c_uint32 * (7 * max(1, n.value)))()
        check(lib().dgb_plan_class_tiles(self.h, precision, rows, n.value, C.byref(n)),
              "dgb_plan_class_tiles")
        return [((rows[7 * i], rows[7 * i + 1], rows[7 * i + 2]), rows[7 * i + 3],
                 (rows[7 * i + 4], rows[7 * i + 5], rows[7 * i + 6])) for i in range(n.value)]

    def set_tile_variant(self, variant, precision=PREC_FP64):
        check(lib().dgb_plan_set_tile_variant(self.h, precision, variant),
              "dgb_plan_set_tile_variant")

    def synth_fill_device(self, u_ptrs, seed, noise=1e-6, stream=0):
        u, k = ptr_array(u_ptrs)
        check(lib().dgb_synth_fill_device(self.h, u, seed, noise, C.c_void_p(stream)),
              "dgb_synth_fill_device")
        if len(u_ptrs) > 24:  # the CCZ4 set: theta_z4 as variable 24
            check(lib().dgb_synth_fill_var_device(self.h, 24, C.c_void_p(int(u_ptrs[24])), seed,
                                                  noise, C.c_void_p(stream)),
                  "dgb_synth_fill_var_device")

    def close(self):
        if self.h:
            lib().dgb_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def constraint_l2(field_ptrs, ndof, mask_ptr=None, threshold=0.0, stream=0):
    """Masked RMS of zipped device vectors (computeConstraintL2Norm)."""
    out = (C.c_double * len(field_ptrs))()
    f, keep = ptr_array(field_ptrs)
    check(lib().dgb_constraint_l2(f, len(field_ptrs), mask_ptr, threshold,
                                  ndof, out, C.c_void_p(stream)), "dgb_constraint_l2")
    return list(out)


CONSTRAINT_NAMES = ("ham", "mom0", "mom1", "mom2", "psi4_real", "psi4_img")

# bssn:: defaults of the constraint report's mask (BSSN_GR/src/parameters.cpp:157-158)
EXTRACTION_VAR_ID = 0  # alpha
EXTRACTION_TOL = 0.3


def constraint_report(plan, uz, state_ptrs, unzipped_ptrs, cons_unzipped_ptrs, cons_ptrs, ndof,
                      threshold=EXTRACTION_TOL, stream=0):
    """The solver's constraint output (BSSN_GR/src/bssnCtx.cpp:332-365) on
    device buffers: unzip the 24 zipped state vectors, physical_constraints
    on every block, zip the 6 outputs into cons_ptrs, and return the masked
    L2 of ham, mom0-2 (mask: the alpha vector >= threshold)."""
    uz.unzip(state_ptrs, unzipped_ptrs, stream)
    plan.physical_constraints(cons_unzipped_ptrs, unzipped_ptrs, stream)
    uz.zip(cons_unzipped_ptrs, cons_ptrs, stream)
    return constraint_l2(cons_ptrs[:4], ndof, state_ptrs[EXTRACTION_VAR_ID], threshold, stream)


def rk4_stage(stage, dst_ptrs, prev_ptrs, k_ptrs, nnodes, dt, chi_floor=1e-4, stream=0):
    d, k1 = ptr_array(dst_ptrs)
    p, k2 = ptr_array(prev_ptrs)
    kk, k3 = ptr_array(k_ptrs)
    check(lib().dgb_rk4_stage(stage, d, p, kk, nnodes, dt, chi_floor, C.c_void_p(stream)),
          "dgb_rk4_stage")


# ----------------------------------------------------------------------------- mesh
class MeshParams(C.Structure):
    _fields_ = [("domain_min", C.c_double * 3), ("domain_max", C.c_double * 3),
                ("max_level", C.c_int), ("min_level", C.c_int), ("ele_order", C.c_int),
                ("num_punctures", C.c_int), ("puncture", (C.c_double * 3) * 4),
                ("fine_radius", C.c_double), ("max_block_refine", C.c_int),
                ("octree_depth", C.c_int)]


def mesh_params(max_level=10, min_level=4, fine_radius=1.0, domain=32.0, max_block_refine=-1,
                punctures=((1.0, 0.0, 0.00123), (-1.0, 0.0, 0.00123)), octree_depth=0):
    """Two-puncture octree on [-domain, domain]^3 (Brill-Lindquist masses at
    (+-1, 0, 0.00123))."""
    p = MeshParams()
    p.domain_min[:] = [-domain] * 3
    p.domain_max[:] = [domain] * 3
    p.max_level, p.min_level, p.ele_order = max_level, min_level, 6
    p.num_punctures = len(punctures)
    for i, c in enumerate(punctures):
        p.puncture[i][:] = list(c)
    p.fine_radius = fine_radius
    p.max_block_refine = max_block_refine
    p.octree_depth = octree_depth
    return p


def hilbert_tables():
    """The element order's curve: (order[state, i], next[state, child])."""
    n = C.c_int()
    check(lib().dgb_mesh_hilbert_tables(None, None, C.byref(n)), "dgb_mesh_hilbert_tables")
    order = np.zeros((n.value, 8), dtype=np.uint8)
    nxt = np.zeros((n.value, 8), dtype=np.uint8)
    check(lib().dgb_mesh_hilbert_tables(order.ctypes.data, nxt.ctypes.data, C.byref(n)),
          "dgb_mesh_hilbert_tables")
    return order, nxt


def block_node(b, params):
    """(anchor of the block's node in units of the finest level, node level,
    regular-grid level) of a block descriptor of a mesh made with params."""
    D = params.max_level
    L = params.domain_max[0] - params.domain_min[0]
    h = (b.ptmax[0] - b.ptmin[0]) / (b.sz[0] - 1)
    reg = D - int(round(np.log2(h * (6 << D) / L)))
    k = int(round(np.log2((b.sz[0] - 7) // 6)))
    anchor = tuple(int(round((b.ptmin[a] + 3 * h - params.domain_min[a]) / (L / (1 << D))))
                   for a in range(3))
    return anchor, reg - k, reg


class Mesh:
    """Host octree mesh and its unzip / zip operators (numpy arrays)."""

    def __init__(self, params):
        self.params = params
        h = C.c_void_p()
        check(lib().dgb_mesh_create(C.byref(params), C.byref(h)), "dgb_mesh_create")
        self.h = h
        s = (C.c_uint64 * 7)()
        check(lib().dgb_mesh_sizes(h, s), "dgb_mesh_sizes")
        (self.num_leaves, self.ndof, self.nblocks, self.nunzipped, self.ninterp,
         self.nsrc, self.nlevels) = [int(x) for x in s]
        self.blocks = (BlockDesc * self.nblocks)()
        check(lib().dgb_mesh_blocks(h, self.blocks), "dgb_mesh_blocks")

    def dof_coords(self):
        xyz = np.zeros((self.ndof, 3))
        check(lib().dgb_mesh_dof_coords(self.h, xyz.ctypes.data), "dgb_mesh_dof_coords")
        return xyz

    def leaves(self):
        lev = np.zeros(self.num_leaves, dtype=np.uint8)
        anc = np.zeros((self.num_leaves, 3), dtype=np.uint32)
        check(lib().dgb_mesh_leaf_levels(self.h, lev.ctypes.data, anc.ctypes.data),
              "dgb_mesh_leaf_levels")
        return lev, anc

    def block_levels(self):
        """Per block: (anchor in units of the finest level, node level, regular-grid
        level), from its descriptor and the mesh's finest level."""
        return [block_node(b, self.params) for b in self.blocks]

    def leaf_patches(self):
        """Per leaf: patch_base, block_side, boundary, corner (n x 3), hx."""
        n = self.num_leaves
        pb = np.zeros(n, dtype=np.uint64)
        bs = np.zeros(n, dtype=np.uint32)
        bd = np.zeros(n, dtype=np.uint8)
        cr = np.zeros((n, 3))
        hx = np.zeros(n)
        check(lib().dgb_mesh_leaf_patches(self.h, pb.ctypes.data, bs.ctypes.data, bd.ctypes.data,
                                          cr.ctypes.data, hx.ctypes.data),
              "dgb_mesh_leaf_patches")
        return {"patch_base": pb, "block_side": bs, "boundary": bd, "corner": cr, "hx": hx}

    def operator(self):
        cp = np.zeros(self.nunzipped, dtype=np.uint32)
        idst = np.zeros(self.ninterp, dtype=np.uint64)
        iref = np.zeros(self.ninterp, dtype=np.uint64)
        srefs = np.zeros(self.nsrc * 343, dtype=np.uint64)
        lptr = np.zeros(self.nlevels + 1, dtype=np.uint64)
        zs = np.zeros(self.ndof, dtype=np.uint64)
        check(lib().dgb_mesh_unzip_operator(self.h, cp.ctypes.data, idst.ctypes.data,
                                            iref.ctypes.data, srefs.ctypes.data, lptr.ctypes.data,
                                            zs.ctypes.data), "dgb_mesh_unzip_operator")
        return {"copy_src": cp, "interp_dst": idst, "interp_ref": iref, "src_refs": srefs,
                "level_ptr": lptr, "zip_src": zs}

    def close(self):
        if self.h:
            lib().dgb_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SENTINEL = 0xFFFFFFFF

# ----------------------------------------------------------------------------- remesh indicator
OCT_NO_CHANGE, OCT_SPLIT, OCT_COARSE, OCT_INVALID = 0, 1, 2, 255
WAVELET_MAX_VARS = 32


def wavelet_tol_radial(corner, tol_min, tol_max=None, r0=0.0, r1=1.0, use_function=False):
    """Per-leaf wavelet tolerance (bssn::computeWTol's radial ramp)."""
    corner = np.ascontiguousarray(corner, dtype=np.float64).reshape(-1, 3)
    tol = np.zeros(len(corner))
    check(lib().dgb_wavelet_tol_radial(corner.ctypes.data, len(corner), tol_min,
                                       tol_min if tol_max is None else tol_max, r0, r1,
                                       1 if use_function else 0, tol.ctypes.data),
          "dgb_wavelet_tol_radial")
    return tol


def remesh_wavelets(unzipped_ptrs, var_ids, unzip_len, nleaves, patch_base_ptr, block_side_ptr,
                    boundary_ptr, tol_ptr, coarse_fac, wmax_ptr, flags_ptr, changed_ptr=None,
                    stream=0):
    """Mesh::isReMeshUnzip's indicator on device arrays (see dgb_remesh_wavelets)."""
    u, keep = ptr_array(unzipped_ptrs)
    vid = (C.c_uint32 * len(var_ids))(*var_ids)
    check(lib().dgb_remesh_wavelets(u, vid, len(var_ids), unzip_len, nleaves,
                                    C.c_void_p(patch_base_ptr), C.c_void_p(block_side_ptr),
                                    C.c_void_p(boundary_ptr), C.c_void_p(tol_ptr), coarse_fac,
                                    C.c_void_p(wmax_ptr), C.c_void_p(flags_ptr),
                                    C.c_void_p(changed_ptr), C.c_void_p(stream)),
          "dgb_remesh_wavelets")


def synth_fill_points(xyz, fields, seed, noise=1e-6, nthreads=0):
    pa, keep = host_ptrs(fields)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    check(lib().dgb_synth_fill_points_host(xyz.ctypes.data, len(xyz), pa, seed, noise, nthreads),
          "dgb_synth_fill_points_host")


class UnzipPlan:
    def __init__(self, op, ndof):
        h = C.c_void_p()
        n = len(op["copy_src"])
        ni = len(op["interp_dst"])
        nsrc = len(op["src_refs"]) // 343
        nlev = max(len(op["level_ptr"]) - 1, 0)
        check(lib().dgb_unzip_plan_create(ndof, n, op["copy_src"].ctypes.data, ni,
                                          op["interp_dst"].ctypes.data,
                                          op["interp_ref"].ctypes.data, nsrc,
                                          op["src_refs"].ctypes.data, nlev,
                                          op["level_ptr"].ctypes.data, op["zip_src"].ctypes.data,
                                          C.byref(h)), "dgb_unzip_plan_create")
        self.h = h

    def unzip(self, zipped_ptrs, unzipped_ptrs, stream=0):
        z, k1 = ptr_array(zipped_ptrs)
        u, k2 = ptr_array(unzipped_ptrs)
        check(lib().dgb_unzip(self.h, z, u, len(zipped_ptrs), C.c_void_p(stream)), "dgb_unzip")

    def zip(self, unzipped_ptrs, zipped_ptrs, stream=0):
        u, k1 = ptr_array(unzipped_ptrs)
        z, k2 = ptr_array(zipped_ptrs)
        check(lib().dgb_zip(self.h, u, z, len(zipped_ptrs), C.c_void_p(stream)), "dgb_zip")

    def close(self):
        if self.h:
            lib().dgb_unzip_plan_destroy(self.h)
            self.h = None


STEP_FUSED_UNZIP = 1


class Stepper:
    def __init__(self, plan, uz, precision=PREC_FP64, fused=False):
        h = C.c_void_p()
        check(lib().dgb_stepper_create_ex(plan.h, uz.h, precision,
                                          STEP_FUSED_UNZIP if fused else 0, C.byref(h)),
              "dgb_stepper_create_ex")
        self.h = h
        self._keep = (plan, uz)

    @property
    def device_bytes(self):
        b = C.c_uint64()
        check(lib().dgb_stepper_device_bytes(self.h, C.byref(b)), "dgb_stepper_device_bytes")
        return b.value

    def step(self, state_ptrs, dt, nsteps=1, chi_floor=1e-4, stream=0):
        s, k = ptr_array(state_ptrs)
        check(lib().dgb_rk4_step(self.h, s, dt, chi_floor, nsteps, C.c_void_p(stream)),
              "dgb_rk4_step")

    def close(self):
        if self.h:
            lib().dgb_stepper_destroy(self.h)
            self.h = None
