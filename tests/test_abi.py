"""CPU tests of the C ABI library: it loads, exports every entry point the
public header declares, and its host-side logic (synthetic workloads, the
integer-pipe exact products, argument checking) behaves.  No GPU compute."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from workloads import SEED2, repack, sample_uneven

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "dendro_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dgb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol(dgb):
    import ctypes as C
    L = C.CDLL(dgb.LIB_PATH)
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding declares every one of them
    assert set(names) <= set(dgb.EXPORTED), set(names) - set(dgb.EXPORTED)


def test_version(dgb):
    assert dgb.lib().dgb_version() >= 1


def test_exact_mul_host_bit_identical(dgb):
    assert dgb.selftest_exact_mul(0, 1 << 21, seed=9) == 0


def test_synth_block_lists(dgb):
    b1 = dgb.synth_blocks(1)
    assert len(b1) == 512
    assert all(tuple(b.sz) == (13, 13, 13) for b in b1)
    h = [(b.ptmax[0] - b.ptmin[0]) / 12 for b in b1]
    assert np.allclose(h, 0.05)
    b2 = dgb.synth_blocks(2, SEED2)
    assert len(b2) == 20000
    sides = np.array([b.sz[0] for b in b2])
    assert [(sides == s).sum() for s in (13, 19, 31, 61)] == [14000, 4000, 1600, 400]
    padded = sum(b.sz[0] ** 3 for b in b2)
    interior = sum((b.sz[0] - 6) ** 3 for b in b2)
    assert padded == 196_652_000 and interior == 105_140_000
    # contiguous layout, blocks inside [-32,32]^3 (owned nodes), levels 4..10
    off = 0
    for b in b2:
        assert b.offset == off
        off += b.sz[0] ** 3
        for a in range(3):
            h = (b.ptmax[a] - b.ptmin[a]) / (b.sz[a] - 1)
            lev = np.log2(64.0 / (6 * h))
            assert abs(lev - round(lev)) < 1e-9 and 4 <= round(lev) <= 10
            assert b.ptmin[a] + 3 * h >= -32 - 1e-9 and b.ptmax[a] - 3 * h <= 32 + 1e-9


def test_synth_fill_deterministic(dgb):
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (2, 1, 0, 0)))
    n = dgb.unzipped_size(blocks)
    a = [np.zeros(n) for _ in range(24)]
    b = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, a, 5, 1e-6, 1)
    dgb.synth_fill_host(blocks, b, 5, 1e-6, 4)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    c = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, c, 6, 1e-6)
    assert not np.array_equal(a[3], c[3])
    # noise amplitude and the Brill-Lindquist floors
    assert np.abs(a[2]).max() <= 1e-6 and np.abs(a[2]).max() > 5e-7
    assert a[1].min() >= 1e-4 - 1e-6 and a[0].max() <= 1.0 + 1e-6


def test_plan_create_needs_init(dgb):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; covered by the GPU tests")
    import ctypes as C
    blocks = dgb.synth_blocks(1)
    h = C.c_void_p()
    st = dgb.lib().dgb_plan_create(blocks, len(blocks), C.byref(dgb.default_params()), C.byref(h))
    assert st == 4  # DGB_ERR_NOT_INIT, not a crash
    assert dgb.lib().dgb_init(0) == 4  # no device here


def test_generated_algebra_up_to_date():
    gen = os.path.join(ROOT, "dendro-5.01_gb300", "codegen", "gen_bssn_algebra.py")
    out = subprocess.run([sys.executable, gen], capture_output=True, text=True, check=True).stdout
    cur = open(os.path.join(ROOT, "dendro-5.01_gb300", "csrc", "bssn_algebra.cuh")).read()
    assert out == cur, "csrc/bssn_algebra.cuh is stale: rerun codegen/gen_bssn_algebra.py"


def test_generated_ccz4_algebra_up_to_date():
    gen = os.path.join(ROOT, "dendro-5.01_gb300", "codegen", "gen_ccz4_algebra.py")
    out = subprocess.run([sys.executable, gen], capture_output=True, text=True, check=True).stdout
    cur = open(os.path.join(ROOT, "dendro-5.01_gb300", "csrc", "ccz4_algebra.cuh")).read()
    assert out == cur, "csrc/ccz4_algebra.cuh is stale: rerun codegen/gen_ccz4_algebra.py"


def test_argument_checks_without_device(dgb):
    """Entry points reject bad arguments with DGB_ERR_INVALID before touching
    the device (no GPU needed)."""
    import ctypes as C
    L = dgb.lib()
    INVALID = 1
    # wavelet indicator: variable count, missing leaf tables, null fields
    u, keep = dgb.ptr_array([0])
    assert L.dgb_remesh_wavelets(u, (C.c_uint32 * 1)(0), 0, 0, 0, None, None, None, None, 0.1,
                                 None, None, None, None) == INVALID
    assert L.dgb_remesh_wavelets(u, (C.c_uint32 * 33)(*range(33)), 33, 0, 0, None, None, None,
                                 None, 0.1, None, None, None, None) == INVALID
    assert L.dgb_remesh_wavelets(u, (C.c_uint32 * 1)(0), 1, 100, 5, None, None, None, None, 0.1,
                                 None, None, None, None) == INVALID
    z = C.c_uint64(0)
    assert L.dgb_remesh_wavelets(u, (C.c_uint32 * 1)(0), 1, 100, 1, C.byref(z), C.byref(z),
                                 C.byref(z), C.byref(z), 0.1, C.byref(z), C.byref(z), None,
                                 None) == INVALID  # field pointer 0
    # tolerance ramp: r1 == r0 is undefined
    corner = np.zeros((2, 3))
    tol = np.zeros(2)
    assert L.dgb_wavelet_tol_radial(corner.ctypes.data, 2, 1e-4, 1e-3, 1.0, 1.0, 1,
                                    tol.ctypes.data) == INVALID
    # null handles and arrays
    assert L.dgb_mesh_leaf_patches(None, None, None, None, None, None) == INVALID
    assert L.dgb_stepper_create_ex(None, None, 0, 0, C.byref(C.c_void_p())) == INVALID
    assert L.dgb_stepper_device_bytes(None, C.byref(z)) == INVALID
    assert L.dgb_plan_class_tiles(None, 0, None, 0, C.byref(C.c_size_t())) == INVALID
    assert L.dgb_bssn_rhs_host(None, None, None, 0) == INVALID
    assert L.dgb_ccz4_rhs_host(None, None, None, None, 0) == INVALID
    assert L.dgb_physical_constraints_host(None, None, None) == INVALID
    # page-locked host memory: sizes, null pointers, foreign pointers
    assert L.dgb_host_alloc(0, C.byref(C.c_void_p())) == INVALID
    assert L.dgb_host_alloc(8, None) == INVALID
    assert L.dgb_host_free(None) == 0
    foreign = np.zeros(4)
    assert L.dgb_host_free(C.c_void_p(foreign.ctypes.data)) == INVALID


def _noalloc_call(dgb, sz=(13, 13, 13), bflag=0, pmin=(0.0, 0.0, 0.0), pmax=(1.2, 1.2, 1.2),
                  prm=None, null_field=False, null_arg=False):
    """dgb_bssnrhs_block_noalloc on placeholder (never dereferenced) pointers:
    every case here is rejected by the entry's argument checks, which run
    before any CUDA call."""
    import ctypes as C
    fake = [C.c_void_p(0x1000 + 8 * v) for v in range(24)]
    if null_field:
        fake[5] = C.c_void_p(0)
    arr = (C.c_void_p * 24)(*fake)
    ptrs = C.cast(arr, dgb.PtrArr)
    prm = prm or dgb.default_params(0.1)
    st = dgb.lib().dgb_bssnrhs_block_noalloc(
        None if null_arg else ptrs, ptrs, 0, (C.c_double * 3)(*pmin), (C.c_double * 3)(*pmax),
        (C.c_uint32 * 3)(*sz), bflag, C.byref(prm), None)
    return st, dgb.lib().dgb_last_error().decode()


@pytest.mark.parametrize("case,status,text", [
    (dict(null_arg=True), 1, "null argument"),
    (dict(null_field=True), 1, "null field pointer"),
    (dict(sz=(6, 13, 13)), 1, "[7, 4096]"),
    (dict(sz=(13, 13, 5000)), 1, "[7, 4096]"),
    (dict(bflag=64), 1, "beyond the six faces"),
    (dict(bflag=1, sz=(11, 13, 13)), 1, "at least 13"),
    (dict(pmax=(1.2, -1.0, 1.2)), 1, "ptmax must exceed ptmin"),
    (dict(sz=(61, 61, 61)), 1, "fixed workspace"),
])
def test_noalloc_argument_checks(dgb, case, status, text):
    st, msg = _noalloc_call(dgb, **case)
    assert st == status and text in msg, (st, msg)


def test_noalloc_refuses_other_bindings(dgb):
    p = dgb.default_params(0.1, fd_order=4)
    st, msg = _noalloc_call(dgb, prm=p)
    assert st == 8 and "6th-order" in msg
    p = dgb.default_params(0.1)
    p.gauge = 1
    st, msg = _noalloc_call(dgb, prm=p)
    assert st == 8 and "gauge" in msg
