"""The oracle's 4th-order BSSN right-hand side (the BSSN_GR solver's own
binding, BSSN_GR/include/rhs.h:23-37: deriv42 first and second derivatives,
upwinded deriv42adv advection, ko_deriv42) against the reference: the
golden vectors of tests/golden/bssn42_reference.npz and, where the reference
tree is present, the reference harness oracle/ref_bssnrhs42.cpp live.  Bar:
1e-13 per-field normwise; the upwinded stencils bit for bit."""
import hashlib
import os

import numpy as np
import pytest

from workloads import SEED1, interior_mask

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bssn42_reference.npz")


def normwise(a, b):
    return max(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300) for x, y in zip(a, b))


def golden_case(dgb, g):
    allb = dgb.synth_blocks(1)
    rows, off = [], 0
    for i, f in g["picks"]:
        b = allb[int(i)]
        rows.append((off, tuple(b.sz), int(f), tuple(b.ptmin), tuple(b.ptmax)))
        off += b.sz[0] * b.sz[1] * b.sz[2]
    blocks = dgb.blocks_array(rows)
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, u, int(g["seed"]), 1e-6)
    for d in range(3):
        u[6 + d] += 0.3 * np.sin(np.arange(n) * (0.37 + d))
    return blocks, u


def test_golden_inputs_regenerate(dgb):
    g = np.load(GOLDEN)
    _, u = golden_case(dgb, g)
    h = hashlib.sha256()
    for a in u:
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(g["input_sha256"])


def test_oracle42_matches_golden(dgb, oracle):
    g = np.load(GOLDEN)
    blocks, u = golden_case(dgb, g)
    n = len(u[0])
    prm = dgb.params_vector(dgb.default_params(float(g["sigma"])))
    r = [np.zeros(n) for _ in range(24)]
    for b in blocks:
        assert oracle.bssnrhs_block(r, u, b, prm, order=4) == 0
    mask = interior_mask(blocks, n)
    assert normwise([x[mask] for x in r], list(g["rhs"])) <= 1e-13


def test_oracle42_differs_from_6th_order(dgb, oracle):
    """The order switch changes the discretisation (guards against a silent
    fall-back to the 6th-order path)."""
    g = np.load(GOLDEN)
    blocks, u = golden_case(dgb, g)
    n = len(u[0])
    prm = dgb.params_vector(dgb.default_params(0.1))
    r4 = [np.zeros(n) for _ in range(24)]
    r6 = [np.zeros(n) for _ in range(24)]
    assert oracle.bssnrhs_blocks(r4, u, blocks, prm, 1, order=4) == 0
    assert oracle.bssnrhs_blocks(r6, u, blocks, prm, 1, order=6) == 0
    mask = interior_mask(blocks, n)
    assert normwise([x[mask] for x in r4], [x[mask] for x in r6]) > 1e-6


def test_oracle42_matches_reference_live(dgb, oracle, reference):
    from test_oracle import boundary_blocks
    from workloads import repack
    cases = [repack(dgb, dgb.synth_blocks(2, 20261205), [0, 1, 2, 3, 5, 8, 13]),
             boundary_blocks(dgb)]
    prm = dgb.params_vector(dgb.default_params(0.1))
    for blocks in cases:
        n = dgb.unzipped_size(blocks)
        u = [np.zeros(n) for _ in range(24)]
        oracle.synth_fill(blocks, u, SEED1, 1e-6)
        for d in range(3):
            u[6 + d] += 0.3 * np.sin(np.arange(n) * (0.37 + d))
        r1 = [np.zeros(n) for _ in range(24)]
        r2 = [np.zeros(n) for _ in range(24)]
        for b in blocks:
            assert oracle.bssnrhs_block(r1, u, b, prm, order=4) == 0
            assert reference.bssnrhs(r2, u, b, prm, order=4) == 0
        mask = interior_mask(blocks, n)
        assert normwise([x[mask] for x in r1], [x[mask] for x in r2]) <= 1e-13


def test_upwind_stencil_bit_exact_live(oracle, reference):
    """deriv42adv of the BSSN_GR file, every flag combination, both shift signs."""
    import ctypes as C
    rng = np.random.default_rng(2)
    u3 = rng.normal(size=(17, 19, 21))
    beta = rng.normal(size=u3.shape)
    L = oracle.L
    L.orc_bssn_adv42.restype = None
    L.orc_bssn_adv42.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                 C.c_void_p, C.c_uint]
    sz = (C.c_uint * 3)(21, 19, 17)
    for bflag in range(64):
        for d in range(3):
            a = np.zeros_like(u3)
            L.orc_bssn_adv42(d, a.ctypes.data, u3.ctypes.data, 0.1, sz, beta.ctypes.data, bflag)
            b = reference.adv42(d, u3, 0.1, beta, bflag)
            inner = np.zeros_like(u3, dtype=bool)
            inner[3:-3, 3:-3, 3:-3] = True
            assert np.array_equal(a[inner], b[inner]), (d, bflag)
