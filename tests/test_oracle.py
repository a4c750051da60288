"""CPU tests of the oracle: pinned to the reference's golden vectors
(tests/golden/bssn_reference.npz, made by tests/golden/make_golden.py from
the reference's own compiled sources) and, where the reference tree exists,
to the reference code itself on more blocks."""
import hashlib
import os

import numpy as np
import pytest

from workloads import SEED1, SEED2, host_fields, interior_mask, normwise, repack, sample_uneven

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bssn_reference.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def golden_inputs(dgb, g):
    blocks = repack(dgb, dgb.synth_blocks(1), [int(b) for b in g["rhs_blocks"]])
    u = host_fields(dgb, blocks, int(g["rhs_seed"]))
    return blocks, u


def test_golden_inputs_regenerate(dgb, golden):
    """The seeded generator still produces the inputs the goldens were made from."""
    blocks, u = golden_inputs(dgb, golden)
    h = hashlib.sha256()
    for a in u:
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(golden["rhs_input_sha256"])


def test_oracle_rhs_matches_golden(dgb, oracle, golden):
    blocks, u = golden_inputs(dgb, golden)
    n = len(u[0])
    r = [np.zeros(n) for _ in range(24)]
    prm = dgb.params_vector(dgb.default_params(float(golden["rhs_sigma"])))
    assert oracle.bssnrhs_blocks(r, u, blocks, prm) == 0
    mask = interior_mask(blocks, n)
    got = [x[mask] for x in r]
    want = list(golden["rhs"])
    err = normwise(got, want, np.ones(len(got[0]), dtype=bool))
    assert err.max() <= 1e-13, dict(zip(dgb.VAR_NAMES, err))


@pytest.mark.parametrize("kind", ["d1", "d2", "ko"])
def test_oracle_stencils_bit_exact(dgb, oracle, golden, kind):
    """Same taps, same order, no contraction: bit-identical to the reference."""
    blocks, u = golden_inputs(dgb, golden)
    b0 = blocks[0]
    sz = tuple(b0.sz)
    chi = u[1][: sz[0] * sz[1] * sz[2]].reshape(sz[2], sz[1], sz[0])
    h = float(golden["stencil_h"])
    for d in range(3):
        got = oracle.stencil(kind, d, chi, h)[3:-3, 3:-3, 3:-3]
        assert np.array_equal(got, golden[f"stencil_{kind}_{d}"]), (kind, d)


def test_oracle_enforce_matches_golden(oracle, golden):
    import ctypes as C
    state = [np.ascontiguousarray(x) for x in golden["enforce_in"]]
    out = [x.copy() for x in state]
    arr = (C.c_void_p * 24)(*[a.ctypes.data for a in out])
    pp = C.cast(arr, C.POINTER(C.c_void_p))
    for node in range(len(out[0])):
        oracle.L.orc_enforce_bssn_constraints(pp, node, float(golden["enforce_chi_floor"]))
    want = golden["enforce_out"]
    for v in range(24):
        np.testing.assert_allclose(out[v], want[v], rtol=2e-15, atol=1e-18)


def test_oracle_rk4_stage_formula(oracle):
    """Stage sums of RK_BSSN::performSingleIteration (rkBSSN.cpp:895-905,
    996-1011) on a state the constraint closure leaves unchanged."""
    rng = np.random.default_rng(3)
    n = 257
    prev = [np.zeros(n) for _ in range(24)]
    prev[0][:] = 0.7
    prev[1][:] = 0.5
    for q in (12, 15, 17):
        prev[q][:] = 1.0
    ks = [[np.zeros(n) for _ in range(24)] for _ in range(4)]
    for s in range(4):
        for v in (0, 1, 2, 6, 9):  # fields the closure does not touch
            ks[s][v][:] = rng.normal(0, 1, n)
    dt = 0.01
    U = [0.0, 0.5, 0.5, 1.0]
    Cc = [1 / 6, 1 / 3, 1 / 3, 1 / 6]
    for s in range(4):
        out = [np.zeros(n) for _ in range(24)]
        oracle.rk4_stage(s, out, prev, ks[: s + 1], dt, 1e-4)
        for v in (2, 6, 9):
            if s < 3:
                want = prev[v] + U[s + 1] * dt * ks[s][v]
            else:
                want = prev[v].copy()
                for q in range(4):
                    want = want + Cc[q] * dt * ks[q][v]
            np.testing.assert_array_equal(out[v], want)


def test_oracle_matches_reference_code(dgb, oracle, reference):
    """Live pin on more blocks: all 512 uniform blocks (both punctures inside)
    and a sample of every size class of the uneven batch."""
    for blocks, seed in ((dgb.synth_blocks(1), SEED1),
                         (repack(dgb, dgb.synth_blocks(2, SEED2),
                                 sample_uneven(dgb.synth_blocks(2, SEED2), (4, 2, 1, 0))), SEED2)):
        u = host_fields(dgb, blocks, seed)
        n = len(u[0])
        prm = dgb.params_vector(dgb.default_params(0.1))
        r1 = [np.zeros(n) for _ in range(24)]
        r2 = [np.zeros(n) for _ in range(24)]
        assert oracle.bssnrhs_blocks(r1, u, blocks, prm) == 0
        for b in blocks:
            assert reference.bssnrhs(r2, u, b, prm) == 0
        err = normwise(r1, r2, interior_mask(blocks, n))
        assert err.max() <= 1e-13, dict(zip(dgb.VAR_NAMES, err))


def boundary_blocks(dgb):
    """13^3 blocks of the uniform workload flagged as domain-boundary blocks
    (every face combination class: single faces, edges, corners, opposite
    faces), laid out contiguously."""
    allb = dgb.synth_blocks(1)
    picks = [(0, 1 | 4 | 16), (7, 2), (63, 2 | 8), (511, 2 | 8 | 32), (300, 4), (301, 48),
             (302, 3), (292, 0)]
    rows, off = [], 0
    for i, f in picks:
        b = allb[i]
        rows.append((off, tuple(b.sz), f, tuple(b.ptmin), tuple(b.ptmax)))
        off += 13 ** 3
    return dgb.blocks_array(rows)


def poison_outside(blocks, u):
    """NaN in the padding beyond each flagged face: a mesh leaves it unfilled."""
    for b in blocks:
        nx, ny, nz = b.sz
        for v in range(24):
            a = u[v][b.offset:b.offset + nx * ny * nz].reshape(nz, ny, nx)
            if b.bflag & 1: a[:, :, :3] = np.nan
            if b.bflag & 2: a[:, :, nx - 3:] = np.nan
            if b.bflag & 4: a[:, :3, :] = np.nan
            if b.bflag & 8: a[:, ny - 3:, :] = np.nan
            if b.bflag & 16: a[:3, :, :] = np.nan
            if b.bflag & 32: a[nz - 3:, :, :] = np.nan


@pytest.mark.parametrize("kind", ["d1", "d2", "ko"])
def test_oracle_boundary_closures_bit_exact(oracle, reference, kind):
    """One-sided closures for every flag combination equal the reference's."""
    rng = np.random.default_rng(0)
    u3 = rng.normal(size=(17, 19, 21))
    for bflag in range(64):
        for d in range(3):
            a = oracle.stencil(kind, d, u3, 0.1, bflag)
            b = reference.stencil(kind, d, u3, 0.1, bflag)
            assert np.array_equal(a, b), (kind, d, bflag)


def test_oracle_boundary_rhs_matches_reference(dgb, oracle, reference):
    """Boundary blocks: closures in the derivatives, the mixed compositions,
    the outgoing-radiation condition bssn_bcs (the reference's own function,
    BSSN_GR/src/rhs.cpp:838-982) and KO agree with the reference harness."""
    blocks = boundary_blocks(dgb)
    u = host_fields(dgb, blocks, SEED1)
    prm = dgb.params_vector(dgb.default_params(0.1))
    n = len(u[0])
    r1 = [np.zeros(n) for _ in range(24)]
    r2 = [np.zeros(n) for _ in range(24)]
    for b in blocks:
        assert oracle.bssnrhs_block(r1, u, b, prm) == 0
        assert reference.bssnrhs(r2, u, b, prm) == 0
    err = normwise(r1, r2, interior_mask(blocks, n))
    assert err.max() <= 1e-13, dict(zip(dgb.VAR_NAMES, err))


def test_oracle_boundary_ignores_unfilled_padding(dgb, oracle):
    blocks = boundary_blocks(dgb)
    u = host_fields(dgb, blocks, SEED1)
    poison_outside(blocks, u)
    prm = dgb.params_vector(dgb.default_params(0.1))
    n = len(u[0])
    r = [np.zeros(n) for _ in range(24)]
    assert oracle.bssnrhs_blocks(r, u, blocks, prm) == 0
    mask = interior_mask(blocks, n)
    assert all(np.isfinite(x[mask]).all() for x in r)
