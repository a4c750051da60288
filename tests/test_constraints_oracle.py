"""CPU tests of the constraint-diagnostics oracle (physical_constraints,
BSSN_GR/src/physcon.cpp:12-96): pinned to the reference's golden vectors
(tests/golden/constraints_reference.npz, made by tests/golden/make_golden.py
from the reference's own compiled sources) and, where the reference tree
exists, to the reference code itself on more blocks and every boundary flag."""
import hashlib
import os

import numpy as np
import pytest

from workloads import SEED2, host_fields, interior_mask, normwise, repack, sample_uneven

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "constraints_reference.npz")
CONS_NAMES = ("ham", "mom0", "mom1", "mom2", "psi4_real", "psi4_img")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def golden_blocks(dgb, g):
    allb = dgb.synth_blocks(1)
    rows, off = [], 0
    for i, f in g["picks"]:
        b = allb[int(i)]
        rows.append((off, tuple(b.sz), int(f), tuple(b.ptmin), tuple(b.ptmax)))
        off += b.sz[0] * b.sz[1] * b.sz[2]
    blocks = dgb.blocks_array(rows)
    return blocks, host_fields(dgb, blocks, int(g["seed"]))


def test_constraint_golden_inputs_regenerate(dgb, golden):
    blocks, u = golden_blocks(dgb, golden)
    h = hashlib.sha256()
    for a in u:
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(golden["input_sha256"])


def test_oracle_constraints_match_golden(dgb, oracle, golden):
    blocks, u = golden_blocks(dgb, golden)
    n = len(u[0])
    c = [np.zeros(n) for _ in range(6)]
    assert oracle.physcon_blocks(c, u, blocks) == 0
    mask = interior_mask(blocks, n)
    got = [x[mask] for x in c]
    want = list(golden["cons"])
    err = normwise(got, want, np.ones(len(got[0]), dtype=bool))
    assert err.max() <= 1e-13, dict(zip(CONS_NAMES, err))


def test_oracle_psi4_axis_guard(dgb, oracle, golden):
    """Psi4 is zero on the z axis, exactly where the reference zeroes it."""
    blocks, u = golden_blocks(dgb, golden)
    n = len(u[0])
    c = [np.zeros(n) for _ in range(6)]
    assert oracle.physcon_blocks(c, u, blocks) == 0
    mask = interior_mask(blocks, n)
    want_zero = golden["cons"][4] == 0.0
    assert want_zero.sum() > 0
    assert np.array_equal(c[4][mask] == 0.0, want_zero)
    assert np.array_equal(c[5][mask] == 0.0, golden["cons"][5] == 0.0)


@pytest.mark.parametrize("kind", ["d1_4", "d2_4"])
def test_oracle_4th_order_stencils_bit_exact(dgb, oracle, golden, kind):
    blocks, u = golden_blocks(dgb, golden)
    sz = tuple(blocks[0].sz)
    chi = u[1][: sz[0] * sz[1] * sz[2]].reshape(sz[2], sz[1], sz[0])
    h = float(golden["stencil_h"])
    for d in range(3):
        got = oracle.stencil(kind, d, chi, h)[3:-3, 3:-3, 3:-3]
        assert np.array_equal(got, golden[f"stencil_{kind}_{d}"]), (kind, d)


@pytest.mark.parametrize("kind", ["d1_4", "d2_4"])
def test_oracle_4th_order_closures_bit_exact(oracle, reference, kind):
    rng = np.random.default_rng(1)
    u3 = rng.normal(size=(17, 19, 21))
    for bflag in range(64):
        for d in range(3):
            a = oracle.stencil(kind, d, u3, 0.1, bflag)
            b = reference.stencil(kind, d, u3, 0.1, bflag)
            assert np.array_equal(a, b), (kind, d, bflag)


def test_oracle_constraints_match_reference_code(dgb, oracle, reference):
    """Live pin: a sample of every size class of the uneven batch."""
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (4, 2, 1, 0)))
    u = host_fields(dgb, blocks, SEED2)
    n = len(u[0])
    c1 = [np.zeros(n) for _ in range(6)]
    c2 = [np.zeros(n) for _ in range(6)]
    assert oracle.physcon_blocks(c1, u, blocks) == 0
    for b in blocks:
        assert reference.physical_constraints(c2, u, b) == 0
    err = normwise(c1, c2, interior_mask(blocks, n))
    assert err.max() <= 1e-13, dict(zip(CONS_NAMES, err))
