"""The allocation-free entry point dgb_bssnrhs_block_noalloc, for callers that
cannot call cudaMalloc (a pre-reserved device-memory pool, a runtime that owns
the allocator, or a step loop that must not synchronise the device): through
the C ABI, on two calls in a row, it gives the same right-hand side as the
plan-based entry point dgb_bssn_rhs, within the FP64 tolerance of the other
parity tests, on interior and domain-boundary blocks (its argument checks,
which run before any CUDA call, are tested without a device in
tests/test_abi.py).  Collected last (file name) so that a stop-at-first-failure run has already
run every other test."""
import ctypes as C

import numpy as np
import pytest

from workloads import SEED2, host_fields, interior_mask, normwise, repack, sample_uneven

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _noalloc(dgb, dr, du, b, prm):
    r, k1 = dgb.ptr_array([t.data_ptr() for t in dr])
    u, k2 = dgb.ptr_array([t.data_ptr() for t in du])
    pmin = (C.c_double * 3)(*b.ptmin)
    pmax = (C.c_double * 3)(*b.ptmax)
    sz = (C.c_uint32 * 3)(*b.sz)
    return dgb.lib().dgb_bssnrhs_block_noalloc(r, u, b.offset, pmin, pmax, sz, b.bflag,
                                                C.byref(prm), None)


def test_noalloc_matches_plan_entry_twice(dgb, gpu):
    torch = gpu
    allb = dgb.synth_blocks(2, SEED2)
    # a 13^3 and a 19^3 block, then a 31^3 block on the second call
    sets = [repack(dgb, allb, sample_uneven(allb, (1, 1, 0, 0))),
            repack(dgb, allb, sample_uneven(allb, (0, 0, 1, 0)))]
    prm = dgb.default_params(0.1)
    for blocks in sets:
        u = host_fields(dgb, blocks, SEED2)
        n = len(u[0])
        du = [torch.from_numpy(a).cuda() for a in u]
        want_d = [torch.full((n,), 3.0, dtype=torch.float64, device="cuda") for _ in range(24)]
        plan = dgb.Plan(blocks, prm)
        plan.rhs_device([t.data_ptr() for t in want_d], [t.data_ptr() for t in du])
        got_d = [torch.full((n,), 3.0, dtype=torch.float64, device="cuda") for _ in range(24)]
        for b in blocks:
            dgb.check(_noalloc(dgb, got_d, du, b, prm), "dgb_bssnrhs_block_noalloc")
        torch.cuda.synchronize()
        got = [t.cpu().numpy() for t in got_d]
        want = [t.cpu().numpy() for t in want_d]
        mask = interior_mask(blocks, n)
        err = normwise(got, want, mask)
        assert np.all(err <= FP64_TOL), dict(zip(dgb.VAR_NAMES, err))
        for v in range(24):
            assert np.all(got[v][~mask] == 3.0)  # padding untouched
        plan.close()


def test_noalloc_boundary_blocks_match_plan_entry(dgb, gpu):
    """Domain-boundary blocks (one-sided closures and the outgoing-radiation
    condition on every face class), with the padding beyond the flagged faces
    left as NaN as an unzip leaves it: the no-alloc entry gives the plan
    entry's right-hand side."""
    from test_oracle import boundary_blocks, poison_outside
    torch = gpu
    blocks = boundary_blocks(dgb)
    u = host_fields(dgb, blocks, SEED2)
    poison_outside(blocks, u)
    n = len(u[0])
    prm = dgb.default_params(0.1)
    du = [torch.from_numpy(a).cuda() for a in u]
    want_d = [torch.full((n,), 3.0, dtype=torch.float64, device="cuda") for _ in range(24)]
    plan = dgb.Plan(blocks, prm)
    plan.rhs_device([t.data_ptr() for t in want_d], [t.data_ptr() for t in du])
    got_d = [torch.full((n,), 3.0, dtype=torch.float64, device="cuda") for _ in range(24)]
    for b in blocks:
        dgb.check(_noalloc(dgb, got_d, du, b, prm), "dgb_bssnrhs_block_noalloc")
    torch.cuda.synchronize()
    got = [t.cpu().numpy() for t in got_d]
    want = [t.cpu().numpy() for t in want_d]
    mask = interior_mask(blocks, n)
    err = normwise(got, want, mask)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.VAR_NAMES, err))
    plan.close()
