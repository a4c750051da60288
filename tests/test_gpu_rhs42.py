"""The CUDA RHS with the BSSN_GR solver's own 4th-order binding
(dgb_bssn_params.fd_order = 4: deriv42, upwinded deriv42adv, ko_deriv42,
BSSN_GR/include/rhs.h:23-37), through the C ABI, against the oracle's
4th-order path (itself pinned to the reference's harness,
tests/test_oracle42.py): FP64 within 1e-12 normwise per field, with a
non-zero shift so that every upwinded form is taken; the device and
host-array entries, interior, uneven and domain-boundary blocks; the
unsupported combinations refused."""
import numpy as np
import pytest

from workloads import SEED1, SEED2, interior_mask, normwise, repack, sample_uneven

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def shifted_fields(dgb, blocks, seed):
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, u, seed, 1e-6)
    for d in range(3):
        u[6 + d] += 0.3 * np.sin(np.arange(n) * (0.37 + d))
    return u


def run_device(torch, plan, u, precision=0):
    du = [torch.from_numpy(a).cuda() for a in u]
    n = len(u[0])
    dr = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") for _ in range(24)]
    plan.rhs_device([t.data_ptr() for t in dr], [t.data_ptr() for t in du], precision)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in dr]


def oracle42(dgb, oracle, blocks, u, sigma):
    n = len(u[0])
    r = [np.zeros(n) for _ in range(24)]
    prm = dgb.params_vector(dgb.default_params(sigma))
    assert oracle.bssnrhs_blocks(r, u, blocks, prm, 0, order=4) == 0
    return r


@pytest.mark.parametrize("case", ["uniform512", "uneven_sample", "boundary"])
def test_rhs42_matches_oracle(dgb, gpu, oracle, case):
    torch = gpu
    if case == "uniform512":
        blocks, seed = dgb.synth_blocks(1), SEED1
    elif case == "uneven_sample":
        allb = dgb.synth_blocks(2, SEED2)
        blocks, seed = repack(dgb, allb, sample_uneven(allb)), SEED2
    else:
        from test_oracle import boundary_blocks
        blocks, seed = boundary_blocks(dgb), SEED1
    u = shifted_fields(dgb, blocks, seed)
    if case == "boundary":
        from test_oracle import poison_outside
        poison_outside(blocks, u)
    plan = dgb.Plan(blocks, dgb.default_params(0.1, fd_order=4))
    got = run_device(torch, plan, u)
    want = oracle42(dgb, oracle, blocks, u, 0.1)
    mask = interior_mask(blocks, len(u[0]))
    err = normwise(got, want, mask)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.VAR_NAMES, err))
    for v in range(24):  # padding untouched
        assert np.all(got[v][~mask] == 7.0)
    # not the 6th-order answer
    plan6 = dgb.Plan(blocks, dgb.default_params(0.1))
    got6 = run_device(torch, plan6, u)
    assert np.max(normwise(got6, want, mask)) > 1e-6
    plan.close()
    plan6.close()


def test_rhs42_host_entry_same_bits(dgb, gpu, monkeypatch):
    """dgb_bssn_rhs_host (chunked pipeline, several chunks) gives the device
    entry's bits at fd_order 4."""
    torch = gpu
    monkeypatch.setenv("DGB_HOST_CHUNK_PTS", "30000")
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (6, 3, 2, 0)))
    u = shifted_fields(dgb, blocks, SEED2)
    plan = dgb.Plan(blocks, dgb.default_params(0.1, fd_order=4))
    dev = run_device(torch, plan, u)
    for rep in range(2):
        host = [np.full(len(u[0]), 7.0) for _ in range(24)]
        plan.rhs_host(host, u)
        for v in range(24):
            assert np.array_equal(dev[v], host[v]), (rep, v)
    plan.close()


def test_rhs42_refusals(dgb, gpu):
    """Mixed precision at fd_order 4, other gauges, unknown orders."""
    blocks = dgb.synth_blocks(1)
    plan = dgb.Plan(blocks, dgb.default_params(0.1, fd_order=4))
    n = plan.unzipped
    u = [np.zeros(n) for _ in range(24)]
    r = [np.zeros(n) for _ in range(24)]
    with pytest.raises(dgb.DgbError, match="UNSUPPORTED"):
        plan.rhs_host(r, u, dgb.PREC_MIXED)
    plan.close()
    for gauge in (1, 2, 3):
        p = dgb.default_params(0.1)
        p.gauge = gauge
        with pytest.raises(dgb.DgbError, match="UNSUPPORTED"):
            dgb.Plan(blocks, p)
    p = dgb.default_params(0.1)
    p.fd_order = 8
    with pytest.raises(dgb.DgbError, match="INVALID"):
        dgb.Plan(blocks, p)
