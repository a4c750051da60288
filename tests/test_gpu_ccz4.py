"""Parity of the CUDA CCZ4 right-hand side (through the C ABI) with the CCZ4
oracle and the reference's golden vectors: ccz4rhs (CCZ4_GR/src/rhs.cpp:12-298)
within 1e-12 normwise per field, padding untouched, the boundary condition on
flagged faces, theta_z4 left out of KO."""
import os

import numpy as np
import pytest

from workloads import SEED1, SEED2, interior_mask, normwise, repack, sample_uneven

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ccz4_reference.npz")


def ccz4_fields(dgb, blocks, seed):
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(25)]
    dgb.synth_fill_host(blocks, u, seed, 1e-6)
    return u


def gpu_ccz4(dgb, torch, blocks, u, params, fill=7.0):
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    du = [torch.from_numpy(a).cuda() for a in u]
    n = len(u[0])
    dr = [torch.full((n,), fill, dtype=torch.float64, device="cuda") for _ in range(25)]
    plan.ccz4_rhs(params, [t.data_ptr() for t in dr], [t.data_ptr() for t in du])
    torch.cuda.synchronize()
    out = [t.cpu().numpy() for t in dr]
    plan.close()
    return out


def oracle_ccz4(dgb, oracle, blocks, u, params):
    n = len(u[0])
    r = [np.zeros(n) for _ in range(25)]
    assert oracle.ccz4rhs_blocks(r, u, blocks, dgb.ccz4_params_vector(params)) == 0
    return r


@pytest.mark.parametrize("which", ["uniform512", "uneven_sample"])
def test_ccz4_matches_oracle(dgb, gpu, oracle, which):
    torch = gpu
    if which == "uniform512":
        blocks, seed = dgb.synth_blocks(1), SEED1
    else:
        allb = dgb.synth_blocks(2, SEED2)
        blocks, seed = repack(dgb, allb, sample_uneven(allb)), SEED2
    u = ccz4_fields(dgb, blocks, seed)
    prm = dgb.default_ccz4_params()
    got = gpu_ccz4(dgb, torch, blocks, u, prm)
    want = oracle_ccz4(dgb, oracle, blocks, u, prm)
    mask = interior_mask(blocks, len(u[0]))
    err = normwise(got, want, mask)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.CCZ4_VAR_NAMES, err))
    for v in range(25):
        assert np.all(got[v][~mask] == 7.0)


def face_mask(blocks, n):
    """Interior points minus the boundary layer of each flagged face."""
    m = np.zeros(n, dtype=bool)
    for b in blocks:
        nx, ny, nz = b.sz
        sel = np.zeros((nz, ny, nx), dtype=bool)
        sel[3:nz - 3, 3:ny - 3, 3:nx - 3] = True
        f = b.bflag
        if f & 1: sel[:, :, 3] = False
        if f & 2: sel[:, :, nx - 4] = False
        if f & 4: sel[:, 3, :] = False
        if f & 8: sel[:, ny - 4, :] = False
        if f & 16: sel[3, :, :] = False
        if f & 32: sel[nz - 4, :, :] = False
        m[b.offset + np.flatnonzero(sel.ravel())] = True
    return m


def test_ccz4_matches_reference_golden(dgb, gpu):
    """Against the reference's own outputs (the harness has no ccz4_bcs, so
    the boundary layer of flagged faces is left out of the comparison)."""
    torch = gpu
    g = np.load(GOLDEN)
    allb = dgb.synth_blocks(1)
    rows, off = [], 0
    for i, f in g["picks"]:
        b = allb[int(i)]
        rows.append((off, tuple(b.sz), int(f), tuple(b.ptmin), tuple(b.ptmax)))
        off += b.sz[0] * b.sz[1] * b.sz[2]
    blocks = dgb.blocks_array(rows)
    u = ccz4_fields(dgb, blocks, int(g["seed"]))
    got = gpu_ccz4(dgb, torch, blocks, u, dgb.default_ccz4_params())
    n = len(u[0])
    mask = interior_mask(blocks, n)
    keep = face_mask(blocks, n)[mask]
    err = normwise([x[mask][keep] for x in got], [w[keep] for w in g["rhs"]],
                   np.ones(int(keep.sum()), dtype=bool))
    assert np.all(err <= FP64_TOL), dict(zip(dgb.CCZ4_VAR_NAMES, err))


def test_ccz4_boundary_blocks(dgb, gpu, oracle):
    """Closures and ccz4_bcs on every face class; NaN beyond flagged faces."""
    from test_oracle import boundary_blocks
    torch = gpu
    blocks = boundary_blocks(dgb)
    u = ccz4_fields(dgb, blocks, SEED1)
    for b in blocks:
        nx, ny, nz = b.sz
        for v in range(25):
            a = u[v][b.offset:b.offset + nx * ny * nz].reshape(nz, ny, nx)
            if b.bflag & 1: a[:, :, :3] = np.nan
            if b.bflag & 2: a[:, :, nx - 3:] = np.nan
            if b.bflag & 4: a[:, :3, :] = np.nan
            if b.bflag & 8: a[:, ny - 3:, :] = np.nan
            if b.bflag & 16: a[:3, :, :] = np.nan
            if b.bflag & 32: a[nz - 3:, :, :] = np.nan
    prm = dgb.default_ccz4_params()
    got = gpu_ccz4(dgb, torch, blocks, u, prm)
    want = oracle_ccz4(dgb, oracle, blocks, u, prm)
    mask = interior_mask(blocks, len(u[0]))
    assert all(np.isfinite(x[mask]).all() for x in got)
    err = normwise(got, want, mask)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.CCZ4_VAR_NAMES, err))


def test_ccz4_theta_not_dissipated(dgb, gpu):
    torch = gpu
    blocks = repack(dgb, dgb.synth_blocks(1), [100, 101])
    u = ccz4_fields(dgb, blocks, 5)
    r0 = gpu_ccz4(dgb, torch, blocks, u, dgb.default_ccz4_params(ko_sigma=0.0))
    r1 = gpu_ccz4(dgb, torch, blocks, u, dgb.default_ccz4_params(ko_sigma=0.4))
    assert np.array_equal(r0[24], r1[24])
    assert not np.array_equal(r0[0], r1[0])


MIXED_TOL = 1e-7  # per-field normwise, compensated FP32 stencils vs FP64


@pytest.mark.parametrize("which", ["uniform512", "uneven_sample", "boundary"])
def test_ccz4_mixed_precision(dgb, gpu, oracle, which):
    """FP32 stencils on interior blocks within MIXED_TOL of the FP64 oracle;
    domain-boundary blocks take the FP64 path (1e-12)."""
    from test_oracle import boundary_blocks
    torch = gpu
    if which == "uniform512":
        blocks, seed = dgb.synth_blocks(1), SEED1
    elif which == "uneven_sample":
        allb = dgb.synth_blocks(2, SEED2)
        blocks, seed = repack(dgb, allb, sample_uneven(allb)), SEED2
    else:
        blocks, seed = boundary_blocks(dgb), SEED1
    u = ccz4_fields(dgb, blocks, seed)
    prm = dgb.default_ccz4_params()
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    du = [torch.from_numpy(a).cuda() for a in u]
    n = len(u[0])
    dr = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") for _ in range(25)]
    plan.ccz4_rhs(prm, [t.data_ptr() for t in dr], [t.data_ptr() for t in du], dgb.PREC_MIXED)
    torch.cuda.synchronize()
    got = [t.cpu().numpy() for t in dr]
    plan.close()
    want = oracle_ccz4(dgb, oracle, blocks, u, prm)
    mask = interior_mask(blocks, n)
    err = normwise(got, want, mask)
    assert np.all(err <= MIXED_TOL), dict(zip(dgb.CCZ4_VAR_NAMES, err))
    for v in range(25):
        assert np.all(got[v][~mask] == 7.0)
    flagged = [b for b in blocks if b.bflag != 0]
    if flagged:
        fmask = interior_mask(flagged, n)
        err = normwise(got, want, fmask)
        assert np.all(err <= FP64_TOL), dict(zip(dgb.CCZ4_VAR_NAMES, err))


@pytest.mark.parametrize("precision,pinned", [("fp64", False), ("mixed", False), ("fp64", True)])
def test_ccz4_host_pipeline_many_chunks(dgb, gpu, precision, pinned, monkeypatch):
    """dgb_ccz4_rhs_host over many chunks, block list not in offset order and
    boundary blocks included: the device entry's bits, padding untouched;
    pinned: the fields in dgb_host_alloc memory (uploaded without staging)."""
    torch = gpu
    monkeypatch.setenv("DGB_HOST_CHUNK_PTS", "30000")
    prec = dgb.PREC_MIXED if precision == "mixed" else dgb.PREC_FP64
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (6, 3, 2, 0)))
    rows = [(b.offset, tuple(b.sz), b.bflag, tuple(b.ptmin), tuple(b.ptmax)) for b in blocks]
    rows = [(o, sz, (63 if i % 3 == 0 else 0), pmin, pmax)
            for i, (o, sz, _, pmin, pmax) in enumerate(rows)]
    blocks = dgb.blocks_array(rows)
    shuffled = dgb.blocks_array(rows[::-1])
    u = ccz4_fields(dgb, blocks, SEED2)
    prm = dgb.default_ccz4_params()
    plan = dgb.Plan(shuffled, dgb.default_params(0.1))
    du = [torch.from_numpy(a).cuda() for a in u]
    n = len(u[0])
    dr = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") for _ in range(25)]
    plan.ccz4_rhs(prm, [t.data_ptr() for t in dr], [t.data_ptr() for t in du], prec)
    torch.cuda.synchronize()
    dev = [t.cpu().numpy() for t in dr]
    if pinned:
        pu = [dgb.host_array(n) for _ in range(25)]
        for v in range(25):
            pu[v][:] = u[v]
        u = pu
    for rep in range(4 if pinned else 2):  # pinned: direct x3, then staged upload
        host = [np.full(n, 7.0) for _ in range(25)]
        plan.ccz4_rhs_host(prm, host, u, prec)
        for v in range(25):
            assert np.array_equal(dev[v], host[v]), (rep, dgb.CCZ4_VAR_NAMES[v])
    plan.close()
