"""Parity of the CUDA RHS (through the C ABI) with the oracle: FP64 within
1e-12 normwise per field, the reference test beds' metric
(BSSN_GR/cuda_gr/src/gpuTestBed.cpp:408-432)."""
import numpy as np
import pytest

from workloads import SEED1, SEED2, host_fields, interior_mask, normwise, repack, sample_uneven

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_RHS_TOL = 1e-7  # per-field normwise, compensated FP32 stencils vs FP64


def device_fields(torch, arrays):
    return [torch.from_numpy(a).cuda() for a in arrays]


def run_device(dgb, torch, plan, u_host, precision=0, rhs_init=None):
    du = device_fields(torch, u_host)
    n = len(u_host[0])
    dr = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") if rhs_init is None
          else torch.from_numpy(rhs_init[v]).cuda() for v in range(24)]
    plan.rhs_device([t.data_ptr() for t in dr], [t.data_ptr() for t in du], precision)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in dr]


def oracle_rhs(dgb, oracle, blocks, u, sigma):
    n = len(u[0])
    r = [np.zeros(n) for _ in range(24)]
    assert oracle.bssnrhs_blocks(r, u, blocks, dgb.params_vector(dgb.default_params(sigma))) == 0
    return r


@pytest.mark.parametrize("variant_blocks", ["uniform512", "uneven_sample"])
def test_rhs_fp64_matches_oracle(dgb, gpu, oracle, variant_blocks):
    torch = gpu
    if variant_blocks == "uniform512":
        blocks = dgb.synth_blocks(1)
        seed, sigma = SEED1, 0.1
    else:
        allb = dgb.synth_blocks(2, SEED2)
        blocks = repack(dgb, allb, sample_uneven(allb))
        seed, sigma = SEED2, 0.1
    u = host_fields(dgb, blocks, seed)
    plan = dgb.Plan(blocks, dgb.default_params(sigma))
    got = run_device(dgb, torch, plan, u)
    want = oracle_rhs(dgb, oracle, blocks, u, sigma)
    mask = interior_mask(blocks, len(u[0]))
    err = normwise(got, want, mask)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.VAR_NAMES, err))
    # padding untouched (rhs.cpp writes interior points only)
    for v in range(24):
        assert np.all(got[v][~mask] == 7.0)


def test_rhs_all_tile_variants_agree(dgb, gpu, oracle):
    """Every compiled tile shape gives the oracle's answer (autotuner safety)."""
    torch = gpu
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (3, 2, 1, 1)))
    u = host_fields(dgb, blocks, SEED2)
    want = oracle_rhs(dgb, oracle, blocks, u, 0.1)
    mask = interior_mask(blocks, len(u[0]))
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    for variant in range(dgb.lib().dgb_num_tile_variants()):
        plan.set_tile_variant(variant)
        got = run_device(dgb, torch, plan, u)
        err = normwise(got, want, mask)
        assert np.all(err <= FP64_TOL), (variant, err.max())
    du = device_fields(torch, u)
    dr = [torch.zeros_like(du[0]) for _ in range(24)]
    plan.autotune([t.data_ptr() for t in dr], [t.data_ptr() for t in du], 0)
    got = run_device(dgb, torch, plan, u)
    assert np.all(normwise(got, want, mask) <= FP64_TOL)
    # one tile cap per block-size class, within the chosen variant's tile
    ct = plan.class_tiles(0)
    assert len(ct) == len({tuple(b.sz) + (b.bflag != 0,) for b in blocks})
    tmax = plan.tile(0)
    for sz, face, cap in ct:
        assert all(1 <= c <= m for c, m in zip(cap, tmax)), (sz, cap, tmax)
    # the host pipeline's chunk plans take the tuned schedule: same bits
    host = [np.zeros(len(u[0])) for _ in range(24)]
    plan.rhs_host(host, u)
    for v in range(24):
        assert np.array_equal(host[v][mask], got[v][mask])


def test_rhs_host_entry_matches_device(dgb, gpu):
    torch = gpu
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (4, 2, 1, 0)))
    u = host_fields(dgb, blocks, SEED2)
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    dev = run_device(dgb, torch, plan, u, rhs_init=[np.full(len(u[0]), 7.0)] * 24)
    host = [np.full(len(u[0]), 7.0) for _ in range(24)]
    plan.rhs_host(host, u)
    for v in range(24):
        assert np.array_equal(dev[v], host[v])


@pytest.mark.parametrize("precision", [0, 1])
def test_rhs_host_pipeline_many_chunks(dgb, gpu, precision, monkeypatch):
    """The host-array entry as a pipeline over many chunks, with the block
    list not in offset order: the same bits as the device entry, and the
    caller's rhs padding untouched."""
    torch = gpu
    monkeypatch.setenv("DGB_HOST_CHUNK_PTS", "30000")
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (6, 3, 2, 0)))
    rows = [(b.offset, tuple(b.sz), b.bflag, tuple(b.ptmin), tuple(b.ptmax)) for b in blocks]
    shuffled = dgb.blocks_array(rows[::-1])  # same layout, list in reverse order
    u = host_fields(dgb, blocks, SEED2)
    plan = dgb.Plan(shuffled, dgb.default_params(0.1))
    dev = run_device(dgb, torch, plan, u, precision, rhs_init=[np.full(len(u[0]), 7.0)] * 24)
    for rep in range(2):  # second call reuses the pipeline
        host = [np.full(len(u[0]), 7.0) for _ in range(24)]
        plan.rhs_host(host, u, precision)
        for v in range(24):
            assert np.array_equal(dev[v], host[v]), (rep, v)
    plan.close()


@pytest.mark.parametrize("all_pinned", [True, False])
def test_rhs_host_pipeline_pinned_inputs(dgb, gpu, all_pinned, monkeypatch):
    """Fields in dgb_host_alloc memory (all 24 pinned) are uploaded straight
    from the caller's arrays on the first three calls and through the staging
    on the fourth (the plan times both modes); with one field pageable every call
    goes through the staging: the same bits as the device entry each time,
    padding untouched."""
    torch = gpu
    monkeypatch.setenv("DGB_HOST_CHUNK_PTS", "30000")
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (6, 3, 2, 0)))
    u = host_fields(dgb, blocks, SEED2)
    n = len(u[0])
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    dev = run_device(dgb, torch, plan, u, rhs_init=[np.full(n, 7.0)] * 24)
    pu = []
    for v in range(24):
        a = dgb.host_array(n) if (all_pinned or v != 5) else np.empty(n)
        a[:] = u[v]
        pu.append(a)
    for rep in range(4):  # direct (two warm-ups), direct, then through the staging
        host = [dgb.host_array(n) for _ in range(24)]
        for a in host:
            a[:] = 7.0
        plan.rhs_host(host, pu)
        for v in range(24):
            assert np.array_equal(dev[v], host[v]), (rep, v)
    plan.close()


@pytest.mark.parametrize("upload,download", [("direct", "store"), ("staged", "copy"),
                                              ("direct", "copy"), ("staged", "store")])
def test_rhs_host_pipeline_output_paths(dgb, gpu, upload, download, monkeypatch):
    """Page-locked inputs and outputs with each upload mode and each output
    path (the kernel storing into the caller's arrays, or download + host
    scatter): the device entry's bits, padding untouched, FP64 and mixed."""
    torch = gpu
    monkeypatch.setenv("DGB_HOST_CHUNK_PTS", "30000")
    monkeypatch.setenv("DGB_HOST_UPLOAD", upload)
    monkeypatch.setenv("DGB_HOST_DOWNLOAD", download)
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (6, 3, 2, 0)))
    u = host_fields(dgb, blocks, SEED2)
    n = len(u[0])
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    pu = []
    for v in range(24):
        a = dgb.host_array(n)
        a[:] = u[v]
        pu.append(a)
    for prec in (dgb.PREC_FP64, dgb.PREC_MIXED):
        dev = run_device(dgb, torch, plan, u, rhs_init=[np.full(n, 7.0)] * 24, precision=prec)
        host = [dgb.host_array(n) for _ in range(24)]
        for a in host:
            a[:] = 7.0
        plan.rhs_host(host, pu, prec)
        for v in range(24):
            assert np.array_equal(dev[v], host[v]), (prec, v)
    plan.close()


def test_block_entry_matches_oracle(dgb, gpu, oracle):
    """dgb_bssnrhs_block_host: the bssnrhs(...) drop-in for one block at an offset."""
    allb = dgb.synth_blocks(2, SEED2)
    idx = sample_uneven(allb, (2, 1, 0, 0))
    blocks = repack(dgb, allb, idx)
    u = host_fields(dgb, blocks, SEED2)
    want = oracle_rhs(dgb, oracle, blocks, u, 0.1)
    got = [np.zeros(len(u[0])) for _ in range(24)]
    import ctypes as C
    prm = dgb.default_params(0.1)
    for b in blocks:
        r, k1 = dgb.host_ptrs(got)
        uu, k2 = dgb.host_ptrs(u)
        pmin = (C.c_double * 3)(*b.ptmin)
        pmax = (C.c_double * 3)(*b.ptmax)
        sz = (C.c_uint32 * 3)(*b.sz)
        dgb.check(dgb.lib().dgb_bssnrhs_block_host(r, uu, b.offset, pmin, pmax, sz, 0,
                                                     C.byref(prm), 0), "block")
    mask = interior_mask(blocks, len(u[0]))
    assert np.all(normwise(got, want, mask) <= FP64_TOL)


def test_rhs_mixed_precision_error(dgb, gpu, oracle):
    torch = gpu
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb))
    u = host_fields(dgb, blocks, SEED2)
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    got = run_device(dgb, torch, plan, u, precision=1)
    want = oracle_rhs(dgb, oracle, blocks, u, 0.1)
    err = normwise(got, want, interior_mask(blocks, len(u[0])))
    print("mixed per-field normwise error:", dict(zip(dgb.VAR_NAMES, np.round(err, 12))))
    assert np.all(np.isfinite(err))
    assert err.max() <= MIXED_RHS_TOL, dict(zip(dgb.VAR_NAMES, err))


def test_synth_device_fill_bit_identical(dgb, gpu):
    torch = gpu
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (3, 2, 1, 1)))
    u = host_fields(dgb, blocks, SEED2)
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    n = len(u[0])
    du = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(24)]
    plan.synth_fill_device([t.data_ptr() for t in du], SEED2, 1e-6)
    torch.cuda.synchronize()
    for v in range(24):
        assert np.array_equal(du[v].cpu().numpy(), u[v])


def test_rk4_stage_matches_oracle(dgb, gpu, oracle):
    torch = gpu
    rng = np.random.default_rng(7)
    n = 5000
    prev = [rng.normal(0, 1e-3, n) for _ in range(24)]
    for v in (12, 15, 17):
        prev[v] += 1.0
    prev[0] += 0.5
    prev[1] += 0.3
    prev[1][:50] = 1e-6  # exercises the chi floor
    ks = [[rng.normal(0, 1e-2, n) for _ in range(24)] for _ in range(4)]
    dt = 0.0125
    for s in range(4):
        want = [np.zeros(n) for _ in range(24)]
        oracle.rk4_stage(s, want, prev, ks[:s + 1], dt, 1e-4)
        dp = device_fields(torch, prev)
        dk = [device_fields(torch, ks[q]) for q in range(4)]
        dd = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(24)]
        dgb.rk4_stage(s, [t.data_ptr() for t in dd], [t.data_ptr() for t in dp],
                      [t.data_ptr() for q in range(4) for t in dk[q]], n, dt, 1e-4)
        got = [t.cpu().numpy() for t in dd]
        for v in range(24):
            np.testing.assert_allclose(got[v], want[v], rtol=1e-13, atol=1e-15)


def test_exact_mul_device_matches_dmul(dgb, gpu):
    """The integer-pipe tap products equal DMUL bit for bit on the device."""
    assert dgb.selftest_exact_mul(1, 1 << 24, seed=3) == 0


@pytest.mark.parametrize("precision", [0, 1])
def test_rhs_boundary_blocks_match_oracle(dgb, gpu, oracle, precision):
    """Domain-boundary blocks (bflag != 0): one-sided closures and the
    outgoing-radiation condition, with the padding beyond the flagged faces
    left as NaN as an unzip leaves it.  Boundary blocks take the FP64 path in
    both precisions."""
    from test_oracle import boundary_blocks, poison_outside
    torch = gpu
    blocks = boundary_blocks(dgb)
    u = host_fields(dgb, blocks, SEED1)
    poison_outside(blocks, u)
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    got = run_device(dgb, torch, plan, u, precision=precision)
    want = oracle_rhs(dgb, oracle, blocks, u, 0.1)
    bmask = np.zeros(len(u[0]), dtype=bool)
    full = interior_mask(blocks, len(u[0]))
    for b in blocks:
        if b.bflag:
            bmask[b.offset:b.offset + 13 ** 3] = True
    mask = full & bmask
    err = normwise(got, want, mask)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.VAR_NAMES, err))
