"""Parity of the CUDA constraint diagnostics (through the C ABI) with the
oracle and with the reference's golden vectors: Hamiltonian, momentum and
Psi4 of physical_constraints (BSSN_GR/src/physcon.cpp:12-96) within 1e-12
normwise per output, Psi4 zeroed on exactly the same axis points, and the
masked L2 norm of computeConstraintL2Norm (BSSN_GR/include/grUtils.tcc:40-88)
over a mesh pipeline unzip -> constraints -> zip -> norm
(BSSN_GR/src/bssnCtx.cpp:332-365)."""
import os

import numpy as np
import pytest

from workloads import SEED1, SEED2, host_fields, interior_mask, normwise, repack, sample_uneven

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "constraints_reference.npz")


def gpu_constraints(dgb, torch, plan, u_host, fill=7.0):
    du = [torch.from_numpy(a).cuda() for a in u_host]
    n = len(u_host[0])
    dc = [torch.full((n,), fill, dtype=torch.float64, device="cuda") for _ in range(6)]
    plan.physical_constraints([t.data_ptr() for t in dc], [t.data_ptr() for t in du])
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in dc]


def oracle_constraints(oracle, blocks, u):
    n = len(u[0])
    c = [np.zeros(n) for _ in range(6)]
    assert oracle.physcon_blocks(c, u, blocks) == 0
    return c


def check(dgb, got, want, mask):
    err = normwise(got, want, mask)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.CONSTRAINT_NAMES, err))
    for c in (4, 5):
        assert np.array_equal(got[c][mask] == 0.0, want[c][mask] == 0.0)


@pytest.mark.parametrize("which", ["uniform512", "uneven_sample"])
def test_constraints_match_oracle(dgb, gpu, oracle, which):
    torch = gpu
    if which == "uniform512":
        blocks, seed = dgb.synth_blocks(1), SEED1
    else:
        allb = dgb.synth_blocks(2, SEED2)
        blocks, seed = repack(dgb, allb, sample_uneven(allb)), SEED2
    u = host_fields(dgb, blocks, seed)
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    got = gpu_constraints(dgb, torch, plan, u)
    want = oracle_constraints(oracle, blocks, u)
    mask = interior_mask(blocks, len(u[0]))
    check(dgb, got, want, mask)
    for c in range(6):
        assert np.all(got[c][~mask] == 7.0)  # padding untouched
    plan.close()


def test_constraints_match_reference_golden(dgb, gpu):
    """Directly against the reference's own outputs (includes a block on the
    z axis and two domain-boundary corner blocks)."""
    torch = gpu
    g = np.load(GOLDEN)
    allb = dgb.synth_blocks(1)
    rows, off = [], 0
    for i, f in g["picks"]:
        b = allb[int(i)]
        rows.append((off, tuple(b.sz), int(f), tuple(b.ptmin), tuple(b.ptmax)))
        off += b.sz[0] * b.sz[1] * b.sz[2]
    blocks = dgb.blocks_array(rows)
    u = host_fields(dgb, blocks, int(g["seed"]))
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    got = gpu_constraints(dgb, torch, plan, u)
    mask = interior_mask(blocks, len(u[0]))
    gm = [x[mask] for x in got]
    want = list(g["cons"])
    ones = np.ones(len(gm[0]), dtype=bool)
    err = normwise(gm, want, ones)
    assert np.all(err <= FP64_TOL), dict(zip(dgb.CONSTRAINT_NAMES, err))
    assert np.array_equal(gm[4] == 0.0, want[4] == 0.0)
    plan.close()


def test_constraints_boundary_blocks(dgb, gpu, oracle):
    """One-sided 4th-order closures on every face class; NaN in the padding
    beyond flagged faces (a mesh leaves it unfilled) never reaches a result."""
    from test_oracle import boundary_blocks, poison_outside
    torch = gpu
    blocks = boundary_blocks(dgb)
    u = host_fields(dgb, blocks, SEED1)
    poison_outside(blocks, u)
    plan = dgb.Plan(blocks, dgb.default_params(0.1))
    got = gpu_constraints(dgb, torch, plan, u)
    want = oracle_constraints(oracle, blocks, u)
    mask = interior_mask(blocks, len(u[0]))
    assert all(np.isfinite(x[mask]).all() for x in got)
    check(dgb, got, want, mask)
    plan.close()


def test_constraint_l2_masked_rms(dgb, gpu):
    torch = gpu
    rng = np.random.default_rng(3)
    n = 1_000_003
    f = [rng.normal(size=n) * (10.0 ** -q) for q in range(4)]
    mask = rng.uniform(size=n)
    mask[::97] = np.nan  # the reference's test (value < threshold) keeps NaN
    thr = 0.3
    df = [torch.from_numpy(a).cuda() for a in f]
    dm = torch.from_numpy(mask).cuda()
    got = dgb.constraint_l2([t.data_ptr() for t in df], n, dm.data_ptr(), thr)
    keep = ~(mask < thr)
    want = [np.sqrt(np.sum(a[keep] ** 2) / keep.sum()) for a in f]
    np.testing.assert_allclose(got, want, rtol=1e-13)
    again = dgb.constraint_l2([t.data_ptr() for t in df], n, dm.data_ptr(), thr)
    assert got == again  # fixed reduction order
    nomask = dgb.constraint_l2([t.data_ptr() for t in df[:1]], n)
    np.testing.assert_allclose(nomask[0], np.sqrt(np.mean(f[0] ** 2)), rtol=1e-13)


def test_constraint_pipeline_on_mesh(dgb, gpu, oracle):
    """unzip -> physical_constraints -> zip -> masked L2 on an octree mesh,
    against the host operator + oracle + numpy."""
    from test_mesh import apply_unzip
    torch = gpu
    m = dgb.Mesh(dgb.mesh_params(max_level=6, min_level=3, fine_radius=1.0))
    op = m.operator()
    uz = dgb.UnzipPlan(op, m.ndof)
    plan = dgb.Plan(m.blocks, dgb.default_params(0.1))
    xyz = m.dof_coords()
    z = [np.zeros(m.ndof) for _ in range(24)]
    dgb.synth_fill_points(xyz, z, 7, 1e-6)
    dz = [torch.from_numpy(a).cuda() for a in z]
    du = [torch.zeros(m.nunzipped, dtype=torch.float64, device="cuda") for _ in range(24)]
    uz.unzip([t.data_ptr() for t in dz], [t.data_ptr() for t in du])
    dc = [torch.zeros(m.nunzipped, dtype=torch.float64, device="cuda") for _ in range(6)]
    plan.physical_constraints([t.data_ptr() for t in dc], [t.data_ptr() for t in du])
    dcz = [torch.zeros(m.ndof, dtype=torch.float64, device="cuda") for _ in range(6)]
    uz.zip([t.data_ptr() for t in dc], [t.data_ptr() for t in dcz])
    thr = 0.5
    got_l2 = dgb.constraint_l2([t.data_ptr() for t in dcz[:4]], m.ndof, dz[1].data_ptr(), thr)
    torch.cuda.synchronize()

    uh = [np.nan_to_num(apply_unzip(op, z[v], m.nunzipped), nan=0.0) for v in range(24)]
    ch = oracle_constraints(oracle, m.blocks, uh)
    zs = op["zip_src"].astype(np.int64)
    want_z = [c[zs] for c in ch]
    got_z = [t.cpu().numpy() for t in dcz]
    err = normwise(got_z, want_z, np.ones(m.ndof, dtype=bool))
    assert np.all(err <= FP64_TOL), dict(zip(dgb.CONSTRAINT_NAMES, err))
    keep = ~(z[1] < thr)
    want_l2 = [np.sqrt(np.sum(w[keep] ** 2) / keep.sum()) for w in want_z[:4]]
    np.testing.assert_allclose(got_l2, want_l2, rtol=1e-11)
    uz.close()
    plan.close()
    m.close()


@pytest.mark.parametrize("pinned", [False, True])
def test_constraints_host_pipeline_many_chunks(dgb, gpu, pinned, monkeypatch):
    """dgb_physical_constraints_host over many chunks (24 fields in, 6 out),
    block list not in offset order, boundary blocks included: the device
    entry's bits, padding of the outputs untouched; pinned: inputs and
    outputs in dgb_host_alloc memory (uploaded without staging)."""
    torch = gpu
    monkeypatch.setenv("DGB_HOST_CHUNK_PTS", "30000")
    allb = dgb.synth_blocks(2, SEED2)
    blocks = repack(dgb, allb, sample_uneven(allb, (6, 3, 2, 0)))
    rows = [(b.offset, tuple(b.sz), (63 if i % 3 == 0 else 0), tuple(b.ptmin), tuple(b.ptmax))
            for i, b in enumerate(blocks)]
    blocks = dgb.blocks_array(rows)
    u = host_fields(dgb, blocks, SEED2)
    plan = dgb.Plan(dgb.blocks_array(rows[::-1]), dgb.default_params(0.1))
    dev = gpu_constraints(dgb, torch, plan, u)
    n = len(u[0])
    if pinned:
        pu = [dgb.host_array(n) for _ in range(24)]
        for v in range(24):
            pu[v][:] = u[v]
        u = pu
    for rep in range(4 if pinned else 2):  # pinned: direct x3, then staged upload
        host = [dgb.host_array(n) if pinned else np.empty(n) for _ in range(6)]
        for h in host:
            h[:] = 7.0
        plan.physical_constraints_host(host, u)
        for c in range(6):
            assert np.array_equal(dev[c], host[c]), (rep, dgb.CONSTRAINT_NAMES[c])
    plan.close()
