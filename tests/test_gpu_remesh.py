"""GPU wavelet refinement indicator (dgb_remesh_wavelets, the indicator of
Mesh::isReMeshUnzip, include/mesh.tcc:2035-2197) against the oracle on the
same unzipped fields: per-leaf wavelet maxima and flags must be identical
bit for bit (the kernel evaluates the oracle's weights in the oracle's
summation order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def unzipped_mesh(dgb, gpu):
    torch = gpu
    m = dgb.Mesh(dgb.mesh_params(max_level=7, min_level=3, fine_radius=1.0))
    op = m.operator()
    uz = dgb.UnzipPlan(op, m.ndof)
    z = [np.zeros(m.ndof) for _ in range(24)]
    dgb.synth_fill_points(m.dof_coords(), z, 11, 1e-6)
    dz = [torch.from_numpy(a).cuda() for a in z]
    du = [torch.zeros(m.nunzipped, dtype=torch.float64, device="cuda") for _ in range(24)]
    uz.unzip([t.data_ptr() for t in dz], [t.data_ptr() for t in du])
    torch.cuda.synchronize()
    uz.close()
    host = [t.cpu().numpy() for t in du]
    yield m, du, host
    m.close()


def run_gpu(dgb, torch, m, du, var_ids, t, tol, coarse_fac, extra_leaf=None):
    base, side, bdy = t["patch_base"], t["block_side"], t["boundary"]
    if extra_leaf is not None:
        base = np.append(base, np.uint64(extra_leaf[0]))
        side = np.append(side, np.uint32(extra_leaf[1]))
        bdy = np.append(bdy, np.uint8(0))
        tol = np.append(tol, 1.0)
    n = len(base)
    d_base = torch.from_numpy(base.astype(np.int64)).cuda()
    d_side = torch.from_numpy(side.astype(np.int32)).cuda()
    d_bdy = torch.from_numpy(bdy).cuda()
    d_tol = torch.from_numpy(np.ascontiguousarray(tol)).cuda()
    wmax = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    flags = torch.full((n,), 77, dtype=torch.uint8, device="cuda")
    changed = torch.full((1,), 12345, dtype=torch.int64, device="cuda")
    dgb.remesh_wavelets([x.data_ptr() for x in du], var_ids, m.nunzipped, n, d_base.data_ptr(),
                        d_side.data_ptr(), d_bdy.data_ptr(), d_tol.data_ptr(), coarse_fac,
                        wmax.data_ptr(), flags.data_ptr(), changed.data_ptr())
    torch.cuda.synchronize()
    return wmax.cpu().numpy(), flags.cpu().numpy(), int(changed.item())


@pytest.mark.parametrize("var_ids", [[0], [0, 7, 13], list(range(24))])
def test_wavelets_match_oracle(dgb, gpu, oracle, unzipped_mesh, var_ids):
    torch = gpu
    m, du, host = unzipped_mesh
    t = m.leaf_patches()
    n = m.num_leaves
    # tolerances that split about a third of the leaves and coarsen another third
    probe, _, _ = oracle.remesh_wavelets(host, var_ids, t["patch_base"], t["block_side"],
                                         t["boundary"], np.full(n, 1e30), 0.1)
    tol = np.full(n, np.quantile(probe, 0.66))
    tol[::7] *= 50.0  # per-leaf tolerance
    want_w, want_f, want_c = oracle.remesh_wavelets(host, var_ids, t["patch_base"],
                                                    t["block_side"], t["boundary"], tol, 0.1)
    assert 0 < np.count_nonzero(want_f == 1) < n and np.count_nonzero(want_f == 2) > 0
    got_w, got_f, got_c = run_gpu(dgb, torch, m, du, var_ids, t, tol, 0.1)
    assert np.array_equal(got_w, want_w), np.abs(got_w - want_w).max()
    assert np.array_equal(got_f, want_f)
    assert got_c == want_c


def test_nan_variable_and_invalid_leaf(dgb, gpu, oracle, unzipped_mesh):
    torch = gpu
    m, du, host = unzipped_mesh
    t = m.leaf_patches()
    n = m.num_leaves
    bad = torch.full_like(du[0], float("nan"))
    fields = [bad] + du[:3]
    hfields = [np.full(m.nunzipped, np.nan)] + host[:3]
    tol = np.full(n, 1e-5)
    want_w, want_f, want_c = oracle.remesh_wavelets(hfields, [0, 2], t["patch_base"],
                                                    t["block_side"], t["boundary"], tol, 0.5)
    # one more leaf whose patch runs past the end of the unzipped vector
    got_w, got_f, got_c = run_gpu(dgb, torch, m, fields, [0, 2], t, tol, 0.5,
                                  extra_leaf=(m.nunzipped - 100, 13))
    assert np.array_equal(got_w[:n], want_w) and np.array_equal(got_f[:n], want_f)
    assert np.isnan(got_w[n]) and got_f[n] == dgb.OCT_INVALID
    assert got_c == want_c


def test_bad_arguments_rejected(dgb, gpu):
    with pytest.raises(dgb.DgbError):
        dgb.remesh_wavelets([0], list(range(33)), 0, 0, 0, 0, 0, 0, 0.1, 0, 0)
    with pytest.raises(dgb.DgbError):
        dgb.remesh_wavelets([0], [0], 1000, 5, 0, 0, 0, 0, 0.1, 0, 0)
