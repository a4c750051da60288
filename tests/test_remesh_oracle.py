"""CPU tests of the wavelet refinement indicator's oracle (Mesh::isReMeshUnzip,
include/mesh.tcc:2035-2197; WaveletEl::compute_wavelets_3D,
src/waveletRefEl.cpp:92-271) and of the mesh's per-leaf patch table.

The oracle is pinned against the reference's own WaveletEl (built with its
RefElement into oracle/_ref/libmesh_ref.so; goldens in
tests/golden/mesh_reference.npz): wavelets within 1e-14 of the data's scale
(both sides interpolate with Lagrange weights of the uniform nodes, the
reference's from a LAPACK solve, so they differ by rounding, and a wavelet is
a small difference of O(1) values); the per-leaf patches and boundary flags
equal the reference's getUnzipElementalNodalValues and isBoundaryOctant.
Known answers pin it further: the wavelets of an interior element vanish for
every polynomial of degree <= 6 per axis (the parent interpolant reproduces
it) and those of a boundary element for degree <= 3; for the monic x^7
(interior) and x^4 (boundary) they equal the interpolation error
prod(x - x_b) over the parent nodes x_b, relative to max(1, |u|)."""
import math
import os

import numpy as np
import pytest

from meshref import GOLDEN_MESH, field, wavelet_test_patches

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "mesh_reference.npz")
WAVELET_TOL = 1e-14  # of max |data|


def test_wavelets_equal_reference_goldens(oracle):
    g = np.load(GOLDEN)
    wp = wavelet_test_patches(seed=int(g["wavelet_patch_seed"]))
    half = len(wp) // 2
    for i, p in enumerate(wp):
        wc, _ = oracle.wavelet_patch(p, boundary=i >= half)
        assert np.max(np.abs(wc - g["wavelet_wc"][i])) <= WAVELET_TOL * np.max(np.abs(p)), i


def test_leaf_patches_and_wavelets_equal_reference_goldens(dgb, oracle):
    """On the level-6 mesh: every leaf's patch of the unzipped smooth field,
    its boundary flag and its wavelet RMS against the reference's own
    (getUnzipElementalNodalValues, isBoundaryOctant, compute_wavelets_3D)."""
    from oracle_py import unzip_apply
    g = np.load(GOLDEN)
    m = dgb.Mesh(dgb.mesh_params(**GOLDEN_MESH))
    uz = unzip_apply(m.operator(), field(m.dof_coords()), m.nunzipped)
    lp = m.leaf_patches()
    elem = g["element_order"].astype(np.int64)
    assert np.array_equal(lp["boundary"][elem], g["element_boundary"])
    n = lp["block_side"]
    rms = np.zeros(len(elem))
    for q, e in enumerate(elem):
        b, s = int(lp["patch_base"][e]), int(n[e])
        idx = b + np.arange(13)[None, None, :] + s * (np.arange(13)[None, :, None]
                                                      + s * np.arange(13)[:, None, None])
        _, rms[q] = oracle.wavelet_patch(uz[idx], boundary=bool(lp["boundary"][e]))
    assert np.max(np.abs(rms - g["element_wavelet_rms"])) <= WAVELET_TOL * np.nanmax(np.abs(uz))


@pytest.fixture(scope="module")
def refmesh():
    import oracle_py
    if not os.path.isdir(oracle_py.REF_ROOT) and not os.path.exists(oracle_py.MESH_REF_SO):
        pytest.skip("reference tree not present on this machine")
    oracle_py.build_ref()
    return oracle_py.MeshReference()


def test_wavelets_equal_reference_live(oracle, refmesh):
    for i, p in enumerate(wavelet_test_patches(n=64, seed=11)):
        for bd in (False, True):
            wc, _ = oracle.wavelet_patch(p, boundary=bd)
            wr = refmesh.wavelets(p.ravel(), (13, 13, 13), bd)
            assert np.max(np.abs(wc - wr)) <= WAVELET_TOL * np.max(np.abs(p)), (i, bd)


def test_leaf_patches_equal_reference_live(dgb, refmesh):
    """Per leaf of a level-8 mesh, the 13^3 patch at patch_base (rows of
    block_side) equals the reference's getUnzipElementalNodalValues bit for
    bit on a random unzipped vector, and the boundary flags agree.  On a leaf
    touching the domain boundary the reference overwrites the padding beyond
    it with the face values (include/mesh.tcc:9178-9246), which the boundary
    wavelets never read (they use points 3..9 per axis): there the 7^3
    nodes are compared."""
    from meshref import leaves_in_octree_units
    m = dgb.Mesh(dgb.mesh_params(max_level=8, min_level=4, fine_radius=1.0))
    anc, lev, md = leaves_in_octree_units(m)
    R = refmesh.build(anc, lev, md)
    u = np.random.default_rng(9).standard_normal(m.nunzipped)
    elem, patches, bdy = R.element_patches(u)
    lp = m.leaf_patches()
    assert np.array_equal(lp["boundary"][elem], bdy)
    ax = np.arange(13)
    for q, e in enumerate(elem):
        b, s = int(lp["patch_base"][e]), int(lp["block_side"][e])
        idx = b + ax[None, None, :] + s * (ax[None, :, None] + s * ax[:, None, None])
        if bdy[q]:
            assert np.array_equal(u[idx][3:10, 3:10, 3:10],
                                  patches[q].reshape(13, 13, 13)[3:10, 3:10, 3:10]), q
        else:
            assert np.array_equal(u[idx].ravel(), patches[q]), q

IDX = np.arange(13, dtype=np.float64)


def patch_of(f):
    k, j, i = np.meshgrid(IDX, IDX, IDX, indexing="ij")
    return f(i, j, k)


def test_interior_reproduces_degree6(oracle):
    rng = np.random.default_rng(3)
    for trial in range(5):
        c = rng.normal(size=(3, 7))

        def f(i, j, k):
            x, y, z = ((a - 6.0) / 6.0 for a in (i, j, k))
            return (np.polyval(c[0], x) * np.polyval(c[1], y) * np.polyval(c[2], z)
                    + 0.3 * x ** 6 * y ** 6 * z ** 6 + 2.0)
        wc, rms = oracle.wavelet_patch(patch_of(f), boundary=False)
        assert np.abs(wc).max() <= 1e-13, (trial, np.abs(wc).max())
        assert rms <= 1e-13


def test_boundary_reproduces_degree3(oracle):
    rng = np.random.default_rng(4)
    c = rng.normal(size=(3, 4))

    def f(i, j, k):
        x, y, z = ((a - 6.0) / 3.0 for a in (i, j, k))
        return np.polyval(c[0], x) * np.polyval(c[1], y) * np.polyval(c[2], z) + x ** 3 * z ** 3

    p = patch_of(f)
    p[:3] = np.nan  # the padding is never read on a boundary element
    wc, rms = oracle.wavelet_patch(p, boundary=True)
    assert np.abs(wc).max() <= 1e-13 and rms <= 1e-13
    assert np.all(wc[27:] == 0.0)


def test_interior_known_answer_x7(oracle):
    wc, rms = oracle.wavelet_patch(patch_of(lambda i, j, k: i ** 7), boundary=False)
    want_1d = []
    for x in (3, 5, 7, 9):
        err = abs(math.prod(x - 2 * b for b in range(7)))
        want_1d.append(err / max(1.0, float(x) ** 7))
    want = np.tile(np.array(want_1d), 16)  # slot (kk*4+jj)*4+i depends on i only
    np.testing.assert_allclose(wc, want, rtol=1e-12, atol=0)
    assert abs(rms - math.sqrt(np.sum(want ** 2)) / 8.0) <= 1e-14 * rms


def test_boundary_known_answer_x4(oracle):
    wc, rms = oracle.wavelet_patch(patch_of(lambda i, j, k: k ** 4), boundary=True)
    want_1d = []
    for x in (4, 6, 8):
        err = abs(math.prod(x - (3 + 2 * b) for b in range(4)))
        want_1d.append(err / max(1.0, float(x) ** 4))
    want = np.repeat(np.array(want_1d), 9)  # slot (kk*3+jj)*3+i depends on kk only
    np.testing.assert_allclose(wc[:27], want, rtol=1e-12, atol=0)
    assert np.all(wc[27:] == 0.0)
    assert abs(rms - math.sqrt(np.sum(want ** 2)) / 8.0) <= 1e-14 * rms


def test_relative_form_below_one(oracle):
    # |u| < 1: the wavelet is the absolute interpolation error
    wc, _ = oracle.wavelet_patch(patch_of(lambda i, j, k: 1e-8 * i ** 7), boundary=False)
    np.testing.assert_allclose(wc[:4], [1e-8 * 2835, 1e-8 * 1575, 1e-8 * 1575, 1e-8 * 2835],
                               rtol=1e-9)


def leaf_table(side):
    """All 13^3 patches of one block with (side - 7) / 6 leaves per axis."""
    m = (side - 7) // 6
    base = [6 * x + side * (6 * y + side * 6 * z) for z in range(m) for y in range(m)
            for x in range(m)]
    return np.array(base, dtype=np.uint64), np.full(len(base), side, dtype=np.uint32)


def test_indicator_flags_and_early_exit(oracle):
    side = 6 * 2 + 7
    base, bs = leaf_table(side)
    n = len(base)
    k, j, i = np.meshgrid(*(np.arange(side, dtype=np.float64),) * 3, indexing="ij")
    smooth = (0.1 * i + 0.02 * j * k).ravel()                  # wavelets 0
    rough = np.random.default_rng(5).normal(size=side ** 3) * 1e-3
    rougher = rough * 10.0
    u = [smooth, rough, rougher]
    bdy = np.zeros(n, dtype=np.uint8)
    # per-variable RMS, one variable at a time
    per = np.stack([oracle.remesh_wavelets(u, [v], base, bs, bdy, np.full(n, 1e9), 0.1)[0]
                    for v in range(3)])
    assert np.all(per[0] <= 1e-14) and np.all(per[2] > per[1])
    tol = per[1] * 1.5  # var 1 below tol, var 2 above
    wmax, flags, changed = oracle.remesh_wavelets(u, [0, 1, 2], base, bs, bdy, tol, 0.1)
    assert np.array_equal(wmax, per[2]) and np.all(flags == 1) and changed == n
    tol = per[1] * 0.5  # var 1 passes tol: var 2 is never looked at
    wmax, flags, changed = oracle.remesh_wavelets(u, [0, 1, 2], base, bs, bdy, tol, 0.1)
    assert np.array_equal(wmax, per[1]) and np.all(flags == 1)
    tol = per[2] * 100.0  # all below coarse_fac * tol
    wmax, flags, changed = oracle.remesh_wavelets(u, [1, 2], base, bs, bdy, tol, 0.1)
    assert np.all(flags == 2) and changed == n
    tol = per[2] * 5.0  # between coarse_fac * tol and tol
    wmax, flags, changed = oracle.remesh_wavelets(u, [1, 2], base, bs, bdy, tol, 0.1)
    assert np.all(flags == 0) and changed == 0
    # a NaN variable yields a NaN RMS, which never raises the running maximum
    bad = rough.copy()
    bad[:] = np.nan
    wmax, flags, _ = oracle.remesh_wavelets([bad, rough], [0, 1], base, bs, bdy,
                                            np.full(n, 1e9), 0.1)
    assert np.array_equal(wmax, per[1])


def test_leaf_patches_cover_mesh(dgb):
    mesh = dgb.Mesh(dgb.mesh_params(max_level=6, min_level=3, fine_radius=1.0))
    t = mesh.leaf_patches()
    lev, anc = mesh.leaves()
    n = mesh.num_leaves
    assert len(t["patch_base"]) == n
    # each leaf's patch lies inside its block, and its corner matches its anchor
    starts = np.array([b.offset for b in mesh.blocks], dtype=np.uint64)
    blk = np.searchsorted(starts, t["patch_base"], side="right") - 1
    for e in range(0, n, max(1, n // 200)):
        b = mesh.blocks[blk[e]]
        side = b.sz[0]
        assert t["block_side"][e] == side
        rel = int(t["patch_base"][e] - b.offset)
        x, y, z = rel % side, (rel // side) % side, rel // (side * side)
        assert x % 6 == 0 and y % 6 == 0 and z % 6 == 0 and max(x, y, z) + 13 <= side
        h = (b.ptmax[0] - b.ptmin[0]) / (side - 1)
        np.testing.assert_allclose(t["hx"][e], h, rtol=1e-15)
        for a, o in enumerate((x, y, z)):
            np.testing.assert_allclose(t["corner"][e, a], b.ptmin[a] + (o + 3) * h, rtol=0,
                                       atol=1e-12)
    size = 6.0 * t["hx"]
    on_face = np.any((np.abs(t["corner"] + 32.0) < 1e-9)
                     | (np.abs(t["corner"] + size[:, None] - 32.0) < 1e-9), axis=1)
    assert np.array_equal(on_face, t["boundary"].astype(bool))
    # leaf order of the table is the mesh's leaf order
    unit = 64.0 / (6 << 6)
    np.testing.assert_allclose(t["corner"], -32.0 + anc * unit, atol=1e-12)
    mesh.close()


def test_tolerance_ramp(dgb):
    corner = np.array([[0.0, 0, 0], [3.0, 4.0, 0], [30.0, 40.0, 0.0], [6.0, 8.0, 0]])
    tol = dgb.wavelet_tol_radial(corner, 1e-5, 1e-3, r0=5.0, r1=10.0, use_function=True)
    np.testing.assert_allclose(tol, [1e-5, 1e-5, 1e-3, 1e-5 + (1e-3 - 1e-5) / 5.0 * 5.0],
                               rtol=1e-14)
    assert np.all(dgb.wavelet_tol_radial(corner, 2e-4) == 2e-4)


def test_indicator_on_host_unzipped_mesh(dgb, oracle):
    """On the octree: a field of degree <= 3 per axis gives zero wavelets on
    every leaf (coarsen everywhere); a sharp Gaussian flags the leaves
    around the punctures for splitting and none far away."""
    from oracle_py import unzip_apply
    mesh = dgb.Mesh(dgb.mesh_params(max_level=6, min_level=3, fine_radius=1.0))
    op = mesh.operator()
    xyz = mesh.dof_coords()
    t = mesh.leaf_patches()
    n = mesh.num_leaves
    x, y, z = (xyz[:, a] / 32.0 for a in range(3))
    cubic = 1.0 + 0.3 * x - 0.2 * y ** 3 + 0.5 * x * y * z + 0.1 * z ** 3
    gauss = np.exp(-np.sum(xyz ** 2, axis=1) / 0.5)
    u = [unzip_apply(op, f, mesh.nunzipped) for f in (cubic, gauss)]
    tol = np.full(n, 1e-4)
    wmax, flags, _ = oracle.remesh_wavelets(u, [0], t["patch_base"], t["block_side"],
                                            t["boundary"], tol, 0.1)
    assert np.abs(wmax).max() <= 1e-12 and np.all(flags == 2)
    wmax, flags, changed = oracle.remesh_wavelets(u, [1], t["patch_base"], t["block_side"],
                                                  t["boundary"], tol, 0.1)
    r = np.linalg.norm(t["corner"] + 3.0 * t["hx"][:, None], axis=1)
    assert np.all(np.isfinite(wmax))
    assert np.any(flags[r < 2.0] == 1)
    assert np.all(flags[r > 10.0] == 2)
    assert changed == np.count_nonzero(flags)
    mesh.close()
