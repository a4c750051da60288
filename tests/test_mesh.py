"""CPU tests of the octree mesh and its unzip / zip operators: property
checks in the style of the reference's mesh tests
(test/include/meshTestUtils.h: isUnzipValid :290 checks that unzip
reproduces a smooth function in the padding): 2:1 balance, blocks cover the
leaves, unzip reproduces any polynomial of degree <= 6 per axis exactly (the
element interpolant is exact for it), and zip(unzip(z)) = z.  The comparison
with the reference's own ot::Mesh is tests/test_mesh_reference.py."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def mesh(dgb):
    return dgb.Mesh(dgb.mesh_params(max_level=6, min_level=3, fine_radius=1.0))


from oracle_py import unzip_apply as apply_unzip  # noqa: E402  (host unzip: the checker)


def padded_coords(blocks):
    pts = []
    for b in blocks:
        nx, ny, nz = b.sz
        h = [(b.ptmax[a] - b.ptmin[a]) / (b.sz[a] - 1) for a in range(3)]
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        pts.append(np.stack([b.ptmin[0] + i.ravel() * h[0], b.ptmin[1] + j.ravel() * h[1],
                             b.ptmin[2] + k.ravel() * h[2]], axis=1))
    return np.concatenate(pts)


def poly(xyz):
    x, y, z = (xyz[:, a] / 32.0 for a in range(3))
    return (1 + 0.3 * x - 0.7 * x ** 3 + 0.2 * x ** 6) * (0.5 - y ** 2 + 0.4 * y ** 5) \
        * (1 + z + 0.8 * z ** 4) + 0.1 * x ** 6 * y ** 6 * z ** 6


def test_two_to_one_balance(mesh):
    lev, anc = mesh.leaves()
    N = 6 << 6
    size = {L: 6 << (6 - L) for L in range(7)}
    idx = {(int(l), *map(int, a)): i for i, (l, a) in enumerate(zip(lev, anc))}

    def leaf_holding(c):
        for L in range(6, -1, -1):
            s = size[L]
            k = (L, c[0] // s * s, c[1] // s * s, c[2] // s * s)
            if k in idx:
                return idx[k]
        raise AssertionError("point not covered by a leaf")

    total = 0
    for i, (l, a) in enumerate(zip(lev, anc)):
        total += size[int(l)] ** 3
        s = size[int(l)]
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if dx == dy == dz == 0:
                        continue
                    c = [int(a[q]) + (-1 if d < 0 else (s if d > 0 else s // 2))
                         for q, d in enumerate((dx, dy, dz))]
                    if min(c) < 0 or max(c) >= N:
                        continue
                    assert lev[leaf_holding(c)] >= l - 1
    assert total == N ** 3  # the leaves tile the domain


def test_blocks_cover_leaves(dgb, mesh):
    lev, anc = mesh.leaves()
    vol = 0.0
    for b in mesh.blocks:
        h = (b.ptmax[0] - b.ptmin[0]) / (b.sz[0] - 1)
        vol += ((b.sz[0] - 7) * h) ** 3
        # p * 2^k + 1 + 6 points per side for 2^k leaves (src/block.cpp:50)
        assert b.sz[0] in (13, 19, 31, 55)
        assert b.sz[0] == b.sz[1] == b.sz[2]
    assert vol == pytest.approx(64.0 ** 3, rel=1e-12)
    # the synthetic fields are finite on every block and the layout is contiguous
    off = 0
    for b in mesh.blocks:
        assert b.offset == off
        off += b.sz[0] ** 3
    assert off == mesh.nunzipped


def test_boundary_flags(mesh):
    for b in mesh.blocks:
        for a in range(3):
            h = (b.ptmax[a] - b.ptmin[a]) / (b.sz[a] - 1)
            lo = abs(b.ptmin[a] + 3 * h + 32.0) < 1e-9
            hi = abs(b.ptmax[a] - 3 * h - 32.0) < 1e-9
            assert bool(b.bflag & (1 << (2 * a))) == lo
            assert bool(b.bflag & (1 << (2 * a + 1))) == hi


def test_unzip_reproduces_polynomials(mesh):
    op = mesh.operator()
    xyz = mesh.dof_coords()
    z = poly(xyz)
    u = apply_unzip(op, z, mesh.nunzipped)
    pts = padded_coords(mesh.blocks)
    inside = np.all(np.abs(pts) <= 32.0 + 1e-9, axis=1)
    assert np.all(np.isnan(u[~inside]))  # beyond domain faces: not written
    want = poly(pts[inside])
    got = u[inside]
    assert np.isfinite(got).all()
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err <= 1e-12, err


def test_zip_of_unzip_is_identity(mesh):
    op = mesh.operator()
    z = np.random.default_rng(1).normal(size=mesh.ndof)
    u = apply_unzip(op, z, mesh.nunzipped)
    assert np.array_equal(u[op["zip_src"].astype(np.int64)], z)


def test_operator_sources_read_only_coarser_levels(mesh):
    op = mesh.operator()
    lp = op["level_ptr"].astype(np.int64)
    assert lp[0] == 0 and lp[-1] == len(op["src_refs"]) // 343
    for l in range(len(lp) - 1):
        refs = op["src_refs"][lp[l] * 343:lp[l + 1] * 343]
        interp = (refs >> np.uint64(63)) != 0
        src = (refs[interp] >> np.uint64(12)) & np.uint64(0x7FFFFFFF)
        assert np.all(src < lp[l])
        for a in range(3):
            assert np.all(((refs[interp] >> np.uint64(4 * a)) & np.uint64(0xF)) <= 12)
    # every padded interpolation names an existing source
    src = (op["interp_ref"] >> np.uint64(12)) & np.uint64(0x7FFFFFFF)
    assert np.all(src < lp[-1])
