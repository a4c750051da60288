"""Helpers shared by the mesh parity tests and the golden generator: the
smooth test field the unzip comparisons use, the mapping between this
library's mesh and the reference's octree coordinates, and per-block
checksums of an unzipped vector."""
import numpy as np

# the level-6 mesh the committed mesh goldens were made on
GOLDEN_MESH = dict(max_level=6, min_level=3, fine_radius=1.0)
# blocks whose full padded grids are stored in the goldens: a domain-corner
# block, blocks next to finer and to coarser neighbours, a 19^3 block
GOLDEN_FULL_BLOCKS = 4


def field(xyz, domain=32.0):
    """Smooth but not polynomial, so interpolation at hanging nodes and in
    coarser-neighbour padding is exercised (exact for no degree)."""
    x, y, z = (xyz[:, a] / domain for a in range(3))
    return np.sin(3.1 * x + 0.3) * np.cos(2.3 * y - 0.2) * np.exp(0.7 * z) + x ** 7 * y


def octree_depth(params):
    return params.octree_depth if params.octree_depth > 0 else params.max_level + 4


def leaves_in_octree_units(mesh):
    """The mesh's leaves as (anchors, levels) in octree units of its depth."""
    lev, anc = mesh.leaves()
    md = octree_depth(mesh.params)
    assert np.all(anc % 6 == 0)
    return (anc // 6 * (1 << (md - mesh.params.max_level))).astype(np.uint32), lev, md


def block_rows(mesh):
    """This library's blocks as rows (node x, y, z in octree units, sizes x,
    y, z, offset, face flags), the reference's refmesh_blocks columns 0-2, 5-9."""
    sc = 1 << (octree_depth(mesh.params) - mesh.params.max_level)
    rows = []
    for b, ((ax, ay, az), _, _) in zip(mesh.blocks, mesh.block_levels()):
        rows.append([ax * sc, ay * sc, az * sc, b.sz[0], b.sz[1], b.sz[2], b.offset, b.bflag])
    return np.array(rows, dtype=np.int64)


def cg_keys_from_octree(xyz):
    """Reference CG coordinates (octree units, multiples of 1/6) as exact integers."""
    return np.rint(np.asarray(xyz) * 6).astype(np.int64)


def cg_keys_from_mesh(mesh):
    """This library's node coordinates in the same integers (6 x octree units)."""
    p = mesh.params
    md = octree_depth(p)
    unit = (p.domain_max[0] - p.domain_min[0]) / (6 << p.max_level)  # domain length per lattice unit
    sc = 1 << (md - p.max_level)
    lat = np.rint((mesh.dof_coords() - np.array(p.domain_min[:])) / unit).astype(np.int64)
    return lat * sc


def checksums(uz, blocks_rows):
    """Per block (offset, sizes from rows): number of NaN points, the sum of
    the finite values, and their sum weighted by cos(0.7 * local index)."""
    out = np.zeros((len(blocks_rows), 3))
    for i, r in enumerate(blocks_rows):
        n = int(r[3] * r[4] * r[5])
        v = uz[int(r[6]):int(r[6]) + n]
        fin = np.isfinite(v)
        w = np.cos(0.7 * np.arange(n))
        out[i] = [np.count_nonzero(~fin), np.sum(v[fin]), np.sum((v * w)[fin])]
    return out


def wavelet_test_patches(n=16, seed=5):
    """Seeded 13^3 patches for the wavelet comparison: smooth products plus
    x^7 terms, half of them with 1e-3 noise; the second half is used as
    boundary elements."""
    rng = np.random.default_rng(seed)
    g = np.arange(13) / 12.0
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    out = []
    for t in range(n):
        a = rng.normal(size=6)
        p = (np.sin(a[0] * X + a[1]) * np.cos(a[2] * Y + a[3]) * np.exp(a[4] * Z) + a[5] * X ** 7
             + (rng.normal(size=X.shape) * 1e-3 if t % 2 else 0.0))
        out.append(p)
    return out


def element_wmax(patches_per_var, boundary, tol):
    """isReMeshUnzip's per-element value from given wavelet slots: the
    largest RMS over the variables, stopping once it passes tol
    (include/mesh.tcc:2130-2150)."""
    wm = 0.0
    for wc in patches_per_var:
        l = np.sqrt(np.sum(wc * wc)) / np.sqrt(len(wc))
        wm = max(wm, l)
        if wm > tol:
            break
    return wm
