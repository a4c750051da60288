"""The library's octree mesh against the reference's own ot::Mesh.

oracle/Makefile.ref builds the reference's mesh (src/mesh.cpp,
include/mesh.tcc, src/octUtils.cpp, FEM/src/refel.cpp ...) with a
single-rank MPI stand-in and an own dgesv_ into oracle/_ref/libmesh_ref.so;
tests/golden/mesh_reference.npz holds what it gave on a level-6 octree
(tests/golden/make_golden.py).  Both are handed this library's leaves.  Bars:
element order, block list (node, sizes, offsets, face flags, order), CG
numbering and zip identical; unzip within 1e-14 normwise (the interpolation
weights here are exact Lagrange weights rounded once, the reference's come
from a LAPACK solve) with the same untouched padding beyond the domain."""
import os

import numpy as np
import pytest

from meshref import (GOLDEN_MESH, block_rows, cg_keys_from_mesh, cg_keys_from_octree, checksums,
                     field, leaves_in_octree_units)
from oracle_py import MESH_REF_SO, REF_ROOT, unzip_apply

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "mesh_reference.npz")
UNZIP_TOL = 1e-14


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def mesh6(dgb):
    return dgb.Mesh(dgb.mesh_params(**GOLDEN_MESH))


def normwise(a, b):
    fin = np.isfinite(b)
    return np.max(np.abs(a[fin] - b[fin])) / np.max(np.abs(b[fin]))


def test_hilbert_curve_is_the_references(dgb, golden):
    """The curve generated from its base order and child symmetries visits
    children and passes states exactly as the reference's tables
    (src/hcurvedata.cpp, as built) do, state for state from the root."""
    order, nxt = dgb.hilbert_tables()
    rot, ht = golden["hilbert_rotations"], golden["hilbert_table"]
    assert order.shape == (24, 8)
    seen, stack = set(), [(0, 0)]
    while stack:
        mine, ref = stack.pop()
        if (mine, ref) in seen:
            continue
        seen.add((mine, ref))
        assert list(order[mine]) == list(rot[ref, :8])
        for c in range(8):
            stack.append((int(nxt[mine, c]), int(ht[ref, c])))
    assert len(seen) == 24


def test_mesh_equals_reference_goldens(dgb, golden, mesh6):
    anc, lev, md = leaves_in_octree_units(mesh6)
    assert md == int(golden["octree_depth"])
    # same input octree as the goldens were made from, in the reference's element order
    assert np.array_equal(np.column_stack([anc, lev]), golden["leaves"])
    assert np.array_equal(np.column_stack([anc, lev]), golden["elements"])
    # block list: node, sizes, offsets, face flags, in the same order
    ref_rows = golden["blocks"][:, [0, 1, 2, 5, 6, 7, 8, 9]]
    assert np.array_equal(block_rows(mesh6), ref_rows)
    assert mesh6.nunzipped == int(ref_rows[-1, 6] + np.prod(ref_rows[-1, 3:6]))
    # CG numbering: owner element (coarsest, first in element order) and place in it
    own = np.cumsum(golden["cg_owner_step"].astype(np.int64))
    el = golden["elements"].astype(np.int64)[own]
    local = golden["cg_local"].astype(np.int64)
    ln = 1 << (md - el[:, 3])
    loc = np.stack([local % 7, (local // 7) % 7, local // 49], axis=1)
    ref_keys = 6 * el[:, :3] + loc * ln[:, None]
    assert np.array_equal(cg_keys_from_mesh(mesh6), ref_keys)
    # unzip of the smooth field on this library's nodes (= the reference's nodes)
    op = mesh6.operator()
    uz = unzip_apply(op, field(mesh6.dof_coords()), mesh6.nunzipped)
    off = 0
    full = golden["unzip_full"]
    for b in golden["unzip_full_blocks"]:
        r = ref_rows[int(b)]
        n = int(np.prod(r[3:6]))
        mine, ref = uz[r[6]:r[6] + n], full[off:off + n]
        off += n
        assert np.array_equal(np.isfinite(mine), np.isfinite(ref))
        assert normwise(mine, ref) <= UNZIP_TOL
    cs_ref = golden["unzip_checksums"]
    cs = checksums(uz, ref_rows)
    assert np.array_equal(cs[:, 0], cs_ref[:, 0])  # untouched points beyond the domain
    scale = np.max(np.abs(cs_ref[:, 1:]))
    assert np.max(np.abs(cs[:, 1:] - cs_ref[:, 1:])) <= 1e-13 * scale
    # zip: each node read from its owner's block
    rng = np.random.default_rng(int(golden["zip_seed"]))
    u = rng.standard_normal(mesh6.nunzipped)
    z = u[op["zip_src"].astype(np.int64)]
    assert np.array_equal(z[:4096], golden["zip_head"])
    assert np.sum(z) == golden["zip_sum"]
    assert np.sum(z * np.cos(0.7 * np.arange(len(z)))) == golden["zip_wsum"]


@pytest.fixture(scope="module")
def refmesh():
    import oracle_py
    if not os.path.isdir(REF_ROOT) and not os.path.exists(MESH_REF_SO):
        pytest.skip("reference tree not present on this machine")
    oracle_py.build_ref()
    return oracle_py.MeshReference()


@pytest.mark.parametrize("case", [
    dict(max_level=8, min_level=4, fine_radius=1.0),                  # depth 12
    dict(max_level=7, min_level=3, fine_radius=0.5, octree_depth=16),  # 2^32-unit nodes split
    dict(max_level=6, min_level=2, fine_radius=2.0, octree_depth=9,
         punctures=((3.0, -5.0, 0.7),)),                              # one off-centre puncture
])
def test_mesh_equals_reference_live(dgb, refmesh, case):
    """The same comparison against the reference built here, on more octrees
    and octree depths, with the whole unzipped vector compared."""
    mesh = dgb.Mesh(dgb.mesh_params(**case))
    anc, lev, md = leaves_in_octree_units(mesh)
    R = refmesh.build(anc, lev, md)
    assert np.array_equal(R.elements(), np.column_stack([anc, lev]))
    ref_rows = R.blocks()[:, [0, 1, 2, 5, 6, 7, 8, 9]]
    assert np.array_equal(block_rows(mesh), ref_rows)
    xyz = R.cg_coords()
    assert np.array_equal(cg_keys_from_mesh(mesh), cg_keys_from_octree(xyz))
    f = field(mesh.dof_coords())
    op = mesh.operator()
    mine = unzip_apply(op, f, mesh.nunzipped)
    ref = R.unzip(f)
    assert np.array_equal(np.isfinite(mine), np.isfinite(ref))
    assert normwise(mine, ref) <= UNZIP_TOL
    u = np.random.default_rng(3).standard_normal(mesh.nunzipped)
    assert np.array_equal(u[op["zip_src"].astype(np.int64)], R.zip(u))
