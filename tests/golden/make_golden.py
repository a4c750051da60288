#!/usr/bin/env python3
"""Generate the golden vectors in this folder from the REFERENCE's own code.

Runs only where the reference tree exists: oracle/Makefile.ref compiles the
reference's sources (QuadGrav/src/derivs.cpp, the generated
BSSN_GR/scripts/bssnrhs_*.h drivers and
BSSN_GR/src/bssneqs_eta_const_standard_gauge.cpp inside the bssnrhs harness
oracle/ref_bssnrhs.cpp, BSSN_GR/src/bssn_constraints.cpp, and the constraint
diagnostics BSSN_GR/scripts/constraint_derivs.h + BSSN_GR/src/physconeqs.cpp
inside oracle/ref_physcon.cpp, and the CCZ4 right-hand side
CCZ4_GR/src/derivs.cpp + the generated CCZ4_GR/scripts/ccz4rhs_*.h drivers +
CCZ4_GR/src/ccz4eqs.cpp inside oracle/ref_ccz4rhs.cpp).

Inputs come from the library's seeded synthetic generator (host fill); their
SHA-256 is stored so that a change of the generator is detected.

  python tests/golden/make_golden.py
"""
import hashlib
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle_py  # noqa: E402
from workloads import SEED1, interior_mask, repack  # noqa: E402

# uniform 13^3 blocks: 288 holds the puncture at x = -1, 0 is a corner block
RHS_BLOCKS = [288, 0]
SIGMA = 0.1


def load_dgb():
    spec = importlib.util.spec_from_file_location("dgb", os.path.join(ROOT, "dendro-5.01_gb300",
                                                                     "dgb.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def sha(arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def constraint_state(n=64, seed=11):
    """A perturbed BSSN state for enforce_bssn_constraints (det != 1, trace != 0)."""
    rng = np.random.default_rng(seed)
    v = [rng.normal(0.0, 1e-2, n) for _ in range(24)]
    for q in (12, 15, 17):
        v[q] += 1.0
    v[0] += 0.6
    v[1] += 0.4
    v[1][:4] = 1e-6  # chi below the floor
    v[0][4:8] = -0.1  # alpha below the floor
    return v


def main():
    dgb = load_dgb()
    oracle_py.build_ref()
    ref = oracle_py.Reference()
    blocks = repack(dgb, dgb.synth_blocks(1), RHS_BLOCKS)
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, u, SEED1, 1e-6)
    prm = dgb.params_vector(dgb.default_params(SIGMA))
    r = [np.zeros(n) for _ in range(24)]
    for b in blocks:
        assert ref.bssnrhs(r, u, b, prm) == 0
    mask = interior_mask(blocks, n)
    rhs = np.stack([x[mask] for x in r])

    # reference stencils on one field (chi) of the puncture block
    b0 = blocks[0]
    sz = tuple(b0.sz)
    chi = u[1][:sz[0] * sz[1] * sz[2]].reshape(sz[2], sz[1], sz[0])
    h = (b0.ptmax[0] - b0.ptmin[0]) / (sz[0] - 1)
    st = {}
    for kind in ("d1", "d2", "ko"):
        for d in range(3):
            st[f"{kind}_{d}"] = ref.stencil(kind, d, chi, h)[3:-3, 3:-3, 3:-3].copy()

    cs = constraint_state()
    out = [x.copy() for x in cs]
    for node in range(len(out[0])):
        ref.enforce(out, node, 1e-4)

    np.savez_compressed(
        os.path.join(HERE, "bssn_reference.npz"),
        rhs_blocks=np.array(RHS_BLOCKS), rhs_seed=np.array(SEED1), rhs_sigma=np.array(SIGMA),
        rhs_input_sha256=np.array(sha(u)), rhs=rhs,
        stencil_h=np.array(h), **{f"stencil_{k}": v for k, v in st.items()},
        enforce_in=np.stack(cs), enforce_out=np.stack(out), enforce_chi_floor=np.array(1e-4))
    print("wrote", os.path.join(HERE, "bssn_reference.npz"))
    constraint_goldens(dgb, ref)
    ccz4_goldens(dgb)
    bssn42_goldens(dgb, ref)


def shifted_fields(dgb, blocks, seed):
    """Seeded synthetic fields with an oscillating shift of size 0.3 added,
    so that every upwinded stencil form is taken."""
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, u, seed, 1e-6)
    for d in range(3):
        u[6 + d] += 0.3 * np.sin(np.arange(n) * (0.37 + d))
    return u


def bssn42_goldens(dgb, ref):
    """bssnrhs with the BSSN_GR solver's own binding (deriv42, upwinded
    deriv42adv, ko_deriv42; BSSN_GR/include/rhs.h:23-37) from the reference
    build (oracle/ref_bssnrhs42.cpp) on the puncture block, a generic block
    and two domain-boundary corner blocks (closures and bssn_bcs)."""
    allb = dgb.synth_blocks(1)
    picks = [(288, 0), (100, 0), (0, 1 | 4 | 16), (511, 2 | 8 | 32)]
    rows, off = [], 0
    for i, f in picks:
        b = allb[i]
        rows.append((off, tuple(b.sz), f, tuple(b.ptmin), tuple(b.ptmax)))
        off += b.sz[0] * b.sz[1] * b.sz[2]
    blocks = dgb.blocks_array(rows)
    u = shifted_fields(dgb, blocks, SEED1)
    n = len(u[0])
    prm = dgb.params_vector(dgb.default_params(SIGMA))
    r = [np.zeros(n) for _ in range(24)]
    for b in blocks:
        assert ref.bssnrhs(r, u, b, prm, order=4) == 0
    mask = interior_mask(blocks, n)
    np.savez_compressed(
        os.path.join(HERE, "bssn42_reference.npz"), picks=np.array(picks), seed=np.array(SEED1),
        sigma=np.array(SIGMA), input_sha256=np.array(sha(u)), rhs=np.stack([x[mask] for x in r]))
    print("wrote", os.path.join(HERE, "bssn42_reference.npz"))


def axis_block(dgb, blocks):
    """First uniform block with interior points on the z axis (x = y = 0)."""
    for i, b in enumerate(blocks):
        h = [(b.ptmax[d] - b.ptmin[d]) / (b.sz[d] - 1) for d in range(3)]
        ok = [any(abs(b.ptmin[d] + k * h[d]) <= 1e-7 for k in range(3, b.sz[d] - 3))
              for d in (0, 1)]
        if all(ok):
            return i
    raise RuntimeError("no block on the axis")


def constraint_goldens(dgb, ref):
    """physical_constraints (BSSN_GR/src/physcon.cpp) of the reference on the
    puncture block, a generic block, a block on the z axis (the Psi4 guard)
    and a domain-boundary corner block (one-sided 4th-order closures)."""
    allb = dgb.synth_blocks(1)
    picks = [(288, 0), (100, 0), (axis_block(dgb, allb), 0), (0, 1 | 4 | 16), (511, 2 | 8 | 32)]
    rows, off = [], 0
    for i, f in picks:
        b = allb[i]
        rows.append((off, tuple(b.sz), f, tuple(b.ptmin), tuple(b.ptmax)))
        off += b.sz[0] * b.sz[1] * b.sz[2]
    blocks = dgb.blocks_array(rows)
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, u, SEED1, 1e-6)
    c = [np.zeros(n) for _ in range(6)]
    for b in blocks:
        assert ref.physical_constraints(c, u, b) == 0
    mask = interior_mask(blocks, n)
    b0 = blocks[0]
    sz = tuple(b0.sz)
    chi = u[1][:sz[0] * sz[1] * sz[2]].reshape(sz[2], sz[1], sz[0])
    h = (b0.ptmax[0] - b0.ptmin[0]) / (sz[0] - 1)
    st = {}
    for kind in ("d1_4", "d2_4"):
        for d in range(3):
            st[f"stencil_{kind}_{d}"] = ref.stencil(kind, d, chi, h, 0)[3:-3, 3:-3, 3:-3].copy()
    np.savez_compressed(
        os.path.join(HERE, "constraints_reference.npz"),
        picks=np.array(picks), seed=np.array(SEED1), input_sha256=np.array(sha(u)),
        cons=np.stack([x[mask] for x in c]), stencil_h=np.array(h), **st)
    print("wrote", os.path.join(HERE, "constraints_reference.npz"))


def ccz4_goldens(dgb):
    """ccz4rhs (CCZ4_GR/src/rhs.cpp:12-298, stencils of CCZ4_GR/src/derivs.cpp)
    of the reference on the puncture block, a generic block and two
    domain-boundary corner blocks (one-sided stencils; the harness has no
    ccz4_bcs), and its upwind / KO stencils on one field."""
    cref = oracle_py.CCZ4Reference()
    allb = dgb.synth_blocks(1)
    picks = [(288, 0), (100, 0), (0, 1 | 4 | 16), (511, 2 | 8 | 32)]
    rows, off = [], 0
    for i, f in picks:
        b = allb[i]
        rows.append((off, tuple(b.sz), f, tuple(b.ptmin), tuple(b.ptmax)))
        off += b.sz[0] * b.sz[1] * b.sz[2]
    blocks = dgb.blocks_array(rows)
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(25)]
    dgb.synth_fill_host(blocks, u, SEED1, 1e-6)
    prm = dgb.ccz4_params_vector(dgb.default_ccz4_params())
    r = [np.zeros(n) for _ in range(25)]
    for b in blocks:
        assert cref.ccz4rhs(r, u, b, prm) == 0
    mask = interior_mask(blocks, n)
    b0 = blocks[0]
    sz = tuple(b0.sz)
    npt = sz[0] * sz[1] * sz[2]
    gt1 = u[13][:npt].reshape(sz[2], sz[1], sz[0])
    beta = [u[6 + d][:npt].reshape(sz[2], sz[1], sz[0]) for d in range(3)]
    h = (b0.ptmax[0] - b0.ptmin[0]) / (sz[0] - 1)
    st = {}
    for d in range(3):
        st[f"stencil_adv_{d}"] = cref.adv(d, gt1, h, beta[d], 0)[3:-3, 3:-3, 3:-3].copy()
        st[f"stencil_ko_{d}"] = cref.stencil("ko_ccz4", d, gt1, h, 0)[3:-3, 3:-3, 3:-3].copy()
    np.savez_compressed(
        os.path.join(HERE, "ccz4_reference.npz"),
        picks=np.array(picks), seed=np.array(SEED1), params=prm, input_sha256=np.array(sha(u)),
        rhs=np.stack([x[mask] for x in r]), stencil_h=np.array(h), **st)
    print("wrote", os.path.join(HERE, "ccz4_reference.npz"))


def mesh_goldens(dgb):
    """The reference's own ot::Mesh (oracle/ref_mesh.cpp over src/mesh.cpp,
    include/mesh.tcc, src/octUtils.cpp, FEM/src/refel.cpp ...) built from
    this library's level-6 octree: its element order, block list
    (octree2BlockDecomposition + performBlocksSetup), CG numbering (owner
    element and place in it, Mesh::buildE2NMap), Mesh::unzip of a smooth
    field (full padded grids of a few blocks and per-block checksums of all)
    and Mesh::zip of a seeded unzipped vector (checksum and head), the
    reference's Hilbert tables (src/hcurvedata.cpp), and the wavelets of
    WaveletEl on seeded patches and on every element's unzipped patch."""
    import ctypes as C

    from meshref import (GOLDEN_FULL_BLOCKS, GOLDEN_MESH, checksums, field,
                         leaves_in_octree_units, wavelet_test_patches)
    mesh = dgb.Mesh(dgb.mesh_params(**GOLDEN_MESH))
    anc, lev, md = leaves_in_octree_units(mesh)
    R = oracle_py.MeshReference().build(anc, lev, md)
    bl = R.blocks()
    el = R.elements()
    own = R.zip_owner()
    xyz = R.cg_coords()
    key = np.rint(xyz * 6).astype(np.int64)
    ex = el[own].astype(np.int64)
    ln = 1 << (md - ex[:, 3])
    loc = np.stack([(key[:, a] - 6 * ex[:, a]) // ln for a in range(3)], axis=1)
    local = loc[:, 0] + 7 * (loc[:, 1] + 7 * loc[:, 2])
    # unzip of the smooth field given at the reference's own CG nodes
    f = field(xyz / (1 << md) * 64.0 - 32.0)
    uz = R.unzip(f)
    cs = checksums(uz, bl[:, [0, 1, 2, 5, 6, 7, 8, 9]])
    # full grids: the domain-corner block, the blocks with most and fewest
    # NaN-free points that take interpolated values ... chosen by a fixed rule
    sizes = bl[:, 5]
    small = np.nonzero(sizes == 13)[0]
    mid = np.nonzero(sizes == 19)[0]
    picks = [int(small[0]), int(small[len(small) // 2]), int(small[-1]), int(mid[len(mid) // 2])]
    assert len(picks) == GOLDEN_FULL_BLOCKS
    full = np.concatenate([uz[bl[i, 8]:bl[i, 8] + bl[i, 5] * bl[i, 6] * bl[i, 7]] for i in picks])
    rng = np.random.default_rng(7)
    u = rng.standard_normal(R.nunzipped)
    z = R.zip(u)
    # WaveletEl::compute_wavelets_3D (src/waveletRefEl.cpp:92-271) on seeded
    # patches (interior, then boundary), and per element of the mesh the
    # reference's own patch (getUnzipElementalNodalValues) wavelets of the
    # smooth field and of chi-like 1/(1+r) data
    wp = wavelet_test_patches()
    half = len(wp) // 2
    wav = np.stack([R.wavelets(p.ravel(), (13, 13, 13), i >= half) for i, p in enumerate(wp)])
    elem, patches, bdy = R.element_patches(uz)
    rms = np.array([np.sqrt(np.sum(w * w)) / 8.0 for w in
                    (R.wavelets(patches[q], (13, 13, 13), bool(bdy[q])) for q in range(len(elem)))])
    rot = C.cast(C.c_void_p.in_dll(R.L, "rotations"), C.POINTER(C.c_char))
    ht = C.cast(C.c_void_p.in_dll(R.L, "HILBERT_TABLE"), C.POINTER(C.c_char))
    rot_t = np.array([[rot[r * 16 + i][0] - 48 for i in range(16)] for r in range(24)], np.uint8)
    ht_t = np.array([[ht[r * 8 + c][0] for c in range(8)] for r in range(24)], np.uint8)
    np.savez_compressed(
        os.path.join(HERE, "mesh_reference.npz"),
        octree_depth=np.array(md), leaves=np.column_stack([anc, lev]).astype(np.uint32),
        elements=el, blocks=bl, cg_owner_step=np.diff(own, prepend=0).astype(np.uint8),
        cg_local=local.astype(np.int16), unzip_checksums=cs, unzip_full_blocks=np.array(picks),
        unzip_full=full, zip_seed=np.array(7), zip_sum=np.array(np.sum(z)),
        zip_wsum=np.array(np.sum(z * np.cos(0.7 * np.arange(len(z))))), zip_head=z[:4096],
        hilbert_rotations=rot_t, hilbert_table=ht_t,
        wavelet_patch_seed=np.array(5), wavelet_wc=wav, element_order=elem.astype(np.int32),
        element_boundary=bdy, element_wavelet_rms=rms)
    R.close()
    print("wrote", os.path.join(HERE, "mesh_reference.npz"))


if __name__ == "__main__":
    if sys.argv[1:] == ["mesh"]:
        oracle_py.build_ref()
        mesh_goldens(load_dgb())
    elif sys.argv[1:] == ["bssn42"]:
        oracle_py.build_ref()
        bssn42_goldens(load_dgb(), oracle_py.Reference())
    else:
        main()
        mesh_goldens(load_dgb())
