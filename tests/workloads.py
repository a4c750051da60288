"""Shared helpers for the tests: synthetic block subsets, host fields, and
the per-field normwise error the reference's own test beds use
(max |a - b| / max |b| over the block interiors, BSSN_GR/src/rhsTestBed.cpp:270-295,
BSSN_GR/cuda_gr/src/gpuTestBed.cpp:408-432)."""
import numpy as np

SEED1 = 20261203 + 1
SEED2 = 20261203 + 2


def repack(dgb, blocks, idx):
    """Blocks idx of a block list, laid out contiguously from offset 0."""
    rows, off = [], 0
    for i in idx:
        b = blocks[i]
        n = b.sz[0] * b.sz[1] * b.sz[2]
        rows.append((off, tuple(b.sz), b.bflag, tuple(b.ptmin), tuple(b.ptmax)))
        off += n
    return dgb.blocks_array(rows)


def host_fields(dgb, blocks, seed, noise=1e-6, nthreads=0):
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(24)]
    dgb.synth_fill_host(blocks, u, seed, noise, nthreads)
    return u


def interior_mask(blocks, n):
    m = np.zeros(n, dtype=bool)
    for b in blocks:
        nx, ny, nz = b.sz
        idx = np.arange(nx * ny * nz).reshape(nz, ny, nx)[3:nz - 3, 3:ny - 3, 3:nx - 3]
        m[b.offset + idx.ravel()] = True
    return m


def normwise(a, b, mask):
    """Per-field max|a-b| / max|b| over masked points."""
    out = []
    for v in range(len(a)):
        den = np.abs(b[v][mask]).max()
        num = np.abs(a[v][mask] - b[v][mask]).max()
        out.append(num / den if den > 0 else num)
    return np.array(out)


def sample_uneven(blocks, per_class=(6, 4, 2, 1)):
    """First few blocks of each size class (13, 19, 31, 61) of the 20k list."""
    want = dict(zip((13, 19, 31, 61), per_class))
    idx = []
    for i, b in enumerate(blocks):
        s = b.sz[0]
        if want.get(s, 0) > 0:
            idx.append(i)
            want[s] -= 1
        if not any(want.values()):
            break
    return idx
