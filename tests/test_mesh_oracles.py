"""The two host restatements of the unzip operator (C in oracle/bssn_oracle.c,
numpy in oracle/oracle_py.py) agree on a mesh with several refinement
levels."""
import numpy as np


def test_c_and_numpy_unzip_agree(dgb):
    import oracle_py
    m = dgb.Mesh(dgb.mesh_params(max_level=7, min_level=3, fine_radius=1.0))
    op = m.operator()
    z = np.random.default_rng(4).normal(size=m.ndof)
    a = oracle_py.unzip_apply(op, z, m.nunzipped)
    b = oracle_py.unzip_apply_numpy(op, z, m.nunzipped)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(a)
    assert np.abs(a[ok] - b[ok]).max() <= 1e-12 * np.abs(b[ok]).max()
