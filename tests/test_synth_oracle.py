"""The oracle's copy of the synthetic workload generator (oracle/synth_oracle.c),
which the benchmark's CPU arms use so that they run without the CUDA
library, against the library's generator; and the host-tuned timing build of
the oracle (liboracle_bench.so) against the portable one."""
import numpy as np

from workloads import repack


def test_block_lists_equal_library(dgb, oracle):
    for which, seed in ((1, 0), (2, 20261205), (2, 7)):
        a = dgb.synth_blocks(which, seed)
        b = oracle.synth_blocks(which, seed, dgb.BlockDesc)
        assert len(a) == len(b) and bytes(a) == bytes(b), (which, seed)


def test_fill_equals_library(dgb, oracle):
    blocks = repack(dgb, dgb.synth_blocks(2, 20261205), range(0, 20000, 500))
    n = dgb.unzipped_size(blocks)
    for nv in (24, 25):
        u1 = [np.zeros(n) for _ in range(nv)]
        u2 = [np.zeros(n) for _ in range(nv)]
        dgb.synth_fill_host(blocks, u1, 77, 1e-6)
        oracle.synth_fill(blocks, u2, 77, 1e-6)
        assert all(np.array_equal(x, y) for x, y in zip(u1, u2))


def test_timing_build_gives_the_same_bits(dgb, oracle):
    import oracle_py
    fast = oracle_py.Oracle(oracle_py.ORACLE_BENCH_SO)
    blocks = repack(dgb, dgb.synth_blocks(2, 20261205), range(0, 20000, 2000))
    n = dgb.unzipped_size(blocks)
    u = [np.zeros(n) for _ in range(24)]
    oracle.synth_fill(blocks, u, 5, 1e-6)
    prm = dgb.params_vector(dgb.default_params(0.1))
    r1 = [np.zeros(n) for _ in range(24)]
    r2 = [np.zeros(n) for _ in range(24)]
    assert oracle.bssnrhs_blocks(r1, u, blocks, prm, 2) == 0
    assert fast.bssnrhs_blocks(r2, u, blocks, prm, 2) == 0
    assert all(np.array_equal(x, y) for x, y in zip(r1, r2))
