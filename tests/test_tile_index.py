"""The tile kernels' division-free index split (csrc/tile_index.cuh): with
m = ceil(2^31 / n), floor(2q * m / 2^32) = floor(q / n) for every region index
q < 2^13 and extent n < 32 the kernels use (checked exhaustively, the same
32-bit arithmetic as the device code)."""
import numpy as np


def test_fixed_point_division_is_exact():
    q = np.arange(1 << 13, dtype=np.uint64)
    for n in range(1, 32):
        m = np.uint64((0x80000000 + n - 1) // n)
        assert m < (1 << 32)
        hi = ((q << np.uint64(1)) * m) >> np.uint64(32)  # __umulhi((uint32_t)q << 1, m)
        assert np.array_equal(hi, q // np.uint64(n)), n
