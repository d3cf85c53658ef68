"""The multiply-high division the learned far field's cell kernel uses for cell
coordinates inside a bin (k_surrogate_cells, struct Magic): q = floor(n m / 2^32)
with m = floor((2^32 - 1) / d) + 1 equals n // d for every divisor d <= 1024
(bin rows and slabs of at most 32 x 32 cells) and every cell index n < 32768
(bins of at most 32^3 cells); d = 1 is passed through unchanged."""
import numpy as np


def test_magic_division_exact_over_the_kernel_ranges():
    n = np.arange(32768, dtype=np.uint64)
    for d in range(2, 1025):
        m = np.uint64((2 ** 32 - 1) // d + 1)
        q = (n * m) >> np.uint64(32)
        assert np.array_equal(q, n // np.uint64(d)), d
