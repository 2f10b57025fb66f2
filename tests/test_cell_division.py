"""Pair finding splits a cell key into its (x, y, z) cell with a multiply-high and a shift instead of an integer
division (nc_magic in mtg_sys.cuh, div_nc in mtg_device.cuh).  The same multiplier and shift restated here must
give n // nc for every key n < nc^3 and every grid the library builds (nc <= 1024).  The overshoot of the
product grows with n, so the largest key with the largest remainder, nc^3 - 1, is the hardest case; a random
sample of keys is checked as well."""
import numpy as np


def nc_magic(nc: int):
    if nc <= 1:
        return 0, 0
    k = 0
    while (2 << k) < nc:
        k += 1
    return ((1 << (32 + k)) + nc - 1) // nc, k


def div_nc(n, mul, sh):
    return ((np.asarray(n, dtype=np.uint64) * np.uint64(mul)) >> np.uint64(32)) >> np.uint64(sh)


def test_magic_division_is_exact_for_every_cell_key():
    rng = np.random.default_rng(0)
    for nc in range(1, 1025):
        mul, sh = nc_magic(nc)
        assert mul < 2 ** 32
        top = nc ** 3
        keys = np.concatenate([np.array([0, top - 1, top - nc, max(top - nc - 1, 0)]),
                               rng.integers(0, top, size=64)]).astype(np.uint64)
        got = div_nc(keys, mul, sh).astype(np.int64)
        assert np.array_equal(got, keys.astype(np.int64) // nc), nc
        # the second split: q1 = key // nc < nc^2, then q1 // nc
        q1 = keys.astype(np.int64) // nc
        assert np.array_equal(div_nc(q1, mul, sh).astype(np.int64), q1 // nc), nc


def test_every_key_of_small_grids():
    for nc in range(1, 65):
        mul, sh = nc_magic(nc)
        keys = np.arange(nc ** 3, dtype=np.uint64)
        assert np.array_equal(div_nc(keys, mul, sh).astype(np.int64), keys.astype(np.int64) // nc), nc
