"""The cell sort's key tables (k_key_table in sort.cu).

The tile-major key of cell (ix, iy, iz) with tile shape (TX, TY, TZ) is
  tile * C + lx + TX * (ly + TY * lz),   tile = tx + NTX * (ty + NTY * tz),
with (tx, lx) = divmod(ix, TX) and so on, C = TX * TY * TZ.  The single-context
sort looks it up as the sum of one term per axis; these tests check that the
sum of the three table terms is that key for every cell, and that the keys are a
permutation of 0 .. ncell-1 (so the counting sort's scan covers every slot).
"""
import numpy as np
import pytest


def tile_key(n, t, ix, iy, iz):
    ntx, nty = n[0] // t[0], n[1] // t[1]
    C = t[0] * t[1] * t[2]
    tx, lx = divmod(ix, t[0])
    ty, ly = divmod(iy, t[1])
    tz, lz = divmod(iz, t[2])
    return (tx + ntx * (ty + nty * tz)) * C + lx + t[0] * (ly + t[1] * lz)


def key_table(n, t):
    """The nx + ny + nz terms k_key_table writes."""
    ntx, nty = n[0] // t[0], n[1] // t[1]
    C = t[0] * t[1] * t[2]
    kx = [(i // t[0]) * C + i % t[0] for i in range(n[0])]
    ky = [(i // t[1]) * ntx * C + t[0] * (i % t[1]) for i in range(n[1])]
    kz = [(i // t[2]) * ntx * nty * C + t[0] * t[1] * (i % t[2]) for i in range(n[2])]
    return np.array(kx), np.array(ky), np.array(kz)


@pytest.mark.parametrize("n,t", [((16, 8, 8), (16, 8, 8)), ((32, 16, 24), (8, 8, 4)), ((48, 24, 16), (16, 8, 8)),
                                 ((24, 24, 24), (12, 8, 6)), ((64, 32, 16), (4, 4, 4))])
def test_table_sum_is_the_tile_major_key(n, t):
    kx, ky, kz = key_table(n, t)
    keys = kx[None, None, :] + ky[None, :, None] + kz[:, None, None]    # [z][y][x]
    iz, iy, ix = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    want = tile_key(n, t, ix, iy, iz)
    assert np.array_equal(keys, want)
    assert np.array_equal(np.sort(keys.ravel()), np.arange(n[0] * n[1] * n[2]))


def test_largest_grid_keys_fit_32_bits():
    n, t = (2048, 2048, 1024), (16, 8, 8)
    kx, ky, kz = key_table(n, t)
    assert int(kx.max() + ky.max() + kz.max()) == n[0] * n[1] * n[2] - 1 <= 0xFFFFFFFF
