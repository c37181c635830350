"""Upload sort (cpic_add_species): after the two-pass counting sort every
tile holds exactly the particles of its cells, those moving left (ux < 0)
before those moving right, and no particle is lost or altered (FP64 form:
bit-exact; mixed form: exact after the cell + offset conversion).  The
store order is visible through cpic_get_particles in the mixed form
without ids; the FP64 store always keeps ids, so its download comes back
in upload order."""
import math

import numpy as np
import pytest

from cpic_gb300 import _lib

pytestmark = pytest.mark.gpu
L = 2 * math.pi


def _state(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, L, n)
    y = rng.uniform(-0.5, L + 0.5, n)            # one periodic wrap in Y
    # clustered in a corner as well, so tiles and rows differ widely in size
    k = n // 4
    x[:k] = rng.uniform(0, L / 16, k)
    y[:k] = rng.uniform(0, L / 16, k)
    ux = rng.normal(0, 0.3, n)
    uy = rng.normal(0, 0.3, n)
    # signs the sort must classify like its histogram: zeros of both
    # signs and values that round to -0.0 in FP32
    ux[1::97] = 0.0
    ux[2::97] = -0.0
    ux[3::97] = -1e-50
    ux[4::97] = 1e-50
    return x, y, ux, uy


def _expected(x, y, ux, uy, prec):
    y = np.where(y >= L, y - L, np.where(y < 0, y + L, y))
    if prec == _lib.MIXED:
        # what the mixed store holds: cell + FP32 offset, FP32 velocity
        dx = L / 64
        idx = 1.0 / dx                          # as the library scales
        px, py = x * idx, y * idx
        fx, fy = np.floor(px), np.floor(py)
        ox = (px - fx).astype(np.float32).astype(np.float64)
        oy = (py - fy).astype(np.float32).astype(np.float64)
        cx = np.where(ox >= 1.0, fx + 1, fx) % 64
        cy = np.where(oy >= 1.0, fy + 1, fy) % 64
        ox = np.where(ox >= 1.0, 0.0, ox)
        oy = np.where(oy >= 1.0, 0.0, oy)
        x, y = (cx + ox) * dx, (cy + oy) * dx
        ux = ux.astype(np.float32).astype(np.float64)
        uy = uy.astype(np.float32).astype(np.float64)
    return x, y, ux, uy


@pytest.mark.parametrize("prec", [_lib.FP64, _lib.MIXED], ids=["fp64", "mixed"])
def test_upload_sort_layout(lib, prec):
    n = 300000
    x, y, ux, uy = _state(n, 5)
    c = _lib.Context(64, 64, L, L, 0.05, 1.0, precision=prec, tile=8, halo=1,
                     track_ids=prec == _lib.FP64)
    c.add_species(-L * L / n, L * L / n, x, y, ux, uy)
    gx, gy, gu, gv = c.particles(0)
    ex, ey, eu, ev = _expected(x, y, ux, uy, prec)
    counts = c.cell_counts().reshape(64, 64)
    if prec == _lib.FP64:
        # by id: every particle unchanged; and the cells hold them all
        for a, b in zip((gx, gy, gu, gv), (ex, ey, eu, ev)):
            assert np.array_equal(a, b)
        assert counts.sum() == n
        c.close()
        return

    # mixed form without ids: store order, tile by tile
    # the same multiset of particles
    got = np.stack([gx, gy, gu, gv])
    exp = np.stack([ex, ey, eu, ev])
    go = np.lexsort(got[::-1])
    eo = np.lexsort(exp[::-1])
    assert np.array_equal(got[:, go], exp[:, eo])

    # tile by tile, in tile order, every particle inside its tile's cells
    tiles = counts.reshape(8, 8, 8, 8).sum(axis=(1, 3)).ravel()   # [ty, tx]
    dx = L / 64
    start = 0
    for t in range(64):
        seg = slice(start, start + int(tiles[t]))
        ty, tx = divmod(t, 8)
        px, py = gx[seg] / dx, gy[seg] / dx
        assert np.all((px >= 8 * tx - 1e-6) & (px < 8 * tx + 8 + 1e-6)), t
        assert np.all((py >= 8 * ty - 1e-6) & (py < 8 * ty + 8 + 1e-6)), t
        # left movers first: the test the sort uses (ux >= 0 is "right")
        right = gu[seg] >= 0
        assert np.all(np.diff(right.astype(np.int8)) >= 0), t
        start += int(tiles[t])
    assert start == n
    c.close()
