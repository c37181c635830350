"""Grids whose sides are not powers of two, and tiles of 1 and 2 cells.

The reference's FFTW solver takes any nx, ny (src/solver.c:246-330); the
library's field solve then runs mixed-radix passes, tiles are the largest
power of two dividing both sides, and tile indices are divided without a
divide instruction.  Tolerances are those of the power-of-two parity tests:
FP64 positions and velocities bit-exact with the oracle from identical
fields, rho, phi and E within 1e-12 of their max norm, field energy within
1e-10 over the run; mixed form within 1e-5 of the FP64 form's field energy.  Square cells
(Ly = L ny / nx), as the reference's Y weights use dx.
"""
import numpy as np
import pytest

from cpic_gb300 import _lib
from tests import cases

pytestmark = pytest.mark.gpu

L = cases.TWO_PI


def rel_max(a, b):
    den = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / den)


def grid_case(nx, ny, ppc=4, **kw):
    return cases.two_stream(nx=nx, ny=ny, n=nx * ny * ppc, Ly=L * ny / nx, **kw)


@pytest.mark.parametrize("nx,ny", [(48, 40), (40, 40), (96, 80), (30, 18), (25, 15), (77, 13),
                                   (6, 10)])
def test_field_solve_any_size(lib, nx, ny):
    """rho -> phi, E from identical rho: mixed-radix passes (primes 3, 5, 7,
    11, 13), odd ny (a last row alone), odd nx (no Nyquist bin)."""
    case = grid_case(nx, ny, ppc=2)
    g, o = cases.make_gpu(case), cases.make_oracle(case)
    g.pre_step()
    o.pre_step()
    rng = np.random.default_rng(nx * 1000 + ny)
    rho = rng.standard_normal((ny, nx))
    o.set_rho(rho)
    g.set_rho(rho)
    o.stage_field_E()
    g.stage_field_E()
    assert rel_max(g.phi(), o.phi()) <= 1e-12
    gex, gey = g.E()
    oex, oey = o.E()
    assert rel_max(gex, oex) <= 1e-12
    assert rel_max(gey, oey) <= 1e-12


def _one_stage(g, o):
    """Identical fields (the oracle's) -> one fused particle stage on both
    sides (the field solves agree within 1e-12, not bit for bit)."""
    ex, ey = o.E()
    g.set_E(ex, ey)
    o.stage_plasma_E()
    assert o.stage_plasma_r() == 0
    o.stage_field_rho()
    o.iter = o.iter + 1
    g.stage_plasma()


@pytest.mark.parametrize("nx,ny,tile", [(48, 40, 0), (40, 40, 8), (30, 18, 0), (25, 15, 0),
                                        (96, 80, 16)])
def test_fp64_stages_bitexact(lib, nx, ny, tile):
    """From identical fields: particles bit-exact after the half kick and two
    full particle stages, rho within 1e-12, per-cell counts exact."""
    case = grid_case(nx, ny)
    g = cases.make_gpu(case, tile=tile)
    o = cases.make_oracle(case)
    g.pre_step()
    o.pre_step()
    assert rel_max(g.rho(), o.rho()) <= 1e-12
    for it in range(3):
        _one_stage(g, o)
        for a, b in zip(g.particles(0), o.particles(0)):
            assert np.array_equal(a, b), "iteration %d" % it
        assert rel_max(g.rho(), o.rho()) <= 1e-12
        assert np.array_equal(g.cell_counts(), o.cell_counts())
        o.stage_field_E()
    g.close()


@pytest.mark.parametrize("nx,ny,tile", [(48, 40, 0), (25, 15, 0)])
def test_fp64_field_energy(lib, nx, ny, tile):
    """Whole steps, each side with its own field solve: field energy within
    1e-10 of the oracle's over 60 steps."""
    case = grid_case(nx, ny)
    g = cases.make_gpu(case, tile=tile)
    o = cases.make_oracle(case)
    g.pre_step()
    o.pre_step()
    worst = 0.0
    for _ in range(60):
        g.step()
        o.step()
        we_g, we_o = g.diag()["WE"], o.diag()["WE"]
        worst = max(worst, abs(we_g - we_o) / we_o)
    assert worst <= 1e-10, worst
    g.close()


@pytest.mark.parametrize("nx,ny", [(48, 40), (25, 15)])
def test_mixed_field_energy(lib, nx, ny):
    """The mixed form on the same grids (cells wrapped without a mask)
    against the FP64 form."""
    case = grid_case(nx, ny, ppc=16)
    f = cases.make_gpu(case)
    m = cases.make_gpu(case, precision=_lib.MIXED)
    f.pre_step()
    m.pre_step()
    worst = 0.0
    for _ in range(60):
        f.step()
        m.step()
        a, b = m.diag()["WE"], f.diag()["WE"]
        worst = max(worst, abs(a - b) / b)
    assert worst <= 1e-5, worst
    f.close()
    m.close()


def test_field_tile_copy_mode(lib):
    """The mixed form stages field tiles with 2D tensor copies when tiles
    have an even width; tiles of one cell, odd grids and the FP64 form
    (E read from global memory) load by threads."""
    even = cases.two_stream(nx=32, ny=32, n=32 * 32 * 2)
    odd = grid_case(25, 15, ppc=2)
    for case, precision, tile, want in ((even, _lib.MIXED, 16, 1), (even, _lib.MIXED, 2, 1),
                                        (even, _lib.MIXED, 1, 0), (odd, _lib.MIXED, 0, 0),
                                        (even, _lib.FP64, 16, 0)):
        c = cases.make_gpu(case, precision=precision, tile=tile)
        assert c.field_tile_copy() == want, (precision, tile)
        c.close()


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_tile_size_changes_nothing(lib, precision):
    """The same plasma with tiles of 1, 2, 4 and 16 cells: identical
    particles and fields (the deposit is exact integer arithmetic and the
    gather reads the same E, so the tiling is invisible; in the mixed form
    the one-cell tiles load their field by threads, the others by 2D tensor
    copies apart from the tiles of the grid's last column and row)."""
    case = cases.two_stream(nx=32, ny=32, n=32 * 32 * 8)
    runs = []
    for tile in (1, 2, 4, 16):
        c = cases.make_gpu(case, precision=precision, tile=tile)
        c.pre_step()
        c.run(12)
        runs.append((c.particles(0), c.rho()))
        c.close()
    p0, r0 = runs[0]
    for p, r in runs[1:]:
        for a, b in zip(p, p0):
            assert np.array_equal(a, b)
        assert np.array_equal(r, r0)
