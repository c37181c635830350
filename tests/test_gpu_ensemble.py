"""Ensembles: independent runs of different grids and particle counts
stepped together by one CUDA graph give exactly the results of the same
runs stepped one by one (the graph replays the same launches), including
across a tile-layout rebuild (which forces a new capture); the autotuner
returns a tile that fits the grid."""
import math

import numpy as np
import pytest

from cpic_gb300 import _lib

pytestmark = pytest.mark.gpu
L = 2 * math.pi


def _member(grid, ppc, v0, amp, seed, prec):
    n = grid * grid * ppc
    x, y, ux, uy = _lib.init_two_stream(seed, 0, n, L, L, v0, 0.0, amp)
    q = -L * L / n
    c = _lib.Context(grid, grid, L, L, 0.05, 1.0, precision=prec)
    c.add_species(q, -q, x, y, ux, uy)
    c.pre_step()
    return c


MEMBERS = [(32, 8, 0.1, 0.05, 1), (64, 37, 0.25, 0.01, 2), (128, 16, 0.4, 0.001, 3),
           (32, 128, 0.3, 0.02, 4), (256, 9, 0.2, 0.03, 5), (64, 100, 0.15, 0.005, 6)]


@pytest.mark.parametrize("prec", [_lib.MIXED, _lib.FP64], ids=["mixed", "fp64"])
def test_ensemble_equals_independent_runs(lib, prec):
    steps = 41                     # iteration 0 + 20 graph launches of 2 steps
    runs = [_member(*m, prec) for m in MEMBERS]
    ens = _lib.Ensemble(runs)
    ms, caps = ens.run(steps)
    # cold beams bunch: some runs' tiles overflow and get rebuilt (the
    # graph is then captured again); the spill path carries records
    # exactly, so the results cannot depend on when that happens
    assert caps >= 1
    for m, c in zip(MEMBERS, runs):
        ref = _member(*m, prec)
        ref.run(steps)
        assert c.iter == ref.iter == steps
        for a, b in zip(c.particles(0), ref.particles(0)):
            assert np.array_equal(a, b)
        assert c.field_energy() == ref.field_energy()
        ref.close()
    ens.close()


def test_ensemble_odd_splits(lib):
    # calls of 2, 5, 3 and 4 steps: eager single steps between graph
    # launches flip every run's store and spill parity, so the graph is
    # captured again whenever it no longer matches
    runs = [_member(*m, _lib.MIXED) for m in MEMBERS[:3]]
    ens = _lib.Ensemble(runs)
    for k in (2, 5, 3, 4):
        ens.run(k)
    for m, c in zip(MEMBERS[:3], runs):
        ref = _member(*m, _lib.MIXED)
        ref.run(14)
        assert c.iter == 14
        for a, b in zip(c.particles(0), ref.particles(0)):
            assert np.array_equal(a, b)
        assert c.field_energy() == ref.field_energy()
        ref.close()
    ens.close()


def _overflowing(prec):
    n = 20000
    rng = np.random.default_rng(3)
    x = rng.uniform(0, L / 4, n)
    y = rng.uniform(0, L, n)
    # a third of the box per step: the destination tiles overflow, and the
    # pattern does not come back onto the initial tiles at a check
    ux = np.full(n, (L / 3) / 0.05)
    uy = rng.uniform(-1, 1, n)
    c = _lib.Context(64, 64, L, L, 0.05, 1.0, precision=prec, tile=8, halo=1)
    c.add_species(-1e-30, 1e-30, x, y, ux, uy)
    c.pre_step()
    return c


def test_ensemble_recaptures_after_rebuild(lib):
    # FP64 form: its spill path is bit-exact with the in-tile path, so the
    # result does not depend on when the host notices the overflow
    runs = [_overflowing(_lib.FP64), _member(64, 16, 0.2, 0.01, 9, _lib.FP64)]
    ens = _lib.Ensemble(runs)
    ms, caps = ens.run(33)
    assert caps >= 2
    refs = [_overflowing(_lib.FP64), _member(64, 16, 0.2, 0.01, 9, _lib.FP64)]
    for c, r in zip(runs, refs):
        r.run(33)
        for a, b in zip(c.particles(0), r.particles(0)):
            assert np.array_equal(a, b)
    assert runs[0].cell_counts().sum() == 20000


def test_autotune_tile(lib):
    for grid, ppc in ((32, 8), (256, 64)):
        tile, ms = _lib.autotune_tile(grid, grid, L, L, 0.05, grid * grid * ppc, 0.2, 0.0)
        assert tile in (4, 8, 16, 32, 64) and grid % tile == 0 and (grid // tile) ** 2 >= 4
        assert ms > 0
        again = _lib.autotune_tile(grid, grid, L, L, 0.05, grid * grid * ppc, 0.2, 0.0)
        assert again == (tile, ms)
