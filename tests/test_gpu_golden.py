"""GPU path against the golden fixtures produced by the reference itself
(tests/golden/make_golden.py).  Tolerances: rho and E within 1e-12 of the
max norm; particle state after the iteration-0 half kick bit-exact given the
reference's field; field energy within 1e-10 relative (FP64 form) and 1e-5
(mixed form); the harmonic-oscillator trace within 1e-9 relative."""
import numpy as np
import pytest

from cpic_gb300 import _lib
from tests import cases, golden_util

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", ["c1_two_stream", "c2_two_species_bz"])
def test_pre_step_and_half_kick(lib, name):
    case, d = golden_util.load(name)
    g = cases.make_gpu(case)
    g.pre_step()
    assert rel_max(g.rho(), d["pre_rho"]) <= 1e-12
    ex, ey = g.E()
    assert rel_max(ex, d["pre_Ex"]) <= 1e-12 and rel_max(ey, d["pre_Ey"]) <= 1e-12
    g.set_E(d["pre_Ex"], d["pre_Ey"])
    g.stage_plasma()
    for s in range(len(case["species"])):
        x, y, ux, uy = g.particles(s)
        n = len(d["step1_x%d" % s])
        for a, k in ((x, "x"), (y, "y"), (ux, "ux"), (uy, "uy")):
            assert np.array_equal(a[:n], d["step1_%s%d" % (k, s)]), (s, k)


@pytest.mark.parametrize("name", ["c1_two_stream", "c2_two_species_bz"])
def test_field_energy_history(lib, name):
    case, d = golden_util.load(name)
    g = cases.make_gpu(case)
    g.pre_step()
    we = []
    for _ in range(len(d["energy"])):
        g.step()
        we.append(g.field_energy())
    rel = np.max(np.abs(np.array(we) - d["energy"]) / d["energy"])
    assert rel <= 1e-10, rel


def test_mixed_field_energy_history(lib):
    case, d = golden_util.load("c1_two_stream")
    g = cases.make_gpu(case, precision=_lib.MIXED)
    g.pre_step()
    we = []
    for _ in range(len(d["energy"])):
        g.step()
        we.append(g.field_energy())
    rel = np.max(np.abs(np.array(we) - d["energy"]) / d["energy"])
    assert rel <= 1e-5, rel


def test_harmonic_trace(lib):
    case = golden_util.harmonic_case()
    x0, ex0 = golden_util.harmonic_trace()
    g = cases.make_gpu(case)
    g.pre_step()
    xs = []
    for _ in range(len(x0)):
        g.step()
        xs.append(g.particles(0)[0][0])
    xs = np.array(xs)
    assert np.max(np.abs(xs - x0) / np.abs(x0)) <= 1e-9
