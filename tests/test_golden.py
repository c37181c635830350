"""The oracle against the golden fixtures produced by the reference itself
(CPU only; runs everywhere, the reference tree is not needed)."""
import numpy as np

from tests import cases, golden_util


def test_c1_pre_step_and_half_kick_bitexact(orc):
    case, d = golden_util.load("c1_two_stream")
    o = cases.make_oracle(case)
    o.pre_step()
    assert np.array_equal(o.rho(), d["pre_rho"])
    ex, ey = o.E()
    assert np.array_equal(ex, d["pre_Ex"]) and np.array_equal(ey, d["pre_Ey"])
    o.step()
    x, y, ux, uy = o.particles(0)
    n = len(d["step1_x0"])
    for a, k in ((x, "x"), (y, "y"), (ux, "ux"), (uy, "uy")):
        assert np.array_equal(a[:n], d["step1_%s0" % k]), k


def test_c1_field_energy_200_steps(orc):
    case, d = golden_util.load("c1_two_stream")
    o = cases.make_oracle(case)
    o.pre_step()
    we = []
    for _ in range(200):
        o.step()
        we.append(o.diag()["WE"])
    rel = np.max(np.abs(np.array(we) - d["energy"]) / d["energy"])
    assert rel <= 1e-10, rel


def test_c2_two_species_bz(orc):
    case, d = golden_util.load("c2_two_species_bz")
    o = cases.make_oracle(case)
    o.pre_step()
    assert np.array_equal(o.rho(), d["pre_rho"])
    o.step()
    for s in range(2):
        x, y, ux, uy = o.particles(s)
        n = len(d["step1_x%d" % s])
        for a, k in ((x, "x"), (y, "y"), (ux, "ux"), (uy, "uy")):
            assert np.array_equal(a[:n], d["step1_%s%d" % (k, s)]), (s, k)
    we = [o.diag()["WE"]]
    for _ in range(99):
        o.step()
        we.append(o.diag()["WE"])
    rel = np.max(np.abs(np.array(we) - d["energy"]) / d["energy"])
    assert rel <= 1e-10, rel


def test_harmonic_trace_bitexact_first_steps(orc):
    from oracle.oracle import Oracle
    case = golden_util.harmonic_case()
    x0, ex0 = golden_util.harmonic_trace()
    o = cases.make_oracle(case)
    o.pre_step()
    for k in range(40):
        o.step()
        assert o.particles(0)[0][0] == x0[k], k
        assert o.particle_E(0)[0][0] == ex0[k], k
