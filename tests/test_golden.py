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


def test_harmonic_field_line_matches_reference_export(orc):
    """The reference's own fixture test/harmonic/E.csv: E and phi of the two
    electrons of conf/harmonic.conf on its 64x64 grid, along the row y = 4,
    printed to 6 significant digits.  The oracle's pre-step field rounds to
    the same digits at every point. The exceptions are points where the
    physical value is zero (E_x at x = 4 and all of E_y, by symmetry). There
    both sides hold rounding noise below 1e-12 of the largest |E_x|."""
    d = np.load(golden_util.HERE + "/harmonic_line64.npz")
    case = golden_util.harmonic_case()
    case.update(nx=64, ny=64)
    o = cases.make_oracle(case)
    o.pre_step()
    ex, ey = o.E()
    row = int(round(d["y"][0] / (case["L"] / case["ny"])))
    assert np.all(d["y"] == d["y"][0]) and np.allclose(d["x"], np.arange(64) * case["L"] / 64)
    got = {"Ex": ex[row, :64], "Ey": ey[row, :64], "phi": o.phi()[row], "rho": o.rho()[row]}
    noise = 1e-12 * np.max(np.abs(d["Ex"]))

    def digits6(v):
        return float("%.6g" % v)

    for k in ("Ex", "phi", "rho"):
        for i in range(64):
            want = d[k][i]
            if abs(want) <= noise:
                assert abs(got[k][i]) <= noise, (k, i)
            else:
                assert digits6(got[k][i]) == want, (k, i, got[k][i], want)
    assert np.max(np.abs(got["Ey"])) <= noise and np.max(np.abs(d["Ey"])) <= noise
