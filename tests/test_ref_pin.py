"""The oracle pinned against the reference itself (CPU only).

The reference is compiled from its own sources with project-written shims
(oracle/build_ref.py) and driven by oracle/ref_harness.c on the same
particle states as the oracle.  Where the reference tree is absent these
tests skip; tests/test_golden.py checks the committed fixtures instead.

Pins (bit-exact unless stated): rho, phi and E after the pre-step; particle
E, positions and velocities after the iteration-0 half kick; full steps
from the reference's own state and fields; rho deposited in the
reference's particle order (conflict-free variant, and the shipped lossy
variant against the oracle's lossy mode); field energy over 200 steps
within 1e-10; grids whose sides are not powers of two; and the
reference's committed harmonic-oscillator traces
(test/harmonic/harm.r0x, harm.E0x) to their printed precision.
"""
import os

import numpy as np
import pytest

from tests import cases, refrun

REF = os.environ.get("CPIC_REFERENCE", "/root/reference")
pytestmark = pytest.mark.skipif(not os.path.isdir(REF) or not refrun.available(),
                                reason="reference tree not present (development machine only)")


def oracle_from(case, species_states, lossy=False):
    """Oracle with the given per-species arrays (already in the order wanted)."""
    from oracle.oracle import Oracle
    Lx, Ly = cases.lengths(case)
    o = Oracle(case["nx"], case["ny"], Lx, Ly, case["dt"], 1.0, case["B"], lossy=lossy)
    for s, st in zip(case["species"], species_states):
        o.add_species(s["q"], s["m"], st["x"], st["y"], st["ux"], st["uy"])
    return o


@pytest.fixture(scope="module")
def c1():
    case = cases.two_stream()
    ref = refrun.run(case, 200, dumps=(1, 2, 3))
    return case, ref


def test_pre_step_fields_bitexact(c1):
    case, ref = c1
    o = cases.make_oracle(case)
    o.pre_step()
    pre = ref["pre"]
    # no particle has moved yet: the reference's list order is the id order
    assert np.array_equal(pre["species"][0]["order"], np.arange(len(case["species"][0]["x"])))
    assert np.array_equal(o.rho(), pre["rho"])
    assert np.array_equal(o.phi(), pre["phi"])
    ex, ey = o.E()
    assert np.array_equal(ex, pre["Ex"]) and np.array_equal(ey, pre["Ey"])


def test_half_kick_bitexact(c1):
    case, ref = c1
    o = cases.make_oracle(case)
    o.pre_step()
    o.step()
    r = refrun.by_id(ref[1]["species"][0])
    x, y, ux, uy = o.particles(0)
    ex, ey = o.particle_E(0)
    for a, b in ((x, r["x"]), (y, r["y"]), (ux, r["ux"]), (uy, r["uy"]), (ex, r["Ex"]), (ey, r["Ey"])):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("k", [2, 3])
def test_full_step_bitexact_from_reference_state(c1, k):
    """Push from the reference's own state and fields: positions and
    velocities bit-exact; the deposit in the reference's particle order is
    bit-exact too."""
    case, ref = c1
    prev = ref[k - 1]["species"][0]
    o = oracle_from(case, [prev])
    o.set_E(ref[k]["Ex"], ref[k]["Ey"])
    o.iter = k - 1
    o.stage_plasma_E()
    assert o.stage_plasma_r() == 0
    x, y, ux, uy = o.particles(0)
    got = {"order": prev["order"], "x": x, "y": y, "ux": ux, "uy": uy,
           "Ex": o.particle_E(0)[0], "Ey": o.particle_E(0)[1]}
    got = refrun.by_id(got)
    r = refrun.by_id(ref[k]["species"][0])
    for key in ("x", "y", "ux", "uy", "Ex", "Ey"):
        assert np.array_equal(got[key], r[key]), key
    # deposit in the reference's list order after its re-bin
    now = ref[k]["species"][0]
    d = oracle_from(case, [now])
    d.stage_field_rho()
    assert np.array_equal(d.rho(), ref[k]["rho"])


def test_field_energy_200_steps(c1):
    case, ref = c1
    o = cases.make_oracle(case)
    o.pre_step()
    we = []
    for _ in range(200):
        o.step()
        we.append(o.diag()["WE"])
    we = np.array(we)
    rel = np.max(np.abs(we - ref["energy"]) / ref["energy"])
    assert rel <= 1e-10, rel


def test_two_species_bz_energy():
    case = cases.two_species(nx=32, ny=32, ppc=4, steps=100)
    ref = refrun.run(case, 100)
    o = cases.make_oracle(case)
    o.pre_step()
    we = []
    for _ in range(100):
        o.step()
        we.append(o.diag()["WE"])
    rel = np.max(np.abs(np.array(we) - ref["energy"]) / ref["energy"])
    assert rel <= 1e-10, rel


@pytest.mark.parametrize("nx,ny", [(48, 40), (25, 15)])
def test_grid_not_power_of_two(nx, ny):
    """Grids whose sides are not powers of two (the reference's FFTW solver
    takes any size): pre-step fields bit-exact, the particles after two
    steps bit-exact, field energy over 60 steps within 1e-10.  Square cells
    (Ly = L ny / nx), as the reference's Y weights use dx."""
    L = cases.TWO_PI
    case = cases.two_stream(nx=nx, ny=ny, n=nx * ny * 4, Ly=L * ny / nx)
    ref = refrun.run(case, 60, dumps=(2,))
    o = cases.make_oracle(case)
    o.pre_step()
    pre = ref["pre"]
    assert np.array_equal(o.rho(), pre["rho"])
    assert np.array_equal(o.phi(), pre["phi"])
    ex, ey = o.E()
    assert np.array_equal(ex, pre["Ex"]) and np.array_equal(ey, pre["Ey"])
    we = []
    for k in range(60):
        o.step()
        we.append(o.diag()["WE"])
        if k == 1:
            r = refrun.by_id(ref[2]["species"][0])
            x, y, ux, uy = o.particles(0)
            for a, b in ((x, r["x"]), (y, r["y"]), (ux, r["ux"]), (uy, r["uy"])):
                assert np.array_equal(a, b)
    rel = np.max(np.abs(np.array(we) - ref["energy"]) / ref["energy"])
    assert rel <= 1e-10, rel


def test_shipped_lossy_deposit_bitexact(c1):
    """The shipped reference loses charge when two lanes of a 4-particle
    pack hit the same node; the oracle's lossy mode reproduces it."""
    case, _ = c1
    ref = refrun.run(case, 3, dumps=(3,), variant="shipped")
    now = ref[3]["species"][0]
    lossy = oracle_from(case, [now], lossy=True)
    lossy.stage_field_rho()
    assert np.array_equal(lossy.rho(), ref[3]["rho"])
    exact = oracle_from(case, [now])
    exact.stage_field_rho()
    q = case["species"][0]["q"]
    n = len(case["species"][0]["x"])
    # total charge in units of -q/e0 per particle
    assert abs(exact.rho().sum() / (-q) - n) < 1e-6 * n
    assert lossy.rho().sum() / (-q) < n


def test_harmonic_traces():
    """conf/harmonic.conf: two electrons on a 1024^2 grid; the reference
    ships the x position and E_x of particle 0 per step (printed with 7
    significant digits)."""
    from oracle.oracle import Oracle
    r0 = np.loadtxt(os.path.join(REF, "test", "harmonic", "harm.r0x"))
    e0 = np.loadtxt(os.path.join(REF, "test", "harmonic", "harm.E0x"))
    o = Oracle(1024, 1024, 8.0, 8.0, 5e-3, 1.0)
    o.add_species(-1.0, 1e-2, [1.0], [4.0], [0.0], [0.0])
    o.add_species(-1.0, 1e-2, [7.0], [4.0], [0.0], [0.0])
    o.pre_step()
    for k in range(60):
        o.step()
        x = o.particles(0)[0][0]
        ex = o.particle_E(0)[0][0]
        assert abs(x - r0[k]) <= 5e-7 * abs(r0[k]) + 1e-12, k
        assert abs(ex - e0[k]) <= 5e-7 * abs(e0[k]) + 1e-12, k


@pytest.mark.skipif(not os.path.exists(os.path.join(refrun.REF_OUT, "ref_harness_shipped_portable")),
                    reason="the portable build is compared where the native AVX2 build exists")
@pytest.mark.parametrize("which", ["two_stream", "two_species"])
def test_portable_intrinsics_build_matches_native(which):
    """The reference built with oracle/shims_portable/x86intrin.h (how it
    builds on the Arm host of the GPU) gives the native AVX2 build's
    results bit for bit: fields and every particle after the pre-step and
    after steps 1-3, and the field energy of every step."""
    case = cases.two_stream() if which == "two_stream" else cases.two_species(nx=32, ny=32, ppc=8)
    steps = 50
    a = refrun.run(case, steps, dumps=(1, 2, 3), variant="shipped")
    b = refrun.run(case, steps, dumps=(1, 2, 3), variant="shipped_portable")
    assert np.array_equal(a["energy"], b["energy"])
    for k in ("pre", 1, 2, 3):
        for f in ("rho", "phi", "Ex", "Ey"):
            assert np.array_equal(a[k][f], b[k][f]), (k, f)
        for sa, sb in zip(a[k]["species"], b[k]["species"]):
            for f in ("order", "x", "y", "ux", "uy", "Ex", "Ey"):
                assert np.array_equal(sa[f], sb[f]), (k, f)
