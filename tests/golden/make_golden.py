"""Generate the golden fixtures in this directory by running the reference
itself (compiled from its own sources by oracle/build_ref.py, conflict-free
deposit variant) on seeded inputs.  Run on the development machine, where
the reference tree exists:  python tests/golden/make_golden.py

Fixtures (numpy .npz):
  c1_two_stream.npz      64x64 two-stream, 10240 electrons, dt 0.05:
                         inputs, pre-step rho/Ex/Ey, state after the
                         iteration-0 half kick (first 2048 ids), field
                         energy of 200 steps.
  c2_two_species_bz.npz  32x32, 4 per cell of electrons and ions (mass
                         ratio 100) in Bz = 0.5: inputs, half-kick state
                         (first 1024 ids per species), 100 energies.
  harmonic.npz           conf/harmonic.conf (two electrons, 1024x1024):
                         x and E_x of particle 0 after each of 1200 steps,
                         from the reference build.
  harmonic_line64.npz    the reference's own fixture test/harmonic/E.csv: the
                         field of the same two electrons on the 64x64 grid
                         (harmonic.conf's commented-out size) along the row
                         y = 4 (64 points, x = 0 ... 7.875): E_x, E_y, phi,
                         rho as exported, 6 significant digits.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests import cases, refrun  # noqa: E402


def inputs(case):
    d = {"nx": case["nx"], "ny": case["ny"], "L": case["L"], "dt": case["dt"], "B": np.array(case["B"]),
         "nspecies": len(case["species"])}
    for i, s in enumerate(case["species"]):
        d["q%d" % i] = s["q"]
        d["m%d" % i] = s["m"]
        for k in ("x", "y", "ux", "uy"):
            d["%s%d" % (k, i)] = np.asarray(s[k])
    return d


REF = os.environ.get("CPIC_REFERENCE", "/root/reference")


def main(which=("c1", "c2", "harmonic", "line")):
    if "line" in which:
        make_harmonic_line()
        if which == ("line",):
            return
    assert refrun.available(), "reference build unavailable"
    if "c1" in which:
        make_c1()
    if "c2" in which:
        make_c2()
    if "harmonic" in which:
        make_harmonic()


def make_c1():
    case = cases.two_stream()
    ref = refrun.run(case, 200, dumps=(1,))
    d = inputs(case)
    d.update(pre_rho=ref["pre"]["rho"], pre_Ex=ref["pre"]["Ex"], pre_Ey=ref["pre"]["Ey"],
             energy=ref["energy"])
    s1 = refrun.by_id(ref[1]["species"][0])
    for k in ("x", "y", "ux", "uy"):
        d["step1_%s0" % k] = s1[k][:2048]
    np.savez_compressed(os.path.join(HERE, "c1_two_stream.npz"), **d)


def make_c2():
    case = cases.two_species(nx=32, ny=32, ppc=4, steps=100)
    ref = refrun.run(case, 100, dumps=(1,))
    d = inputs(case)
    d.update(pre_rho=ref["pre"]["rho"], pre_Ex=ref["pre"]["Ex"], pre_Ey=ref["pre"]["Ey"],
             energy=ref["energy"])
    for i in range(2):
        s1 = refrun.by_id(ref[1]["species"][i])
        for k in ("x", "y", "ux", "uy"):
            d["step1_%s%d" % (k, i)] = s1[k][:1024]
    np.savez_compressed(os.path.join(HERE, "c2_two_species_bz.npz"), **d)


def make_harmonic():
    # conf/harmonic.conf: two electrons of charge -1, mass 1e-2 at (1, 4)
    # and (7, 4), 1024x1024 grid, L = 8, dt = 5e-3, e0 = 1
    case = dict(nx=1024, ny=1024, L=8.0, dt=5e-3, B=(0.0, 0.0, 0.0),
                species=[dict(q=-1.0, m=1e-2, x=np.array([1.0]), y=np.array([4.0]),
                              ux=np.zeros(1), uy=np.zeros(1)),
                         dict(q=-1.0, m=1e-2, x=np.array([7.0]), y=np.array([4.0]),
                              ux=np.zeros(1), uy=np.zeros(1))])
    steps = list(range(1, 1201))
    xs, es = [], []
    # dump every step of particle 0 (species 0)
    ref = refrun.run(case, 1200, dumps=steps)
    for k in steps:
        sp = ref[k]["species"][0]
        xs.append(sp["x"][0])
        es.append(sp["Ex"][0])
    np.savez_compressed(os.path.join(HERE, "harmonic.npz"), x0=np.array(xs), Ex0=np.array(es))


def make_harmonic_line():
    # columns of E.csv: E_X, E_Y, Points_0, Points_1, Points_2,
    # Points_Magnitude, phi, rho, Point ID
    t = np.genfromtxt(os.path.join(REF, "test", "harmonic", "E.csv"), delimiter=",", skip_header=1)
    np.savez_compressed(os.path.join(HERE, "harmonic_line64.npz"), Ex=t[:, 0], Ey=t[:, 1],
                        x=t[:, 2], y=t[:, 3], phi=t[:, 6], rho=t[:, 7])


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or ("c1", "c2", "harmonic", "line"))
