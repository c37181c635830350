"""Synthetic workloads shared by the tests and the benchmark.

Normalised units: e0 = 1, electron q/m = -1, plasma frequency 1, so the
electron macro-charge is q = -Lx*Ly/N and m = -q.  Inputs come from the
library's seeded init methods (SplitMix64 counter RNG), so the oracle and the
GPU receive identical arrays.
"""
import math

from cpic_gb300 import _lib

TWO_PI = 2.0 * math.pi


def two_stream(nx=64, ny=64, n=10240, v0=0.2, vth=0.0, amp=0.01, dt=0.05, L=TWO_PI, seed=1234,
               steps=200, Ly=None):
    """Two-stream instability (64x64, 10240 electrons: the CPU-runnable case).
    Ly: the domain's y length (default L; give L * ny / nx for square cells
    on a rectangular grid, as the reference's Y weights use dx)."""
    Ly = L if Ly is None else Ly
    q = -L * Ly / n
    x, y, ux, uy = _lib.init_two_stream(seed, 0, n, L, Ly, v0, vth, amp)
    return dict(nx=nx, ny=ny, L=L, Ly=Ly, dt=dt, B=(0.0, 0.0, 0.0), steps=steps,
                species=[dict(q=q, m=-q, x=x, y=y, ux=ux, uy=uy)])


def two_species(nx=512, ny=512, ppc=16, vth_e=0.05, mass_ratio=100.0, vth_i=0.005, Bz=0.5,
                dt=0.05, L=TWO_PI, seed=4321, steps=500):
    """Electrons and ions in a uniform Bz (512x512, 16 per cell per species)."""
    n = nx * ny * ppc
    qe = -L * L / n
    me = -qe
    xe, ye, uxe, uye = _lib.init_maxwellian(seed, 0, n, L, L, vth_e)
    xi, yi, uxi, uyi = _lib.init_maxwellian(seed, 1, n, L, L, vth_i)
    return dict(nx=nx, ny=ny, L=L, dt=dt, B=(0.0, 0.0, Bz), steps=steps,
                species=[dict(q=qe, m=me, x=xe, y=ye, ux=uxe, uy=uye),
                         dict(q=-qe, m=mass_ratio * me, x=xi, y=yi, ux=uxi, uy=uyi)])


def lengths(case):
    """(Lx, Ly) of a case."""
    return case["L"], case.get("Ly", case["L"])


def make_gpu(case, precision=_lib.FP64, **kw):
    Lx, Ly = lengths(case)
    ctx = _lib.Context(case["nx"], case["ny"], Lx, Ly, case["dt"], 1.0, case["B"],
                       precision=precision, **kw)
    for s in case["species"]:
        ctx.add_species(s["q"], s["m"], s["x"], s["y"], s["ux"], s["uy"])
    return ctx


def make_oracle(case, lossy=False):
    from oracle.oracle import Oracle
    Lx, Ly = lengths(case)
    o = Oracle(case["nx"], case["ny"], Lx, Ly, case["dt"], 1.0, case["B"], lossy=lossy)
    for s in case["species"]:
        o.add_species(s["q"], s["m"], s["x"], s["y"], s["ux"], s["uy"])
    return o
