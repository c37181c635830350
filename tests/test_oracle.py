"""The oracle pinned against the reference's own known answers and physics
tests (CPU only).

- CIC weights: the known-answer vector of test/interpolate.c.disabled:20-26
  (rel = (1/4, 3/4) -> w00 = 3/16, w10 = 1/16, w01 = 9/16, w11 = 3/16,
  i0 = (1, 2) for x = (3.25, 3.75), x0 = (2, 1), dx = 1).
- Poisson: a single Fourier mode has the closed-form discrete solution
  phi = rho / (2 cos kx + 2 cos ky - 4) (solver.c:269-280).
- constant speed: one particle keeps |u - u0| <= 1e-10 every step
  (test/constant-speed.c:90-91, conf/constant-speed.conf).
- cyclotron: one electron in Bz stays on the analytic circle within
  v*dt^2 (test/cyclotron.c:317-322, conf/cyclotron.conf).
"""
import math

import numpy as np
import pytest

from oracle import oracle


def test_cic_weights_known_answer(orc):
    w, i0 = oracle.weights(2. + 1. + 1. / 4., 1. + 2. + 3. / 4., 2.0, 1.0, 1.0, 1.0)
    # w = [w00, w01, w10, w11]
    assert w[0] == 3. / 16.
    assert w[2] == 1. / 16.
    assert w[1] == 9. / 16.
    assert w[3] == 3. / 16.
    assert list(i0) == [1, 2]


def test_weights_partition_of_unity(orc):
    rng = np.random.default_rng(0)
    for _ in range(1000):
        x, y = rng.uniform(0, 2 * math.pi, 2)
        w, i0 = oracle.weights(x, y, 0.0, 0.0, 2 * math.pi / 64, 2 * math.pi / 64)
        assert abs(w.sum() - 1.0) < 1e-10          # interpolate.c:95-99
        assert (w >= 0).all()


def test_poisson_single_mode(orc):
    nx, ny = 64, 32
    kx, ky = 3, 5
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny))
    rho = np.cos(2 * np.pi * (kx * X / nx + ky * Y / ny))
    lam = 2 * math.cos(2 * math.pi * kx / nx) + 2 * math.cos(2 * math.pi * ky / ny) - 4
    phi = oracle.poisson(rho)
    assert np.max(np.abs(phi - rho / lam)) < 1e-13
    # the k = 0 mode is removed (G(0,0) = 0)
    phi0 = oracle.poisson(rho + 5.0)
    assert np.max(np.abs(phi0 - rho / lam)) < 1e-12


@pytest.mark.parametrize("nx,ny", [(32, 16), (48, 40), (25, 15), (77, 13), (240, 120)])
def test_poisson_matches_numpy(orc, nx, ny):
    """Powers of two (radix 2) and sides with other factors (the
    mixed-radix path: 3, 5, 7, 11 and 13, odd sides, a prime side)."""
    rng = np.random.default_rng(nx * 1000 + ny)
    rho = rng.standard_normal((ny, nx))
    k = np.fft.rfft2(rho)
    cx = np.cos(2 * np.pi * np.arange(nx // 2 + 1) / nx)
    cy = np.cos(2 * np.pi * np.arange(ny) / ny)
    G = 1.0 / (2 * (cx[None, :] + cy[:, None]) - 4)
    G[0, 0] = 0.0
    ref = np.fft.irfft2(k * G, s=(ny, nx))
    assert np.max(np.abs(oracle.poisson(rho) - ref)) < 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_poisson_large_side_not_power_of_two_is_fast(orc):
    """A 1920 x 1920 solve (sides 2^7 3 5) within seconds: the mixed-radix
    path, not a direct DFT (about ten minutes per solve at this size)."""
    import time
    rho = np.random.default_rng(3).standard_normal((1920, 1920))
    t = time.perf_counter()
    phi = oracle.poisson(rho)
    assert time.perf_counter() - t < 30.0
    assert np.isfinite(phi).all()


def test_constant_speed(orc):
    # conf/constant-speed.conf: 1 electron, 64x64, L = 32, dt = 0.5,
    # u = (1.33333, 0.282828), r0 = (4, 16), e0 = 1, q = -1, m = 1e-2
    o = oracle.Oracle(64, 64, 32.0, 32.0, 0.5, 1.0, (0.0, 0.0, 0.0), plasma_chunks=4)
    o.add_species(-1.0, 1.0e-2, [4.0], [16.0], [1.33333], [0.282828])
    o.pre_step()
    u0 = None
    for it in range(2000):
        o.step()
        x, y, ux, uy = o.particles(0)
        if u0 is None:
            u0 = (ux[0], uy[0])
        assert abs(ux[0] - u0[0]) <= 1e-10 and abs(uy[0] - u0[1]) <= 1e-10, it


def test_cyclotron(orc):
    # conf/cyclotron.conf: 1 electron, 4x4, L = 32, Bz = -1, dt = 0.05,
    # u = (0, 10), r0 = (2, 16), e0 = 8.85e-12, q = -1, m = 1
    dt, v = 0.05, 10.0
    o = oracle.Oracle(4, 4, 32.0, 32.0, dt, 8.85e-12, (0.0, 0.0, -1.0), plasma_chunks=4)
    o.add_species(-1.0, 1.0, [2.0], [16.0], [0.0], [v])
    o.pre_step()
    o.step()                          # iteration 0: backward half kick
    pts = []
    for it in range(2000):
        o.step()
        x, y, ux, uy = o.particles(0)
        pts.append((x[0], y[0]))
    pts = np.array(pts)
    # positions wrap periodically in the 32-box: unwrap, then fit a circle
    un = np.unwrap(pts / 32.0 * 2 * np.pi, axis=0) * 32.0 / (2 * np.pi)
    A = np.c_[un[:, 0], un[:, 1], np.ones(len(un))]
    b = -(un[:, 0] ** 2 + un[:, 1] ** 2)
    D, E, F = np.linalg.lstsq(A, b, rcond=None)[0]
    cx, cy = -D / 2, -E / 2
    rad = np.hypot(un[:, 0] - cx, un[:, 1] - cy)
    # the radius of a cyclotron orbit is v / |qB/m| = 10
    assert abs(np.mean(rad) - v) <= v * dt * dt
    assert np.max(np.abs(rad - np.mean(rad))) <= v * dt * dt


def test_reference_build_goes_stale_with_its_inputs(tmp_path):
    """The reference build is redone when a project file it compiles or
    includes (here the oracle's FFT header) is newer than its stamp."""
    import os
    from oracle import build_ref
    import time
    stamp = tmp_path / "built.txt"
    stamp.write_text("x")
    later = time.time() + 86400
    os.utime(stamp, (later, later))
    assert not build_ref._stale(str(stamp))
    header = os.path.join(os.path.dirname(build_ref.__file__), "orc_fft.h")
    t = os.path.getmtime(header) - 10
    os.utime(stamp, (t, t))
    assert build_ref._stale(str(stamp))
