"""The reference's own host program and test drivers, unchanged, running the
time step on the GPU through the drop-in sim layer
(cpic_gb300/dropin/sim_gpu.c, linked by tests/dropin_build.py from the
reference tree or its staged view).

- test/constant-speed.c: |u - u0| <= 1e-10 over its 50,000 cycles
  (test/constant-speed.c:90-91);
- test/cyclotron.c as shipped (strict check): the reference's own Boris
  phase lag fails it; the GPU run reports the error the oracle's trajectory
  gives under the driver's formula (test/cyclotron.c:80-236, 317-322);
- test/harmonic.c: the x position of electron 0 it prints every cycle
  against the reference's trace (tests/golden/harmonic.npz, from the
  reference build), to the printed precision;
- the stage entry points (stage_field_E, stage_plasma_E, stage_plasma_r,
  stage_field_rho, comm_plasma) called one by one give the host views of
  sim_step and of sim_run bit for bit;
- src/cpic.c on a two-stream .conf with output enabled: the reference's field
  writer (output.c:601) writes bin/<iter>/{rho,phi,E_X,E_Y}.bin and the XDMF
  files; the written fields match the oracle (1e-12 of the max norm after
  the pre-step, field energy 1e-10 over the run).
"""
import math
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from tests import cases, dropin_build, golden_util

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TWO_STREAM_CONF = os.path.join(ROOT, "cpic_gb300", "dropin", "conf", "two_stream_64.conf")


@pytest.fixture(scope="module")
def out(lib):
    if dropin_build.ref_root() is None:
        pytest.skip("no reference tree (nor its staged view) to build the host program from")
    return dropin_build.build()


def run(out, prog, args=(), env=None, timeout=900):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([os.path.join(out, prog)] + list(args), cwd=dropin_build.ref_root(),
                          capture_output=True, text=True, timeout=timeout, env=e)


def test_constant_speed_driver(out):
    r = run(out, "test_constant_speed_gpu")
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "OK: Particle remains with constant speed" in r.stdout


def test_cyclotron_driver(out):
    """test/cyclotron.c as shipped (WEAK_CHECK 0) measures the distance to
    the analytic orbit point, and the reference's own algorithm fails it:
    Boris rotates by 2 atan(w dt / 2) instead of w dt per step, so after 5000
    steps the phase lag puts the particle 0.52 from that point against a
    limit of v dt^2 = 0.025.  The GPU run must fail the same way, with the
    error the oracle's trajectory gives under the driver's own formula
    (cyclotron.c:80-236): 0.523678 there."""
    r = run(out, "test_cyclotron_gpu")
    m = re.search(r"^FAIL .*The error ([-+0-9.e]+) exceeds the limit ([-+0-9.e]+)", r.stdout, re.M)
    assert r.returncode == 1 and m, r.stdout[-2000:] + r.stderr[-2000:]
    err, limit = float(m.group(1)), float(m.group(2))
    # the same measure on the oracle's trajectory
    from oracle.oracle import Oracle
    dt, steps, v, B = 0.05, 5000, 10.0, (0.0, 0.0, -1.0)
    o = Oracle(4, 4, 32.0, 32.0, dt, 8.85e-12, B, plasma_chunks=4)
    o.add_species(-1.0, 1.0, [2.0], [16.0], [0.0], [v])
    o.pre_step()
    freq = -1.0                      # |q| B_z / m
    radius = v / freq
    uxB = np.cross([0.0, v, 0.0], B)
    center = np.array([2.0, 16.0]) + (uxB * radius / np.linalg.norm(uxB))[:2]
    worst = 0.0
    for k in range(steps):
        o.step()                     # iter k + 1; the driver uses t = k dt
        x, y, _, _ = o.particles(0)
        t = k * dt
        R = radius * np.array([math.cos(t * freq), math.sin(t * freq)])
        worst = max(worst, float(np.hypot(*(np.array([x[0], y[0]]) - center - R))))
    o.close()
    assert limit == pytest.approx(v * dt * dt, rel=1e-6)
    # the electron's own field cancels at its position only to the FFT's
    # rounding, which differs between the GPU solver and the oracle's: the
    # trajectories agree to 1e-4 after 5000 steps (tests/test_gpu_physics.py)
    assert abs(err - worst) <= 1e-4, (err, worst)


def test_harmonic_driver_trace(out):
    r = run(out, "test_harmonic_gpu")
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    x0, _ = golden_util.harmonic_trace()
    pat = re.compile(r"iter=\s*(\d+) .*?r0=\(([-+0-9.e]+) ([-+0-9.e]+)\)")
    got = {int(m.group(1)): float(m.group(2)) for m in pat.finditer(r.stderr + r.stdout)}
    assert len(got) >= len(x0) - 1, len(got)
    # the driver prints after each sim_step, with iter already advanced
    worst = max(abs(got[k] - x0[k - 1]) / abs(x0[k - 1]) for k in got if 1 <= k <= len(x0))
    assert worst <= 1e-6, worst          # %+e prints 7 significant digits


def conf_with(path, cycles, host_sync, output_dir=None, stop_sem=0.0, grid=None):
    """The two-stream .conf with the given cycles and options; grid = (nx,
    ny, particles) sets the grid (square cells: Ly = 2 pi ny / nx) and the
    electron count and charge to match."""
    txt = open(TWO_STREAM_CONF).read()
    if grid:
        nx, ny, n = grid
        Lx, Ly = cases.TWO_PI, cases.TWO_PI * ny / nx
        q = Lx * Ly / n
        txt = re.sub(r"points = \[\d+, \d+\]", "points = [%d, %d]" % (nx, ny), txt)
        txt = re.sub(r"particles = \d+", "particles = %d" % n, txt)
        txt = re.sub(r"charge = [-0-9.e]+", "charge = %r" % -q, txt)
        txt = re.sub(r"mass = [-0-9.e]+", "mass = %r" % q, txt)
        txt = re.sub(r"space_length = \[[^]]*\]", "space_length = [%r, %r]" % (Lx, Ly), txt)
    txt = re.sub(r"cycles = \d+", "cycles = %d" % cycles, txt)
    txt = re.sub(r"host_sync = \d+", "host_sync = %d" % host_sync, txt)
    txt = re.sub(r"stop_SEM = [0-9.]+", "stop_SEM = %r" % stop_sem, txt)
    if output_dir:
        txt += 'output = { path = "%s"; slices = 1; alignment = 4096; }\n' % output_dir
    with open(path, "w") as f:
        f.write(txt)


def read_dump(path):
    raw = open(path, "rb").read()
    off = 0

    def take(n, dt):
        nonlocal off
        a = np.frombuffer(raw, dt, n, off)
        off += a.nbytes
        return a

    ns = int(take(1, np.int64)[0])
    species = []
    for _ in range(ns):
        n = int(take(1, np.int64)[0])
        rec = take(n, np.dtype([("id", "<i8"), ("v", "<f8", 6)]))
        species.append(rec.copy())
    nx, ny = (int(v) for v in take(2, np.int64))
    fields = [take(nx * ny, np.float64).reshape(ny, nx).copy() for _ in range(4)]
    return species, fields


def test_stage_entry_points_match_sim_step(out):
    steps = 25
    with tempfile.TemporaryDirectory() as d:
        dumps = {}
        for mode, sync in (("run", 0), ("step", 1), ("stages", 1)):
            conf = os.path.join(d, "%s.conf" % mode)
            conf_with(conf, steps, sync)
            dump = os.path.join(d, "%s.bin" % mode)
            r = run(out, "dropin_stages", [conf, str(steps), mode, dump])
            assert r.returncode == 0, (mode, r.stderr[-2000:])
            dumps[mode] = read_dump(dump)
    ref_sp, ref_f = dumps["run"]
    for mode in ("step", "stages"):
        sp, f = dumps[mode]
        for a, b in zip(sp, ref_sp):
            assert np.array_equal(np.sort(a["id"]), np.sort(b["id"])), mode
            ia, ib = np.argsort(a["id"]), np.argsort(b["id"])
            # positions and velocities (E at the particles is refreshed by the
            # stage path only: sim_run's final view carries no gathered E)
            assert np.array_equal(a["v"][ia, :4], b["v"][ib, :4]), mode
        for x, y in zip(f, ref_f):
            assert np.array_equal(x, y), mode
    # the E the stage path leaves at the particles is the field gathered at
    # their pre-push positions (stage_plasma_E), identical for both paths
    a, b = dumps["step"][0][0], dumps["stages"][0][0]
    assert np.array_equal(a["v"][np.argsort(a["id"])], b["v"][np.argsort(b["id"])])


def parse_xdmf_attr(path, name):
    """(real shape, view start, view shape) of one field from the XDMF the
    reference's writer produces (output.c:401-446)."""
    txt = open(path).read()
    i = txt.index('Name="%s"' % name)
    blk = txt[i:txt.index("</Attribute>", i)]
    nums = re.findall(r"<DataItem Dimensions=\"3 3\" Format=\"XML\">\s*([^<]*)</DataItem>", blk)[0].split()
    start = (int(nums[1]), int(nums[2]))
    end = (int(nums[7]), int(nums[8]))
    real = re.findall(r'Dimensions="1 (\d+) (\d+)" DataType="Float"', blk)[0]
    return (int(real[0]), int(real[1])), start, (end[0] - start[0], end[1] - start[1])


def read_field(out_dir, it, name):
    real, start, shape = parse_xdmf_attr(os.path.join(out_dir, "xdmf", "fields-iter%d.xdmf" % it), name)
    raw = np.fromfile(os.path.join(out_dir, "bin", str(it), name + ".bin"), np.float64)
    m = raw[:real[0] * real[1]].reshape(real)
    return m[start[0]:start[0] + shape[0], start[1]:start[1] + shape[1]]


def test_cpic_main_writes_fields_matching_oracle(out):
    steps = 20
    with tempfile.TemporaryDirectory(dir=os.path.join(ROOT, "tests", "_dropin")) as d:
        od = os.path.join(d, "out")
        conf = os.path.join(d, "two_stream.conf")
        conf_with(conf, steps, 0, output_dir=od)
        r = run(out, "cpic_gpu", [conf])
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        assert "Simulation ends" in r.stdout
        case = cases.two_stream(seed=1)
        o = cases.make_oracle(case)
        o.pre_step()
        for it in range(steps):
            rho, phi = read_field(od, it, "rho"), read_field(od, it, "phi")
            ex, ey = read_field(od, it, "E_X"), read_field(od, it, "E_Y")
            orho, ophi = o.rho(), o.phi()
            oex, oey = o.E()
            if it == 0:
                for a, b in ((rho, orho), (phi, ophi), (ex, oex[:64]), (ey, oey[:64])):
                    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
            we = 0.5 * np.sum(ex ** 2 + ey ** 2) * (case["L"] / 64) ** 2
            owe = 0.5 * np.sum(oex[:64] ** 2 + oey[:64] ** 2) * (case["L"] / 64) ** 2
            assert abs(we - owe) <= 1e-10 * owe, it
            # the next output is after the next step's field solve (the
            # oracle's next step solves the same rho again: no change)
            o.step()
            o.stage_field_E()


def test_cpic_main_grid_not_power_of_two(out):
    """cpic's own main on a 48 x 40 grid (the reference's solver takes any
    size): every written field against the oracle, rho, phi and E within
    1e-12 of their max norm at the first output and the field energy within
    1e-10 at every one."""
    steps, nx, ny, n = 12, 48, 40, 48 * 40 * 4
    with tempfile.TemporaryDirectory(dir=os.path.join(ROOT, "tests", "_dropin")) as d:
        od = os.path.join(d, "out")
        conf = os.path.join(d, "grid.conf")
        conf_with(conf, steps, 0, output_dir=od, grid=(nx, ny, n))
        r = run(out, "cpic_gpu", [conf])
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        case = cases.two_stream(nx=nx, ny=ny, n=n, seed=1, Ly=cases.TWO_PI * ny / nx)
        o = cases.make_oracle(case)
        o.pre_step()
        cell = (cases.TWO_PI / nx) ** 2
        for it in range(steps):
            rho, phi = read_field(od, it, "rho"), read_field(od, it, "phi")
            ex, ey = read_field(od, it, "E_X"), read_field(od, it, "E_Y")
            assert rho.shape == (ny, nx) and ex.shape == (ny, nx)
            oex, oey = o.E()
            if it == 0:
                for a, b in ((rho, o.rho()), (phi, o.phi()), (ex, oex[:ny]), (ey, oey[:ny])):
                    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
            we = 0.5 * np.sum(ex ** 2 + ey ** 2) * cell
            owe = 0.5 * np.sum(oex[:ny] ** 2 + oey[:ny] ** 2) * cell
            assert abs(we - owe) <= 1e-10 * owe, it
            o.step()
            o.stage_field_E()


def test_cpic_main_sampling_stats(out):
    with tempfile.TemporaryDirectory() as d:
        conf = os.path.join(d, "two_stream.conf")
        conf_with(conf, 60, 0, stop_sem=0.5)
        r = run(out, "cpic_gpu", [conf])
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        stats = re.findall(r"^stats iter=(\d+) last=\S+ mean=\S+ std=\S+ sem=\S+ rsem=\S+ mem=\d+ "
                           r"solver=\S+$", r.stdout, re.M)
        assert len(stats) >= 30
