"""Running the reference (built from its own sources by oracle/build_ref.py)
from Python: the .conf of a case, and the timed CPU arm of the benchmark.

TEST AND BENCHMARK INFRASTRUCTURE: used by tests/refrun.py and by bench.py's
reference arm; the product never imports it.
"""
import os
import subprocess
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def write_conf(path, case, cycles):
    """A .conf with the keys sim_read_config requires (src/sim.c:51-84);
    particles are placed by the harness, so the init method is a
    placeholder."""
    sp = []
    for s in case["species"]:
        sp.append("""	{
		name = "s"
		particles = %d
		charge = %r
		mass = %r
		drift_velocity = [0.0, 0.0]
		init_method = "position delta"
		position_delta = [0.0, 0.0]
		position_init = [0.0, 0.0]
	}""" % (len(s["x"]), float(s["q"]), float(s["m"])))
    L = float(case["L"])
    txt = """species = (
%s
)
field = { magnetic = [%r, %r, %r] }
grid = { points = [%d, %d] }
simulation = {
	dimensions = 2
	solver = "MFT"
	enable_fftw_threads = 0
	plasma_chunks = 1
	random_seed = 1
	cycles = %d
	time_step = %r
	space_length = [%r, %r]
	sampling_period = { energy = 0; field = 0; particle = 0 }
	stop_SEM = 0.0
	realtime_plot = 0
	pblock_nmax = 1024
}
constants = { light_speed = 1.0; vacuum_permittivity = 1.0 }
""" % (",\n".join(sp), float(case["B"][0]), float(case["B"][1]), float(case["B"][2]), case["nx"],
       case["ny"], cycles, float(case["dt"]), L, float(case.get("Ly", L)))
    with open(path, "w") as f:
        f.write(txt)



def harness(variant="shipped"):
    """Path of the reference harness binary of a variant, or None when the
    reference has not been built on this host."""
    exe = os.path.join(OUT, "ref_harness_%s" % variant)
    return exe if os.path.exists(exe) else None


def time_two_stream(procs, grid, n, v0, vth, amp, dt, L, warmup, steps, seed=99):
    """`procs` concurrent processes of the reference's own code (the shipped
    build), each the full grid with n particles of the seeded two-stream state
    (seed + process index), `warmup` untimed steps, then `steps` steps timed
    together: every process waits at a file barrier before its timed steps.
    Returns (particles per process, window start, window end, per-process
    per-step seconds)."""
    exe = harness()
    if exe is None:
        raise RuntimeError("the reference is not built here (oracle/build_ref.py)")
    q = -L * L / n
    case = dict(nx=grid, ny=grid, L=L, dt=dt, B=(0.0, 0.0, 0.0),
                species=[dict(q=q, m=-q, x=np.empty(n))])
    with tempfile.TemporaryDirectory() as d:
        conf = os.path.join(d, "case.conf")
        write_conf(conf, case, warmup + steps + 1)
        ps = [subprocess.Popen([exe, conf, "two_stream:%d:%r:%r:%r" % (seed + i, v0, vth, amp), d,
                                "%d+%d" % (warmup, steps)], stdout=subprocess.DEVNULL,
                               stderr=subprocess.PIPE) for i in range(procs)]
        t_end = time.monotonic() + 1800
        while sum(1 for f in os.listdir(d) if f.startswith("ready.")) < procs:
            if any(p.poll() not in (None, 0) for p in ps) or time.monotonic() > t_end:
                for p in ps:
                    p.kill()
                raise RuntimeError("reference harness failed before its timed steps: %s"
                                   % b"".join(p.stderr.read() or b"" for p in ps if p.poll())[-2000:])
            time.sleep(0.01)
        open(os.path.join(d, "go"), "w").close()
        for p in ps:
            if p.wait() != 0:
                raise RuntimeError("reference harness failed: %s" % p.stderr.read()[-2000:])
        res = []
        for f in sorted(os.listdir(d)):
            if f.startswith("times."):
                raw = open(os.path.join(d, f), "rb").read()
                npart = int(np.frombuffer(raw, np.int64, 1)[0])
                t = np.frombuffer(raw, np.float64, steps + 1, 8)
                res.append((npart, float(t[0]), float(t[-1]), np.diff(t)))
    if len(res) != procs:
        raise RuntimeError("missing timing files")
    return res
