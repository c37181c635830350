"""Step cost of the reference's own build against the oracle's C restatement on
the same host and the same state: the check that the oracle, which stands in
for the reference as the timed CPU baseline where the reference does not
build (its AVX2 host code is x86-only), is not slower than the reference.

Both run one process on one core. The reference harness (oracle/_ref) is run
for 1 and for 4 steps after its pre-step; the difference over 3 steps is its
cost per step, with set-up and dumps cancelled. The oracle times the same
3 steps directly.

Usage: python oracle/ref_speed.py [grid] [particles per cell]
       python oracle/ref_speed.py two_species                (needs the
reference tree; test infrastructure, not part of the library)
"""
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from tests import cases, refrun  # noqa: E402


def reference_step_s(case, variant):
    exe = os.path.join(refrun.REF_OUT, "ref_harness_%s" % variant)
    wall = {}
    with tempfile.TemporaryDirectory() as d:
        conf = os.path.join(d, "case.conf")
        state = os.path.join(d, "state.bin")
        refrun.write_state(state, case)
        for n in (1, 4):
            refrun.write_conf(conf, case, n)
            t0 = time.perf_counter()
            subprocess.run([exe, conf, state, d, str(n)], check=True, capture_output=True)
            wall[n] = time.perf_counter() - t0
    return (wall[4] - wall[1]) / 3


def oracle_step_s(case):
    from oracle.oracle import Oracle
    o = Oracle(case["nx"], case["ny"], case["L"], case["L"], case["dt"], 1.0, case["B"])
    for s in case["species"]:
        o.add_species(s["q"], s["m"], s["x"], s["y"], s["ux"], s["uy"])
    o.pre_step()
    o.step()
    t0 = time.perf_counter()
    for _ in range(3):
        o.step()
    dt = (time.perf_counter() - t0) / 3
    o.close()
    return dt


def main():
    if not refrun.available():
        print(json.dumps({"unavailable": "the reference build (oracle/_ref) is not present"}))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "two_species":
        # electrons and ions (mass ratio 100) in Bz = 0.5, 512x512, 16 per cell each
        case = cases.two_species()
        n = sum(len(s["x"]) for s in case["species"])
        name = "two species 512x512, %d particles, Bz 0.5, dt 0.05" % n
    else:
        grid = int(sys.argv[1]) if len(sys.argv) > 1 else 1024
        ppc = int(sys.argv[2]) if len(sys.argv) > 2 else 10
        n = grid * grid * ppc
        case = cases.two_stream(nx=grid, ny=grid, n=n, v0=0.2, vth=0.01, amp=0.01)
        name = "two-stream %dx%d, %d electrons, dt 0.05" % (grid, grid, n)
    res = {"case": name, "particles": n, "host": os.uname().machine, "cores": 1}
    for v in ("shipped", "exact"):
        t = reference_step_s(case, v)
        res["reference_" + v] = {"s_per_step": t, "particle_steps_per_s": n / t}
    t = oracle_step_s(case)
    res["oracle"] = {"s_per_step": t, "particle_steps_per_s": n / t}
    res["oracle_over_reference_shipped"] = res["oracle"]["particle_steps_per_s"] / \
        res["reference_shipped"]["particle_steps_per_s"]
    print(json.dumps(res))


if __name__ == "__main__":
    main()
