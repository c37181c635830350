"""Charge and field-energy gap between the reference as shipped and its
conflict-free variant, both compiled from the reference's own sources by
oracle/build_ref.py (x86-64 only).

The shipped AVX2 deposit loses a contribution when two or more of a 4-lane
particle pack deposit to the same node (src/simd_avx2.h:232-249).  The
conflict-free variant adds lane by lane.  This script runs both on the same
injected states and prints, per case, the total-charge gap after the
pre-step deposit and after the last step, and the largest relative
field-energy gap over the run.

Usage: python oracle/shipped_gap.py  (needs the reference tree; test
infrastructure, not part of the library)
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from tests import cases, refrun  # noqa: E402


def gap(name, case, nsteps):
    runs = {v: refrun.run(case, nsteps, dumps=(nsteps,), variant=v) for v in ("exact", "shipped")}
    # rho holds w * (-q / e0) per node (src/interpolate.c:307): summed over
    # the nodes it is the charge the particles carry, with the sign flipped
    scale = sum(len(s["x"]) * abs(s["q"]) for s in case["species"])
    out = {"case": name, "particles": int(sum(len(s["x"]) for s in case["species"])),
           "steps": nsteps}
    for when in ("pre", nsteps):
        qe = float(np.sum(runs["exact"][when]["rho"]))
        qs = float(np.sum(runs["shipped"][when]["rho"]))
        key = "pre_step" if when == "pre" else "step_%d" % nsteps
        out["charge_" + key] = {"exact": qe, "shipped": qs,
                                "gap_over_total_abs_charge": abs(qs - qe) / scale}
    we, ws = runs["exact"]["energy"], runs["shipped"]["energy"]
    k = min(len(we), len(ws))
    rel = np.abs(ws[:k] - we[:k]) / np.abs(we[:k])
    out["field_energy"] = {"steps_compared": int(k), "max_rel_gap": float(rel.max()),
                           "final_rel_gap": float(rel[-1]),
                           "exact_final": float(we[k - 1]), "shipped_final": float(ws[k - 1])}
    return out


def main():
    if not refrun.available():
        print(json.dumps({"unavailable": "the reference build (oracle/_ref) is not present"}))
        return
    res = [gap("two-stream 64x64, 10240 electrons, dt 0.05", cases.two_stream(), 200),
           gap("two species 512x512, 16 per cell each, Bz 0.5, dt 0.05", cases.two_species(), 20)]
    for r in res:
        print(json.dumps(r))


if __name__ == "__main__":
    main()
