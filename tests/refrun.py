"""Run the reference (built from its own sources by oracle/build_ref.py) on a
given particle state and read its dumps.  Only usable where the reference
tree exists (the development machine); tests that need it skip otherwise.
"""
import os
import subprocess
import tempfile

import numpy as np

from oracle.ref_run import write_conf  # noqa: F401  (the .conf of a case)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_OUT = os.path.join(ROOT, "oracle", "_ref")


def available():
    try:
        from oracle import build_ref
    except ImportError:
        return False
    return build_ref.build() is not None


def write_state(path, case):
    with open(path, "wb") as f:
        for s in case["species"]:
            np.array([len(s["x"])], np.int64).tofile(f)
            for k in ("x", "y", "ux", "uy"):
                np.ascontiguousarray(s[k], np.float64).tofile(f)


def read_dump(path):
    raw = open(path, "rb").read()
    nx, ny, ns = np.frombuffer(raw, np.int64, 3)
    off = 24

    def take(count, dt=np.float64):
        nonlocal off
        a = np.frombuffer(raw, dt, count, off)
        off += a.nbytes
        return a

    out = {"rho": take(nx * ny).reshape(ny, nx), "phi": take(nx * ny).reshape(ny, nx),
           "Ex": take((ny + 1) * nx).reshape(ny + 1, nx), "Ey": take((ny + 1) * nx).reshape(ny + 1, nx),
           "species": []}
    for _ in range(ns):
        n = int(take(1, np.int64)[0])
        rec = np.frombuffer(raw, np.dtype([("id", "<i8"), ("v", "<f8", 6)]), n, off)
        off += rec.nbytes
        out["species"].append({"order": rec["id"].copy(), "x": rec["v"][:, 0].copy(),
                               "y": rec["v"][:, 1].copy(), "ux": rec["v"][:, 2].copy(),
                               "uy": rec["v"][:, 3].copy(), "Ex": rec["v"][:, 4].copy(),
                               "Ey": rec["v"][:, 5].copy()})
    return out


def by_id(sp):
    """Species arrays reordered by particle id."""
    o = np.argsort(sp["order"], kind="stable")
    return {k: v[o] for k, v in sp.items()}


def run(case, nsteps, dumps=(), variant="exact"):
    """Returns {"pre": dump, "energy": array, step: dump ...}."""
    exe = os.path.join(REF_OUT, "ref_harness_%s" % variant)
    with tempfile.TemporaryDirectory() as d:
        conf = os.path.join(d, "case.conf")
        state = os.path.join(d, "state.bin")
        write_conf(conf, case, max(nsteps, 1))
        write_state(state, case)
        r = subprocess.run([exe, conf, state, d, str(nsteps)] + [str(k) for k in dumps],
                           capture_output=True, text=True, timeout=3600)
        if r.returncode != 0:
            raise RuntimeError("reference harness failed: %s" % r.stderr[-2000:])
        out = {"pre": read_dump(os.path.join(d, "pre.bin")),
               "energy": np.fromfile(os.path.join(d, "energy.bin"), np.float64)}
        for k in dumps:
            out[k] = read_dump(os.path.join(d, "step%d.bin" % k))
    return out
