"""ctypes wrapper of the oracle (cpic_oracle.c), the CPU restatement of the
reference's FP64 time step.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "cpic_oracle.c")

D = ctypes.POINTER(ctypes.c_double)
I64 = ctypes.POINTER(ctypes.c_int64)
_LIB = None


def build(force=False):
    """Compile the oracle with the reference's FP semantics (no contraction)."""
    deps = [SRC, os.path.join(HERE, "orc_fft.h"), os.path.join(HERE, "seed_init.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           SRC, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    build()
    lib = ctypes.CDLL(LIB)
    sig = [
        ("orc_create", ctypes.c_void_p, [ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, D, ctypes.c_int64]),
        ("orc_destroy", None, [ctypes.c_void_p]),
        ("orc_set_lossy_deposit", None, [ctypes.c_void_p, ctypes.c_int]),
        ("orc_iter", ctypes.c_int64, [ctypes.c_void_p]),
        ("orc_set_iter", None, [ctypes.c_void_p, ctypes.c_int64]),
        ("orc_error", ctypes.c_int, [ctypes.c_void_p]),
        ("orc_add_species", ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int64, D, D, D, D, D]),
        ("orc_set_particles", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, D, D, D, D]),
        ("orc_get_particles", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, D, D, D, D, D, D]),
        ("orc_get_rho", None, [ctypes.c_void_p, D]),
        ("orc_set_rho", None, [ctypes.c_void_p, D]),
        ("orc_get_phi", None, [ctypes.c_void_p, D]),
        ("orc_get_E", None, [ctypes.c_void_p, D, D]),
        ("orc_set_E", None, [ctypes.c_void_p, D, D]),
        ("orc_stage_field_E", ctypes.c_int, [ctypes.c_void_p]),
        ("orc_stage_plasma_E", ctypes.c_int, [ctypes.c_void_p]),
        ("orc_stage_plasma_r", ctypes.c_int, [ctypes.c_void_p]),
        ("orc_stage_field_rho", ctypes.c_int, [ctypes.c_void_p]),
        ("orc_pre_step", ctypes.c_int, [ctypes.c_void_p]),
        ("orc_step", ctypes.c_int, [ctypes.c_void_p]),
        ("orc_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
        ("orc_diag", None, [ctypes.c_void_p, D]),
        ("orc_cell_counts", None, [ctypes.c_void_p, I64]),
        ("orc_weights", None, [ctypes.c_double] * 6 + [D, I64]),
        ("orc_poisson", None, [ctypes.c_int64, ctypes.c_int64, D, D]),
        ("orc_init_two_stream", None, [ctypes.c_uint64, ctypes.c_int, ctypes.c_int64] + [ctypes.c_double] * 5
         + [D] * 4),
        ("orc_init_maxwellian", None, [ctypes.c_uint64, ctypes.c_int, ctypes.c_int64] + [ctypes.c_double] * 5
         + [D] * 4),
    ]
    for name, res, args in sig:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(D)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """FP64 CPU restatement of one simulation (same interface shape as
    cpic_gb300.Context)."""

    def __init__(self, nx, ny, Lx, Ly, dt, e0=1.0, B=(0.0, 0.0, 0.0), plasma_chunks=1, lossy=False):
        self.lib = load()
        b = (ctypes.c_double * 3)(*B)
        self.h = self.lib.orc_create(nx, ny, Lx, Ly, dt, e0, b, plasma_chunks)
        if not self.h:
            raise RuntimeError("orc_create failed")
        self.lib.orc_set_lossy_deposit(self.h, 1 if lossy else 0)
        self.nx, self.ny = nx, ny
        self.counts = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_species(self, q, m, x, y, ux, uy, uz=None):
        x, y, ux, uy = (_f64(a) for a in (x, y, ux, uy))
        uzp = _dp(_f64(uz)) if uz is not None else None
        s = self.lib.orc_add_species(self.h, q, m, len(x), _dp(x), _dp(y), _dp(ux), _dp(uy), uzp)
        self.counts.append(len(x))
        return s

    def set_particles(self, s, x, y, ux, uy):
        x, y, ux, uy = (_f64(a) for a in (x, y, ux, uy))
        self.lib.orc_set_particles(self.h, s, _dp(x), _dp(y), _dp(ux), _dp(uy), None)

    def particles(self, s):
        n = self.counts[s]
        out = [np.empty(n) for _ in range(4)]
        self.lib.orc_get_particles(self.h, s, *[_dp(a) for a in out], None, None, None)
        return out

    def particle_E(self, s):
        n = self.counts[s]
        ex, ey = np.empty(n), np.empty(n)
        self.lib.orc_get_particles(self.h, s, None, None, None, None, None, _dp(ex), _dp(ey))
        return ex, ey

    def pre_step(self):
        self.lib.orc_pre_step(self.h)

    def step(self):
        r = self.lib.orc_step(self.h)
        if r:
            raise RuntimeError("oracle step failed (velocity above umax)")

    def run(self, n):
        for _ in range(n):
            self.step()

    def stage_field_E(self):
        self.lib.orc_stage_field_E(self.h)

    def stage_plasma_E(self):
        self.lib.orc_stage_plasma_E(self.h)

    def stage_plasma_r(self):
        return self.lib.orc_stage_plasma_r(self.h)

    def stage_field_rho(self):
        self.lib.orc_stage_field_rho(self.h)

    @property
    def iter(self):
        return self.lib.orc_iter(self.h)

    @iter.setter
    def iter(self, v):
        self.lib.orc_set_iter(self.h, v)

    def rho(self):
        out = np.empty((self.ny, self.nx))
        self.lib.orc_get_rho(self.h, _dp(out))
        return out

    def set_rho(self, rho):
        self.lib.orc_set_rho(self.h, _dp(_f64(rho)))

    def phi(self):
        out = np.empty((self.ny, self.nx))
        self.lib.orc_get_phi(self.h, _dp(out))
        return out

    def E(self):
        ex, ey = np.empty((self.ny + 1, self.nx)), np.empty((self.ny + 1, self.nx))
        self.lib.orc_get_E(self.h, _dp(ex), _dp(ey))
        return ex, ey

    def set_E(self, ex, ey):
        self.lib.orc_set_E(self.h, _dp(_f64(ex)), _dp(_f64(ey)))

    def diag(self):
        out = np.empty(5)
        self.lib.orc_diag(self.h, _dp(out))
        return dict(WE=out[0], KE=out[1], Q=out[2], Px=out[3], Py=out[4])

    def cell_counts(self):
        out = np.empty((self.ny, self.nx), np.int64)
        self.lib.orc_cell_counts(self.h, out.ctypes.data_as(I64))
        return out


def weights(x, y, x0, y0, dx, dy):
    lib = load()
    w = np.empty(4)
    i0 = np.empty(2, np.int64)
    lib.orc_weights(x, y, x0, y0, dx, dy, _dp(w), i0.ctypes.data_as(I64))
    return w, i0


def poisson(rho):
    lib = load()
    rho = _f64(rho)
    ny, nx = rho.shape
    phi = np.empty_like(rho)
    lib.orc_poisson(nx, ny, _dp(rho), _dp(phi))
    return phi


def init_two_stream(seed, species, n, Lx, Ly, v0, vth, amp):
    """Seeded two-stream state (x, y, ux, uy), the same arrays as the
    product's init method of that name."""
    lib = load()
    out = [np.empty(n) for _ in range(4)]
    lib.orc_init_two_stream(seed, species, n, Lx, Ly, v0, vth, amp, *[_dp(a) for a in out])
    return out


def init_maxwellian(seed, species, n, Lx, Ly, vth, driftx=0.0, drifty=0.0):
    """Seeded uniform positions with a drifting Maxwellian (x, y, ux, uy)."""
    lib = load()
    out = [np.empty(n) for _ in range(4)]
    lib.orc_init_maxwellian(seed, species, n, Lx, Ly, vth, driftx, drifty, *[_dp(a) for a in out])
    return out
