"""ctypes binding of libcpic_gb300.so (include/cpic_gpu.h).

The library is the product: there is no Python or CPU fallback.  If the
shared object has not been built, `load()` raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

FP64 = 0
MIXED = 1

STATUS = {
    0: "CPIC_OK", -1: "CPIC_EINVAL", -2: "CPIC_ENOMEM", -3: "CPIC_ECUDA", -4: "CPIC_EUMAX",
    -5: "CPIC_ENAN", -6: "CPIC_ECAPACITY", -7: "CPIC_EDONE", -8: "CPIC_ENODEV", -9: "CPIC_ESTATE",
    -10: "CPIC_ETIMEOUT",
}


class CpicError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed: %s (%d)" % (what, STATUS.get(code, "?"), code))
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int64), ("ny", ctypes.c_int64),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double),
        ("dt", ctypes.c_double), ("e0", ctypes.c_double),
        ("B", ctypes.c_double * 3),
        ("plasma_chunks", ctypes.c_int64), ("cycles", ctypes.c_int64),
        ("precision", ctypes.c_int32), ("tile_x", ctypes.c_int32), ("tile_y", ctypes.c_int32),
        ("halo", ctypes.c_int32), ("track_ids", ctypes.c_int32),
        ("particles_per_thread", ctypes.c_int32), ("reserved", ctypes.c_int32 * 6),
    ]


class AdjParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int64), ("ny", ctypes.c_int64),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double),
        ("dt", ctypes.c_double), ("e0", ctypes.c_double),
        ("q", ctypes.c_double), ("m", ctypes.c_double), ("Bz", ctypes.c_double),
        ("nsteps", ctypes.c_int64), ("checkpoint_every", ctypes.c_int64),
        ("precision", ctypes.c_int32), ("reserved", ctypes.c_int32 * 7),
    ]


_LIB = None
D = ctypes.POINTER(ctypes.c_double)

# (name, restype, argtypes) for every entry point of include/cpic_gpu.h
SIGNATURES = [
    ("cpic_create", ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]),
    ("cpic_destroy", None, [ctypes.c_void_p]),
    ("cpic_add_species", ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int64, D, D, D, D]),
    ("cpic_pre_step", ctypes.c_int, [ctypes.c_void_p]),
    ("cpic_step", ctypes.c_int, [ctypes.c_void_p]),
    ("cpic_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    ("cpic_stage_field_E", ctypes.c_int, [ctypes.c_void_p]),
    ("cpic_stage_plasma", ctypes.c_int, [ctypes.c_void_p]),
    ("cpic_iter", ctypes.c_int64, [ctypes.c_void_p]),
    ("cpic_nspecies", ctypes.c_int, [ctypes.c_void_p]),
    ("cpic_species_count", ctypes.c_int64, [ctypes.c_void_p, ctypes.c_int]),
    ("cpic_get_particles", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, D, D, D]),
    ("cpic_set_particles", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, D, D, D]),
    ("cpic_gather_E", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, D, D]),
    ("cpic_get_rho", ctypes.c_int, [ctypes.c_void_p, D]),
    ("cpic_get_phi", ctypes.c_int, [ctypes.c_void_p, D]),
    ("cpic_get_E", ctypes.c_int, [ctypes.c_void_p, D, D]),
    ("cpic_set_E", ctypes.c_int, [ctypes.c_void_p, D, D]),
    ("cpic_set_rho", ctypes.c_int, [ctypes.c_void_p, D]),
    ("cpic_cell_counts", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    ("cpic_diag", ctypes.c_int, [ctypes.c_void_p, D]),
    ("cpic_field_energy", ctypes.c_int, [ctypes.c_void_p, D]),
    ("cpic_selftest_wait", ctypes.c_int, [ctypes.c_uint32]),
    ("cpic_compact", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("cpic_fp64_peak", ctypes.c_int, [ctypes.c_int64, D, D]),
    ("cpic_status_bits", ctypes.c_uint32, [ctypes.c_void_p]),
    ("cpic_time_steps", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, D, D, D]),
    ("cpic_tile_info", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    ("cpic_layout_stats", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    ("cpic_field_tile_copy", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    ("cpic_poisson_noalloc", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_int64, ctypes.c_void_p]),
    ("cpic_ensemble_create", ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_void_p)]),
    ("cpic_ensemble_destroy", None, [ctypes.c_void_p]),
    ("cpic_ensemble_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, D,
                                         ctypes.POINTER(ctypes.c_int32)]),
    ("cpic_autotune_tile", ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int64, ctypes.c_double,
                                          ctypes.c_double, ctypes.POINTER(ctypes.c_int32), D]),
    ("cpic_autotune_layout", ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int64, ctypes.c_double,
                                            ctypes.c_double, ctypes.POINTER(ctypes.c_int32),
                                            ctypes.POINTER(ctypes.c_int32), D]),
    ("cpic_adj_create", ctypes.c_int, [ctypes.POINTER(AdjParams), ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    ("cpic_adj_destroy", None, [ctypes.c_void_p]),
    ("cpic_adj_forward", ctypes.c_int, [ctypes.c_void_p, D, D, D, D, D]),
    ("cpic_adj_backward", ctypes.c_int, [ctypes.c_void_p, D, D, D, D]),
    ("cpic_adj_times", ctypes.c_int, [ctypes.c_void_p, D, D]),
    ("cpic_uniform", None, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int64, D]),
    ("cpic_normal", None, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int64, D]),
    ("cpic_init_two_stream", None, [ctypes.c_uint64, ctypes.c_int, ctypes.c_int64,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, D, D, D, D]),
    ("cpic_init_maxwellian", None, [ctypes.c_uint64, ctypes.c_int, ctypes.c_int64,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, D, D, D, D]),
]


def load(path=None):
    """Load the shared library (build it first with cpic_gb300.build)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or _build.LIB
    if not os.path.exists(path):
        raise RuntimeError("libcpic_gb300.so is not built (%s); run cpic_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(D)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def init_two_stream(seed, species, n, Lx, Ly, v0, vth, amp):
    lib = load()
    out = [np.empty(n, np.float64) for _ in range(4)]
    lib.cpic_init_two_stream(seed, species, n, Lx, Ly, v0, vth, amp, *[_dp(a) for a in out])
    return out


def init_maxwellian(seed, species, n, Lx, Ly, vth, driftx=0.0, drifty=0.0):
    lib = load()
    out = [np.empty(n, np.float64) for _ in range(4)]
    lib.cpic_init_maxwellian(seed, species, n, Lx, Ly, vth, driftx, drifty, *[_dp(a) for a in out])
    return out


def uniform(seed, stream, n):
    lib = load()
    out = np.empty(n, np.float64)
    lib.cpic_uniform(seed, stream, n, _dp(out))
    return out


class Context:
    """One resident simulation (cpic_ctx_t)."""

    def __init__(self, nx, ny, Lx, Ly, dt, e0=1.0, B=(0.0, 0.0, 0.0), precision=FP64,
                 plasma_chunks=1, cycles=0, tile=0, halo=0, track_ids=True, ppt=0):
        self.lib = load()
        p = Params()
        p.nx, p.ny, p.Lx, p.Ly, p.dt, p.e0 = nx, ny, Lx, Ly, dt, e0
        p.B[0], p.B[1], p.B[2] = B
        p.plasma_chunks, p.cycles = plasma_chunks, cycles
        p.precision, p.tile_x, p.tile_y, p.halo = precision, tile, tile, halo
        p.track_ids = 1 if track_ids else 0
        p.particles_per_thread = ppt
        h = ctypes.c_void_p()
        self._check(self.lib.cpic_create(ctypes.byref(p), ctypes.byref(h)), "cpic_create")
        self.h = h
        self.nx, self.ny = nx, ny
        self.counts = []

    @staticmethod
    def _check(r, what):
        if r < 0:
            raise CpicError(r, what)
        return r

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpic_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_species(self, q, m, x, y, ux, uy):
        x, y, ux, uy = (_f64(a) for a in (x, y, ux, uy))
        s = self._check(self.lib.cpic_add_species(self.h, q, m, len(x), _dp(x), _dp(y), _dp(ux), _dp(uy)),
                        "cpic_add_species")
        self.counts.append(len(x))
        return s

    def pre_step(self):
        self._check(self.lib.cpic_pre_step(self.h), "cpic_pre_step")

    def step(self):
        return self._check(self.lib.cpic_step(self.h), "cpic_step")

    def run(self, n):
        self._check(self.lib.cpic_run(self.h, n), "cpic_run")

    def stage_field_E(self):
        self._check(self.lib.cpic_stage_field_E(self.h), "cpic_stage_field_E")

    def stage_plasma(self):
        self._check(self.lib.cpic_stage_plasma(self.h), "cpic_stage_plasma")

    @property
    def iter(self):
        return self.lib.cpic_iter(self.h)

    def particles(self, s):
        n = self.counts[s]
        out = [np.empty(n, np.float64) for _ in range(4)]
        self._check(self.lib.cpic_get_particles(self.h, s, *[_dp(a) for a in out]), "cpic_get_particles")
        return out

    def set_particles(self, s, x, y, ux, uy):
        x, y, ux, uy = (_f64(a) for a in (x, y, ux, uy))
        self._check(self.lib.cpic_set_particles(self.h, s, _dp(x), _dp(y), _dp(ux), _dp(uy)),
                    "cpic_set_particles")

    def gather_E(self, s):
        n = self.counts[s]
        ex, ey = np.empty(n), np.empty(n)
        self._check(self.lib.cpic_gather_E(self.h, s, _dp(ex), _dp(ey)), "cpic_gather_E")
        return ex, ey

    def rho(self):
        out = np.empty((self.ny, self.nx))
        self._check(self.lib.cpic_get_rho(self.h, _dp(out)), "cpic_get_rho")
        return out

    def set_rho(self, rho):
        rho = _f64(rho)
        self._check(self.lib.cpic_set_rho(self.h, _dp(rho)), "cpic_set_rho")

    def phi(self):
        out = np.empty((self.ny, self.nx))
        self._check(self.lib.cpic_get_phi(self.h, _dp(out)), "cpic_get_phi")
        return out

    def E(self):
        ex, ey = np.empty((self.ny + 1, self.nx)), np.empty((self.ny + 1, self.nx))
        self._check(self.lib.cpic_get_E(self.h, _dp(ex), _dp(ey)), "cpic_get_E")
        return ex, ey

    def set_E(self, ex, ey):
        ex, ey = _f64(ex), _f64(ey)
        self._check(self.lib.cpic_set_E(self.h, _dp(ex), _dp(ey)), "cpic_set_E")

    def cell_counts(self):
        out = np.empty((self.ny, self.nx), np.int64)
        self._check(self.lib.cpic_cell_counts(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
                    "cpic_cell_counts")
        return out

    def diag(self):
        out = np.empty(5)
        self._check(self.lib.cpic_diag(self.h, _dp(out)), "cpic_diag")
        return dict(WE=out[0], KE=out[1], Q=out[2], Px=out[3], Py=out[4])

    def compact(self, slack_pct):
        self._check(self.lib.cpic_compact(self.h, slack_pct), "cpic_compact")

    def field_energy(self):
        out = np.empty(2)
        self._check(self.lib.cpic_field_energy(self.h, _dp(out)), "cpic_field_energy")
        return out[0]

    def status(self):
        return self.lib.cpic_status_bits(self.h)

    def time_steps(self, n):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.cpic_time_steps(self.h, n, ctypes.byref(a), ctypes.byref(b),
                                             ctypes.byref(c)), "cpic_time_steps")
        return dict(ms_total=a.value, ms_plasma=b.value, ms_field=c.value)

    def layout_stats(self):
        out = (ctypes.c_int64 * 4)()
        self._check(self.lib.cpic_layout_stats(self.h, out), "cpic_layout_stats")
        return dict(last_spill=out[0], rebuilds=out[1], slack_pct=out[2], blocks_per_sm=out[3])

    def field_tile_copy(self):
        """1 when the fused kernel copies field tiles with 2D tensor copies."""
        out = ctypes.c_int32()
        self._check(self.lib.cpic_field_tile_copy(self.h, ctypes.byref(out)), "cpic_field_tile_copy")
        return out.value

    def tile_info(self):
        out = (ctypes.c_int32 * 4)()
        self._check(self.lib.cpic_tile_info(self.h, out), "cpic_tile_info")
        return dict(tile_x=out[0], tile_y=out[1], halo=out[2], slack_pct=out[3])


class Adjoint:
    """Differentiable run (cpic_adj_t): loss = final field energy, gradient
    with respect to the initial particle state."""

    def __init__(self, nx, ny, Lx, Ly, dt, e0, q, m, n, nsteps, checkpoint_every, Bz=0.0,
                 precision=FP64):
        self.lib = load()
        p = AdjParams()
        p.nx, p.ny, p.Lx, p.Ly, p.dt, p.e0 = nx, ny, Lx, Ly, dt, e0
        p.q, p.m, p.Bz = q, m, Bz
        p.nsteps, p.checkpoint_every, p.precision = nsteps, checkpoint_every, precision
        h = ctypes.c_void_p()
        r = self.lib.cpic_adj_create(ctypes.byref(p), n, ctypes.byref(h))
        if r < 0:
            raise CpicError(r, "cpic_adj_create")
        self.h, self.n = h, n

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpic_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, x, y, ux, uy):
        x, y, ux, uy = (_f64(a) for a in (x, y, ux, uy))
        out = ctypes.c_double()
        r = self.lib.cpic_adj_forward(self.h, _dp(x), _dp(y), _dp(ux), _dp(uy), ctypes.byref(out))
        if r < 0:
            raise CpicError(r, "cpic_adj_forward")
        return out.value

    def backward(self):
        g = [np.empty(self.n, np.float64) for _ in range(4)]
        r = self.lib.cpic_adj_backward(self.h, *[_dp(a) for a in g])
        if r < 0:
            raise CpicError(r, "cpic_adj_backward")
        return g

    def times(self):
        f, b = ctypes.c_double(), ctypes.c_double()
        self.lib.cpic_adj_times(self.h, ctypes.byref(f), ctypes.byref(b))
        return f.value, b.value


class Ensemble:
    """Independent prepared runs (Context objects) stepped by one CUDA graph."""

    def __init__(self, runs):
        self.lib = load()
        self.runs = list(runs)
        arr = (ctypes.c_void_p * len(self.runs))(*[r.h.value for r in self.runs])
        h = ctypes.c_void_p()
        r = self.lib.cpic_ensemble_create(arr, len(self.runs), ctypes.byref(h))
        if r < 0:
            raise CpicError(r, "cpic_ensemble_create")
        self.h = h

    def run(self, nsteps):
        ms = ctypes.c_double()
        caps = ctypes.c_int32()
        r = self.lib.cpic_ensemble_run(self.h, nsteps, ctypes.byref(ms), ctypes.byref(caps))
        if r < 0:
            raise CpicError(r, "cpic_ensemble_run")
        return ms.value, caps.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpic_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_tile(nx, ny, Lx, Ly, dt, n, v0, vth, precision=MIXED, e0=1.0):
    """(tile, ms per step) chosen by the library's autotuner."""
    lib = load()
    p = Params()
    p.nx, p.ny, p.Lx, p.Ly, p.dt, p.e0 = nx, ny, Lx, Ly, dt, e0
    p.plasma_chunks, p.precision = 1, precision
    t = ctypes.c_int32()
    ms = ctypes.c_double()
    r = lib.cpic_autotune_tile(ctypes.byref(p), n, v0, vth, ctypes.byref(t), ctypes.byref(ms))
    if r < 0:
        raise CpicError(r, "cpic_autotune_tile")
    return t.value, ms.value


def autotune_layout(nx, ny, Lx, Ly, dt, n, v0, vth, precision=MIXED, e0=1.0):
    """(tile, particles per thread, ms per step) chosen by the library's
    autotuner over both."""
    lib = load()
    p = Params()
    p.nx, p.ny, p.Lx, p.Ly, p.dt, p.e0 = nx, ny, Lx, Ly, dt, e0
    p.plasma_chunks, p.precision = 1, precision
    t, ppt = ctypes.c_int32(), ctypes.c_int32()
    ms = ctypes.c_double()
    r = lib.cpic_autotune_layout(ctypes.byref(p), n, v0, vth, ctypes.byref(t), ctypes.byref(ppt),
                                 ctypes.byref(ms))
    if r < 0:
        raise CpicError(r, "cpic_autotune_layout")
    return t.value, ppt.value, ms.value


def fp64_peak(iters=1 << 16):
    """Measured FP64 GFLOP/s of the current device (cpic_fp64_peak)."""
    lib = load()
    g, ms = ctypes.c_double(), ctypes.c_double()
    r = lib.cpic_fp64_peak(iters, ctypes.byref(g), ctypes.byref(ms))
    if r < 0:
        raise CpicError(r, "cpic_fp64_peak")
    return g.value, ms.value
