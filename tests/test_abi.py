"""The C ABI library without a GPU: it loads, exports every entry point that
include/*.h declares, and its host-only init methods are deterministic."""
import ctypes
import os
import re

import numpy as np

from cpic_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"CPIC_API\s+[\w\s\*]+?\b(cpic_\w+)\s*\(", text):
            syms.add(m.group(1))
    return syms


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert syms == bound, syms ^ bound
    for s in syms:
        assert hasattr(lib, s), s


def test_no_device_reports_enodev(lib):
    import torch
    if torch.cuda.is_available():
        return
    p = _lib.Params()
    p.nx = p.ny = 64
    p.Lx = p.Ly = 1.0
    p.dt = 0.1
    p.e0 = 1.0
    h = ctypes.c_void_p()
    assert lib.cpic_create(ctypes.byref(p), ctypes.byref(h)) == -8


def test_invalid_params_rejected(lib):
    p = _lib.Params()
    p.nx, p.ny = 48, 64                 # not a power of two
    p.Lx = p.Ly = 1.0
    p.dt = 0.1
    p.e0 = 1.0
    h = ctypes.c_void_p()
    assert lib.cpic_create(ctypes.byref(p), ctypes.byref(h)) == -1
    p.nx = 64
    p.B[0] = 1.0                        # in-plane B: the reference rejects u_z != 0
    assert lib.cpic_create(ctypes.byref(p), ctypes.byref(h)) == -1


def splitmix_uniform(seed, stream, n):
    M = (1 << 64) - 1
    G = 0x9E3779B97F4A7C15

    def mix(z):
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    base = mix((seed * G + mix((stream + 0x632BE59BD9B4E019) & M)) & M)
    return np.array([(mix((base + (i + 1) * G) & M) >> 11) * 2.0 ** -53 for i in range(n)])


def test_uniform_stream_matches_splitmix(lib):
    a = _lib.uniform(1234, 5, 64)
    assert np.array_equal(a, splitmix_uniform(1234, 5, 64))


def test_two_stream_init_deterministic(lib):
    L = 2 * np.pi
    a = _lib.init_two_stream(7, 0, 1000, L, L, 0.2, 0.01, 0.01)
    b = _lib.init_two_stream(7, 0, 1000, L, L, 0.2, 0.01, 0.01)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    x, y, ux, uy = a
    assert ((x >= 0) & (x < L)).all() and ((y >= 0) & (y < L)).all()
    assert abs(ux[:500].mean() - 0.2) < 0.01 and abs(ux[500:].mean() + 0.2) < 0.01
