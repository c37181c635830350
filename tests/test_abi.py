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


def test_exports_libconfig_subset(lib):
    text = open(os.path.join(ROOT, "include", "libconfig.h")).read()
    names = set(re.findall(r"\b(config_\w+)\s*\(", text))
    assert len(names) >= 30
    for s in names:
        assert hasattr(lib, s), s


def test_conf_parser_reads_reference_syntax(lib, tmp_path):
    conf = tmp_path / "a.conf"
    inc = tmp_path / "b.conf"
    inc.write_text('extra = { k = 0x10L; }\n')
    conf.write_text("""# comment
species = ( { name = "e" "lectron"; particles = 3; charge = -1.0 },
            { name = "ion"; particles = 4; charge = 1.0e+0 } );
grid = { points = [64, 32] }   // trailing
/* block
   comment */
simulation : { time_step = 5.0e-2; flag = true; space_length = [6.28, 3.14]; }
@include "b.conf"
""")

    class C(ctypes.Structure):
        _fields_ = [("pad", ctypes.c_char * 512)]
    c = C()
    lib.config_init(ctypes.byref(c))
    assert lib.config_read_file(ctypes.byref(c), str(conf).encode()) == 1
    v = ctypes.c_double()
    lib.config_lookup.restype = ctypes.c_void_p
    assert lib.config_lookup_float(ctypes.byref(c), b"simulation.time_step", ctypes.byref(v)) == 1
    assert v.value == 5.0e-2
    i = ctypes.c_int()
    assert lib.config_lookup_int(ctypes.byref(c), b"grid.points.[1]", ctypes.byref(i)) == 1
    assert i.value == 32
    # an integer setting is not a float (no auto-conversion, as libconfig)
    assert lib.config_lookup_float(ctypes.byref(c), b"grid.points.[0]", ctypes.byref(v)) == 0
    ll = ctypes.c_longlong()
    assert lib.config_lookup_int64(ctypes.byref(c), b"extra.k", ctypes.byref(ll)) == 1
    assert ll.value == 16
    s = ctypes.c_char_p()
    assert lib.config_lookup_string(ctypes.byref(c), b"species.[0].name", ctypes.byref(s)) == 1
    assert s.value == b"electron"
    sp = lib.config_lookup(ctypes.byref(c), b"species")
    lib.config_setting_length.argtypes = [ctypes.c_void_p]
    assert lib.config_setting_length(sp) == 2
    lib.config_destroy(ctypes.byref(c))
    bad = tmp_path / "bad.conf"
    bad.write_text("a = ;\n")
    c2 = C()
    lib.config_init(ctypes.byref(c2))
    assert lib.config_read_file(ctypes.byref(c2), str(bad).encode()) == 0
    lib.config_error_line.restype = ctypes.c_int
    assert lib.config_error_line(ctypes.byref(c2)) == 1
    lib.config_destroy(ctypes.byref(c2))


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
    p.nx, p.ny = 3, 64                  # below the 4-cell minimum
    p.Lx = p.Ly = 1.0
    p.dt = 0.1
    p.e0 = 1.0
    h = ctypes.c_void_p()
    assert lib.cpic_create(ctypes.byref(p), ctypes.byref(h)) == -1
    p.nx = 1 << 15                      # above 16384
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


def test_oracle_init_matches_library_init(lib):
    """The CPU legs of the benchmark build their inputs with the oracle's
    restatement of the seeded init methods (so they load no product
    library); it must give the product's arrays bit for bit."""
    from oracle import oracle
    L = 2 * np.pi
    for args in ((2024, 0, 5001, L, L, 0.2, 0.01, 0.01), (3, 1, 777, L, 2 * L, 0.1, 0.0, 0.05),
                 (9, 0, 640, L, L, 0.3, 0.02, 0.0)):
        a = _lib.init_two_stream(*args)
        b = oracle.init_two_stream(*args)
        for u, v in zip(a, b):
            assert np.array_equal(u, v)
    a = _lib.init_maxwellian(11, 1, 3000, L, L, 0.05, 0.01, -0.02)
    b = oracle.init_maxwellian(11, 1, 3000, L, L, 0.05, 0.01, -0.02)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
