"""Links the reference's host program and test drivers against the GPU
library through the drop-in sim layer (cpic_gb300/dropin/sim_gpu.c), the
way a maintainer integrates it: the reference tree's src/*.c minus sim.c,
plus sim_gpu.c, plus libcpic_gb300.so.

TEST INFRASTRUCTURE.  MPI, FFTW and HDF5 are absent here, so the same
single-rank shims as the oracle's reference build stand in for them
(oracle/shims); libconfig is this project's parser.  Outputs go to
tests/_dropin/ (git-ignored): cpic_gpu (src/cpic.c's main),
test_constant_speed_gpu, test_cyclotron_gpu and test_harmonic_gpu (test/*.c
unchanged).
x86-64 only, because the reference uses AVX2 intrinsics.
"""
import concurrent.futures as cf
import os
import platform
import subprocess
import sys

REF = os.environ.get("CPIC_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_dropin")
LIBDIR = os.path.join(ROOT, "cpic_gb300", "_build")
HOST_SOURCES = ["field", "particle", "mover", "interpolate", "comm_plasma", "comm_field", "plist",
                "mat", "plasma", "specie", "config", "perf", "utils", "solver", "output", "boundary"]
CFLAGS = ["-std=gnu11", "-O2", "-ffp-contract=off", "-DNDEBUG", "-DUSE_VECTOR_256",
          "-march=core-avx2", "-Wno-unknown-pragmas", "-w"]
PROGRAMS = {"cpic_gpu": os.path.join(REF, "src", "cpic.c"),
            "test_constant_speed_gpu": os.path.join(REF, "test", "constant-speed.c"),
            "test_cyclotron_gpu": os.path.join(REF, "test", "cyclotron.c"),
            "test_harmonic_gpu": os.path.join(REF, "test", "harmonic.c")}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build():
    """Returns OUT, or None when the reference tree or x86-64 is absent."""
    if not os.path.isdir(REF) or platform.machine() not in ("x86_64", "AMD64"):
        return None
    if not os.path.exists(os.path.join(LIBDIR, "libcpic_gb300.so")):
        raise RuntimeError("build the GPU library first (cpic_gb300/build.py)")
    os.makedirs(OUT, exist_ok=True)
    inc = ["-iquote", os.path.join(REF, "src"), "-I", os.path.join(ROOT, "oracle", "shims"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(REF, "include")]
    jobs, objs = [], []
    for s in HOST_SOURCES:
        o = os.path.join(OUT, s + ".o")
        jobs.append(["gcc"] + CFLAGS + inc + ["-c", os.path.join(REF, "src", s + ".c"), "-o", o])
        objs.append(o)
    o = os.path.join(OUT, "sim_gpu.o")
    jobs.append(["gcc"] + CFLAGS + inc + ["-c", os.path.join(ROOT, "cpic_gb300", "dropin", "sim_gpu.c"),
                                          "-o", o])
    objs.append(o)
    o = os.path.join(OUT, "shim_runtime.o")
    jobs.append(["gcc", "-std=gnu11", "-O2", "-I", os.path.join(ROOT, "oracle", "shims"), "-c",
                 os.path.join(ROOT, "oracle", "shims", "shim_runtime.c"), "-o", o])
    objs.append(o)
    mains = {}
    for name, src in PROGRAMS.items():
        o = os.path.join(OUT, name + "_main.o")
        jobs.append(["gcc"] + CFLAGS + ["-I", os.path.join(REF, "src")] + inc + ["-c", src, "-o", o])
        mains[name] = o
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    for name, o in mains.items():
        _run(["gcc", "-o", os.path.join(OUT, name), o] + objs
             + ["-L", LIBDIR, "-lcpic_gb300", "-Wl,-rpath," + LIBDIR, "-lm", "-lpthread"])
    return OUT


if __name__ == "__main__":
    print(build())
    sys.exit(0)
