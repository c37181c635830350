"""Links the reference's host program and test drivers against the GPU
library through the drop-in sim layer (cpic_gb300/dropin/sim_gpu.c), the
way a maintainer integrates it: the reference tree's src/*.c minus sim.c,
plus sim_gpu.c, plus libcpic_gb300.so.

TEST INFRASTRUCTURE.  MPI, FFTW and HDF5 are absent here, so the same
single-rank shims as the oracle's reference build stand in for them
(oracle/shims); libconfig is this project's parser.  Outputs go to
tests/_dropin/ (git-ignored): cpic_gpu (src/cpic.c's main),
test_constant_speed_gpu, test_cyclotron_gpu and test_harmonic_gpu (test/*.c
unchanged).  The reference tree is the one oracle/build_ref.py finds (the
tree itself, or its staged view on the GPU host); on hosts without AVX2 the
portable intrinsics (oracle/shims_portable) stand in for the x86 ones.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402

REF = build_ref.REF
OUT = os.path.join(HERE, "_dropin")
LIBDIR = os.path.join(ROOT, "cpic_gb300", "_build")
HOST_SOURCES = ["field", "particle", "mover", "interpolate", "comm_plasma", "comm_field", "plist",
                "mat", "plasma", "specie", "config", "perf", "utils", "solver", "output", "boundary"]
# The stage entry points the drop-in defines for the GPU; the reference's own
# definitions (field.c, particle.c, mover.c, comm_plasma.c) are made weak in
# their objects (objcopy, the sources stay untouched), so the drop-in's win.
GPU_STAGES = ["stage_field_E", "stage_plasma_E", "stage_plasma_r", "stage_field_rho", "comm_plasma",
              "particle_comm_initial"]
# program -> (tree, path, extra flags).  test/harmonic.c prints its trace
# with the reference's debug macro, which only its debug builds enable
# (GLOBAL_DEBUG, Makefile:74).
PROGRAMS = {"cpic_gpu": ("ref", "src/cpic.c", []),
            "test_constant_speed_gpu": ("ref", "test/constant-speed.c", []),
            "test_cyclotron_gpu": ("ref", "test/cyclotron.c", []),
            "test_harmonic_gpu": ("ref", "test/harmonic.c", ["-DGLOBAL_DEBUG"]),
            "dropin_stages": ("repo", "tests/dropin_stages.c", [])}


def ref_root():
    """The reference tree the drop-in builds against, or None."""
    return build_ref.ref_root()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build():
    """Returns OUT, or None when no reference tree is available."""
    ref = ref_root()
    if ref is None:
        return None
    if not os.path.exists(os.path.join(LIBDIR, "libcpic_gb300.so")):
        raise RuntimeError("build the GPU library first (cpic_gb300/build.py)")
    os.makedirs(OUT, exist_ok=True)
    cflags = [f for f in build_ref.cflags(not build_ref.is_x86()) if f != "-std=c11"] + ["-std=gnu11"]
    inc = ["-iquote", os.path.join(ref, "src"), "-I", os.path.join(ROOT, "oracle", "shims"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ref, "include")]
    jobs, objs = [], []
    for s in HOST_SOURCES:
        o = os.path.join(OUT, s + ".o")
        jobs.append(["gcc"] + cflags + inc + ["-c", os.path.join(ref, "src", s + ".c"), "-o", o])
        objs.append(o)
    o = os.path.join(OUT, "sim_gpu.o")
    jobs.append(["gcc"] + cflags + inc + ["-c", os.path.join(ROOT, "cpic_gb300", "dropin", "sim_gpu.c"),
                                          "-o", o])
    objs.append(o)
    o = os.path.join(OUT, "shim_runtime.o")
    jobs.append(["gcc", "-std=gnu11", "-O2", "-I", os.path.join(ROOT, "oracle", "shims"), "-c",
                 os.path.join(ROOT, "oracle", "shims", "shim_runtime.c"), "-o", o])
    objs.append(o)
    mains = {}
    for name, (tree, f, extra) in PROGRAMS.items():
        o = os.path.join(OUT, name + "_main.o")
        jobs.append(["gcc"] + cflags + extra + ["-I", os.path.join(ref, "src")] + inc
                    + ["-c", os.path.join(ref if tree == "ref" else ROOT, f), "-o", o])
        mains[name] = o
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    weaken = []
    for g in GPU_STAGES:
        weaken += ["--weaken-symbol", g]
    for s in ("field", "particle", "mover", "comm_plasma"):
        _run(["objcopy"] + weaken + [os.path.join(OUT, s + ".o")])
    for name, o in mains.items():
        _run(["gcc", "-o", os.path.join(OUT, name), o] + objs
             + ["-L", LIBDIR, "-lcpic_gb300", "-Wl,-rpath," + LIBDIR, "-lm", "-lpthread"])
    return OUT


if __name__ == "__main__":
    print(build())
    sys.exit(0)
