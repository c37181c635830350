"""Build the reference (rodarima/cpic) from its own sources, in place,
against the project-written shims, into oracle/_ref/ (git-ignored).

TEST INFRASTRUCTURE ONLY.  Two variants:
  shipped: src/*.c as they are (keeps the AVX2 lane-conflict loss of the
           charge deposit, src/simd_avx2.h:392-410);
  exact:   the same files through a symlink farm whose simd_avx2.h adds
           colliding lanes one by one (oracle/exact/simd_avx2.h).
Each variant yields ref_harness_<variant> (oracle/ref_harness.c) and the
reference's own tests test_constant_speed_<variant>,
test_cyclotron_<variant> (test/*.c), which read conf/*.conf relative to
the reference tree.

The reference needs MPI, FFTW3-MPI, libconfig, OmpSs-2/nanos6 and HDF5,
none of which exist here: mpi.h, fftw3*.h, nanos6/debug.h and hdf5.h come
from oracle/shims, libconfig.h from include/ with this project's parser
(cpic_gb300/csrc/cpic_conf.c).  The MFT_TAP backend (mft_tap.c, tap.c,
mft_worker.c) and the plotter are left out; cpic.c is left out because the
harness and the tests bring their own main.

Hosts.  On x86-64 the reference's AVX2 code compiles with the system
intrinsics headers (-march=core-avx2).  Elsewhere (the Arm host of the GPU)
oracle/shims_portable/x86intrin.h stands in for them, lane by lane with the
same IEEE semantics; on x86-64 the same portable build is made as a third
variant (shipped_portable) that a CPU test checks bit for bit against the
native one.

Where the tree comes from (ref_root): the directory named by CPIC_REFERENCE
(default /root/reference) when it exists; there stage() also copies the
tree's src/, include/, test/ and conf/ into oracle/_ref/tree/, the build
input of the same builds on the GPU host, where the reference tree itself
is absent.  oracle/_ref/ is git-ignored: the copy is never committed, and it
is refreshed from the tree at every build here.  The reference tree is read,
never written.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

REF = os.environ.get("CPIC_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
TREE = os.path.join(OUT, "tree")
STAGED_DIRS = ("src", "include", "test", "conf")
SOURCES = ["sim", "field", "particle", "mover", "interpolate", "comm_plasma", "comm_field", "plist",
           "mat", "plasma", "specie", "config", "perf", "utils", "solver", "output", "boundary"]
BASE_CFLAGS = ["-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-DNDEBUG", "-DUSE_VECTOR_256",
               "-Wno-unknown-pragmas", "-w"]
PORTABLE_INC = ["-I", os.path.join(HERE, "shims_portable")]


def is_x86():
    return platform.machine() in ("x86_64", "AMD64")


def cflags(portable):
    """Compiler flags of a reference build: native AVX2 on x86-64, else the
    portable intrinsics (which go ahead of the system headers)."""
    return BASE_CFLAGS + (PORTABLE_INC if portable else ["-march=core-avx2"])


def stage():
    """Copies the reference tree's src/, include/, test/ and conf/ (data
    files included) into oracle/_ref/tree/.  Returns the staged root, or
    None when the reference tree is absent."""
    if not os.path.isdir(os.path.join(REF, "src")):
        return None
    for d in STAGED_DIRS:
        src_d = os.path.join(REF, d)
        if not os.path.isdir(src_d):
            continue
        for dirpath, _, files in os.walk(src_d):
            rel = os.path.relpath(dirpath, REF)
            dst_d = os.path.join(TREE, rel)
            os.makedirs(dst_d, exist_ok=True)
            for f in files:
                dst = os.path.join(dst_d, f)
                if os.path.lexists(dst):
                    os.remove(dst)
                shutil.copy2(os.path.join(dirpath, f), dst)
    return TREE


def ref_root():
    """The reference tree to build from: CPIC_REFERENCE when present (after
    refreshing the staged view), else the staged view if it holds the
    sources, else None."""
    if os.path.isdir(os.path.join(REF, "src")):
        stage()
        return REF
    if os.path.isfile(os.path.join(TREE, "src", "sim.c")):
        return TREE
    return None


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError("%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _farm(ref, variant):
    """Directory holding the variant's src view (symlinks only)."""
    if variant != "exact":
        return os.path.join(ref, "src")
    d = os.path.join(OUT, "exact_src")
    os.makedirs(d, exist_ok=True)
    for f in os.listdir(os.path.join(ref, "src")):
        if not (f.endswith(".c") or f.endswith(".h")):
            continue
        dst = os.path.join(d, f)
        src = os.path.join(HERE, "exact", f) if f == "simd_avx2.h" else os.path.join(ref, "src", f)
        if os.path.lexists(dst):
            os.remove(dst)
        os.symlink(src, dst)
    return d


def variants():
    """(name, portable) of the variants this host builds."""
    if is_x86():
        return [("shipped", False), ("exact", False), ("shipped_portable", True)]
    return [("shipped", True), ("exact", True)]


def _stale(stamp):
    """Whether a file of this project that the build compiles or includes
    (the shims, the oracle's FFT and generator headers, the harness, the
    configuration parser) is newer than the stamp."""
    deps = [os.path.join(HERE, "shims", f) for f in os.listdir(os.path.join(HERE, "shims"))]
    deps += [os.path.join(HERE, f) for f in ("orc_fft.h", "seed_init.h", "ref_harness.c")]
    deps += [os.path.join(HERE, "shims_portable", f)
             for f in os.listdir(os.path.join(HERE, "shims_portable"))]
    deps += [os.path.join(HERE, "exact", f) for f in os.listdir(os.path.join(HERE, "exact"))]
    deps.append(os.path.join(ROOT, "cpic_gb300", "csrc", "cpic_conf.c"))
    t = os.path.getmtime(stamp)
    return any(os.path.getmtime(d) > t for d in deps if os.path.isfile(d))


def build(force=False):
    ref = ref_root()
    if ref is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    # one stamp per host architecture: the copy of this directory on the GPU
    # host carries the stamp of this one but none of its binaries
    stamp = os.path.join(OUT, "built_%s.txt" % platform.machine())
    if os.path.exists(stamp) and not force and not _stale(stamp):
        return OUT
    inc = ["-I", os.path.join(HERE, "shims"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ref, "include")]
    jobs = []
    common_objs = []
    o = os.path.join(OUT, "shim_runtime.o")
    jobs.append(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-I", os.path.join(HERE, "shims"),
                 "-c", os.path.join(HERE, "shims", "shim_runtime.c"), "-o", o])
    common_objs.append(o)
    o = os.path.join(OUT, "cpic_conf.o")
    jobs.append(["gcc", "-std=gnu11", "-O2", "-c", os.path.join(ROOT, "cpic_gb300", "csrc", "cpic_conf.c"),
                 "-o", o])
    common_objs.append(o)
    variant_objs = {}
    for v, portable in variants():
        src = _farm(ref, v)
        extra = ['-DORC_REF_SIMD_AVX2="%s"' % os.path.join(ref, "src", "simd_avx2.h")] if v == "exact" else []
        flags = cflags(portable)
        vinc = ["-iquote", src] + inc
        objs = []
        for s in SOURCES:
            o = os.path.join(OUT, "%s_%s.o" % (v, s))
            jobs.append(["gcc"] + flags + extra + vinc + ["-c", os.path.join(src, s + ".c"), "-o", o])
            objs.append(o)
        for name, path in (("harness", os.path.join(HERE, "ref_harness.c")),
                           ("t_cs", os.path.join(ref, "test", "constant-speed.c")),
                           ("t_cy", os.path.join(ref, "test", "cyclotron.c"))):
            o = os.path.join(OUT, "%s_%s.o" % (v, name))
            jobs.append(["gcc"] + flags + extra + ["-I", src] + inc + ["-c", path, "-o", o])
        variant_objs[v] = objs
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    for v, objs in variant_objs.items():
        for name, exe in (("harness", "ref_harness_%s" % v), ("t_cs", "test_constant_speed_%s" % v),
                          ("t_cy", "test_cyclotron_%s" % v)):
            _run(["gcc", "-o", os.path.join(OUT, exe), os.path.join(OUT, "%s_%s.o" % (v, name))]
                 + objs + common_objs + ["-lm", "-lpthread"])
    with open(stamp, "w") as f:
        f.write("reference built from %s/src with oracle shims (%s)\n"
                % (ref, ", ".join(v for v, _ in variants())))
    return OUT


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
