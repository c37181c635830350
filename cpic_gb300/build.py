"""In-tree build of the CUDA library libcpic_gb300.so for sm_103a.

Each translation unit is compiled in parallel with nvcc; the FP64 unit and
the host context are built with --fmad=false (the FP64 form must round like
the reference's C code), the mixed-precision unit with FMA contraction on.
Outputs go to cpic_gb300/_build/ (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcpic_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
               "-Xptxas", "-v", "-I", os.path.join(ROOT, "include")] + ARCH

UNITS = [
    ("cpic_ctx.cu", ["--fmad=false"]),
    ("cpic_fp64.cu", ["--fmad=false"]),
    ("cpic_mixed.cu", ["--fmad=true"]),
    ("cpic_noalloc.cu", ["--fmad=false"]),
    ("cpic_adjoint.cu", ["--fmad=true"]),
    ("cpic_peak.cu", ["--fmad=true"]),
]
C_UNITS = ["cpic_init.c", "cpic_conf.c"]


def _nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _sources():
    files = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    files.append(os.path.join(ROOT, "include", "cpic_gpu.h"))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _sources())


def build(verbose=False, force=False):
    """Compile every unit and link the shared library.  Returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for name, flags in UNITS:
        obj = os.path.join(OUT, name.replace(".cu", ".o"))
        objs.append(obj)
        jobs.append([nvcc] + NVCC_COMMON + flags + ["-c", os.path.join(SRC, name), "-o", obj])
    for name in C_UNITS:
        obj = os.path.join(OUT, name.replace(".c", ".o"))
        objs.append(obj)
        jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-fopenmp", "-ffp-contract=off",
                     "-I", os.path.join(ROOT, "include"), "-c", os.path.join(SRC, name), "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    link = [nvcc, "-shared"] + ARCH + ["-Xcompiler", "-fopenmp", "-o", LIB] + objs + ["-lgomp"]
    logs.append(_run(link))
    if verbose:
        sys.stdout.write("\n".join(logs))
    with open(os.path.join(OUT, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force=True)
    print(LIB)
