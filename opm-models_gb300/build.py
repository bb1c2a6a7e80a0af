"""Build libgbfv.so in-tree (opm-models_gb300/_build/) for sm_103a.

Translation units are compiled in parallel and linked with nvcc.  The
linearization kernels are compiled with ``-fmad=false`` so their FP64
rounding follows the written operation order; host code is compiled with
``-ffp-contract=off`` for the same reason (boundary fluid states and face
geometry are evaluated on the host).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgbfv.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr"] + ARCH

UNITS = {
    "linearize.cu": ["-fmad=false"],
    "solver.cu": [],
    "amg.cu": ["-fmad=false"],
    "gbfv.cu": [],
    "noalloc.cu": [],
    "batchround.cu": ["-fmad=false"],
    "restart.cu": [],
    "vtk.cu": [],
    "problem.cu": [],
    "vcfv.cu": ["-fmad=false"],
    "gilu.cu": [],
}


def _nvcc():
    for c in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        try:
            subprocess.run([c, "--version"], capture_output=True, check=True)
            return c
        except (OSError, subprocess.CalledProcessError):
            continue
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "gbfv.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    nvcc = _nvcc()

    def compile_unit(item):
        src, extra = item
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [nvcc] + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
