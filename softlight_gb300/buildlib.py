"""Builds the in-tree CUDA library softlight_gb300/libslg.so for sm_103a.

Every translation unit is compiled with --fmad=false (no contraction of a*b+c
into one rounding), IEEE division and square root and no flush-to-zero, and
host code with -ffp-contract=off, because the draw path reproduces the
reference CPU rasteriser's binary32 arithmetic bit for bit.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libslg.so")

SOURCES = ["slg_builtin_raster_rgba8.cu", "slg_builtin_raster_rgbaf.cu", "slg_builtin_raster_rf.cu",
           "slg_builtin_vertex.cu", "slg_kernels.cu", "slg_context.cu", "slg_adjoint.cu"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-Xptxas", "-warn-spills",
]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(verbose=False, force=False):
    """Compile the CUDA sources and link libslg.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inc = os.path.join(HERE, "..", "include")
    deps += [os.path.join(inc, f) for f in os.listdir(inc)]
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(d) for d in deps if os.path.exists(d))
        if os.path.getmtime(LIB) >= newest and os.path.getmtime(LIB) >= os.path.getmtime(__file__):
            return LIB
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", tmp, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
