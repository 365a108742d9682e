"""In-tree build of the CUDA library ``libgalnode.so`` for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel and the
objects are linked into one shared library next to this file.  No CMake, no
setuptools: a rebuild is a few nvcc invocations.
"""

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgalnode.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "177"]
SOURCES = ["galnode.cu", "evolve_plain.cu", "evolve_surrogate.cu", "evolve_fast.cu", "evolve_fast_surrogate.cu",
           "evolve_forest_plain.cu", "evolve_forest_fast.cu", "forest.cu", "calibrate.cu", "surrogate_train.cu",
           "trees.cpp", "trees_gpu.cu"]
# Host code whose FP64 results must match the oracle's bit for bit: no contraction.
NO_CONTRACT = {"forest.cu"}
# Device code whose FP64 arithmetic follows the oracle's operation by operation: no FMA contraction.
NO_FMAD = {"trees_gpu.cu"}
# Sources whose host code uses OpenMP.
OPENMP = {"trees.cpp", "trees_gpu.cu", "forest.cu"}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if src in OPENMP:
        cmd[1:1] = ["-Xcompiler", "-fopenmp"]
    if src in NO_CONTRACT:
        cmd[1:1] = ["-Xcompiler", "-ffp-contract=off"]
    if src in NO_FMAD:
        cmd[1:1] = ["--fmad=false"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    """Compile every CUDA source and link ``libgalnode.so``."""
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        for _, log in results:
            print(log)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
