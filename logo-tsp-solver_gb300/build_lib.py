"""Builds liblogo_gpu.so in-tree for sm_103a (no torch involved).

Each .cu translation unit is compiled by nvcc in parallel into _build/, then
linked into logo-tsp-solver_gb300/liblogo_gpu.so with the static CUDA runtime.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblogo_gpu.so")
SOURCES = ["sweep.cu", "tour.cu", "coop.cu", "capi.cu", "diag.cu", "construct.cpp", "batch.cu",
           "capi_batch.cu", "noalloc.cu", "neighbour.cu",
           "serve.cu", "capi_server.cu"]
# host files whose floating point must not be contracted into FMAs
NO_CONTRACT = {"construct.cpp"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I" + os.path.join(HERE, "..", "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return "nvcc"


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if src in NO_CONTRACT:
        cmd += ["-Xcompiler", "-ffp-contract=off"]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose_ptxas=False, force=False):
    """Compiles every translation unit and links the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "logo_gpu.h"))
    if (not force and not verbose_ptxas and os.path.exists(LIB) and
            os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "static", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(verbose_ptxas="-v" in sys.argv, force=True)
    print(LIB)
