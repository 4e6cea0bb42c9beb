"""Build libsmx_gb300.so (the GB300 engine behind include/smx_gb300.h).

Compiles every CUDA translation unit for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`), in parallel, into
symmetrix_gb300/_build/.  No cmake, no torch extension machinery: plain nvcc/g++.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsmx_gb300.so")
ROOT = os.path.dirname(HERE)

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
            "-I", SRC, "-I", os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-I", SRC, "-I", os.path.join(ROOT, "include")]

CU_SOURCES = ["k_edge.cu", "k_layer1.cu", "k_umma.cu", "k_node.cu", "k_md.cu", "engine.cu", "md.cu", "noalloc.cu", "pair.cu"]
CXX_SOURCES = ["model.cpp", "model_cache.cpp"]


def _deps():
    src = [f for f in os.listdir(SRC) if f.endswith((".cu", ".cuh", ".h", ".hpp", ".cpp"))]
    return [os.path.join(SRC, f) for f in src] + [os.path.join(ROOT, "include", "smx_gb300.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps())


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r


def build(force=False, verbose_ptxas=False):
    """Compile (if sources changed) and return the path of libsmx_gb300.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(OUT, f + ".o")
        objs.append(o)
        extra = ["-Xptxas", "-v"] if verbose_ptxas else []
        jobs.append([NVCC] + ARCH + CU_FLAGS + extra + ["-c", os.path.join(SRC, f), "-o", o])
    for f in CXX_SOURCES:
        o = os.path.join(OUT, f + ".o")
        objs.append(o)
        jobs.append(["g++"] + CXX_FLAGS + ["-c", os.path.join(SRC, f), "-o", o])
    logs = []
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for cmd, r in ex.map(_compile, jobs):
            if r.returncode != 0:
                raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
            logs.append(r.stderr)
    tmp = LIB + ".tmp"
    r = subprocess.run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    if verbose_ptxas:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
