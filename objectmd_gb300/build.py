"""Builds libomdg.so for sm_103a with nvcc, in-tree (objectmd_gb300/_build/).

One -gencode (compute_103a -> sm_103a), translation units compiled in
parallel, no CMake.  The library links the CUDA runtime statically and
carries no PyTorch symbols.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libomdg.so")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC", "-Xptxas",
           "-warn-spills"] + ARCH
SOURCES = ["api.cu", "nlist.cu", "eam.cu", "eam_fast.cu", "pair.cu", "threebody.cu", "integrate.cu", "io.cu",
           "static_count.cu", "nn_net.cu", "nn_train.cu", "nn_potential.cu", "ttm.cu", "table.cpp",
           "checkpoint.cpp", "output.cu", "waits.cu", "fdtd.cu"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    headers = [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "omdg.h"))
    if not _newer(obj, [src] + headers):
        return obj
    cmd = [NVCC] + CUFLAGS + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, proc.stdout, proc.stderr))
    if verbose and proc.stderr.strip():
        print(proc.stderr, flush=True)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(SRC, s) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _newer(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (proc.stdout, proc.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
