"""Build libmsq_cuda.so in-tree: one nvcc job per translation unit, in
parallel, for sm_103a only, then one link step.

Usage: python mixed-mlx_gb300/build.py [--debug]
"""
from __future__ import annotations

import concurrent.futures as futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmsq_cuda.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu"))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC)
                    if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(INCLUDE, "msq_cuda.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d)
                                   for d in deps if os.path.exists(d)):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
    return obj


def build(debug: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-DMSQ_BOUNDS_CHECK=1"] if debug else []
    srcs = sources()
    with futures.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
    if verbose:
        print(LIB)
    return LIB


def build_backend_check() -> str:
    """Compile the C++ driver of the cuda_backend mirror (tests/cpp), linked
    against libmsq_cuda.so; the GPU tests run it like the reference's CLI."""
    root = os.path.dirname(HERE)
    src = os.path.join(root, "tests", "cpp", "cuda_backend_check.cpp")
    exe = os.path.join(root, "tests", "cpp", "cuda_backend_check")
    lib = build()
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(src),
                                                           os.path.getmtime(lib)):
        return exe
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    cmd = ["g++", "-std=c++17", "-O2", src, "-o", exe, "-I" + CSRC, "-I" + INCLUDE,
           "-I" + os.path.join(cuda, "include"), "-L" + HERE, "-lmsq_cuda",
           "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + HERE,
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{res.stderr}")
    return exe


if __name__ == "__main__":
    build(debug="--debug" in sys.argv, verbose=True)
    if "--driver" in sys.argv:
        print(build_backend_check())
