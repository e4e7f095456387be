"""Build recipe of the GPU library (libamie_gpu.so), in-tree, for sm_103a.

Each .cu translation unit is compiled by its own nvcc process in parallel and
the objects are linked into one shared library next to this file.  Nothing
here needs cmake or torch; `nvcc` from the CUDA toolkit is enough.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libamie_gpu.so")
SOURCES = ["common.cu", "assemble.cu", "solver.cu", "fields.cu", "noalloc.cu", "cut_rules.cu", "damage.cu"]
# per-file flags: the damage grading mirrors the reference's arithmetic operation by operation
FILE_FLAGS = {"damage.cu": ["--fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "include"), "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *FILE_FLAGS.get(src, []), *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
    return obj


def _stale(objs) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(REPO, "include", "amie_gpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and not _stale(None):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    return LIB


def build_cpp_test() -> str:
    """The C++ driver of gpu::Assembly used by tests/test_cpp_assembly.py."""
    lib = build()
    exe = os.path.join(BUILD, "test_gpu_assembly")
    srcs = [os.path.join(HERE, "host", "gpu_assembly.cpp"), os.path.join(REPO, "tests", "cpp", "test_gpu_assembly.cpp")]
    if os.path.exists(exe) and all(os.path.getmtime(s) < os.path.getmtime(exe) for s in srcs + [lib]):
        return exe
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), "-I", os.path.join(HERE, "host"), *srcs,
           "-L", HERE, "-lamie_gpu", f"-Wl,-rpath,{HERE}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed:\n{r.stderr[-4000:]}")
    return exe


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
