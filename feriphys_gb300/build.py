"""Build libferiphys_gb300.so in-tree for sm_103a (nvcc + g++, no cmake).

Each translation unit compiles in parallel into feriphys_gb300/_build/, then
nvcc links the shared library next to this file.  Device code is compiled with
-fmad=false and host code with -ffp-contract=off: the step keeps the
reference's f32 evaluation order, and a fused multiply-add would change the
rounding of every force term.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libferiphys_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build feriphys_gb300")


def _cuda_include(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "feriphys_gb300.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def _compile(src: str, nvcc: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc, "-c", path, "-o", obj, "-O3", "-std=c++17", *ARCH, "-lineinfo", "-fmad=false",
               "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC, "-I", INCLUDE, *extra]
    else:
        cmd = ["g++", "-c", path, "-o", obj, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
               "-fno-fast-math", "-I", CSRC, "-I", INCLUDE, "-I", _cuda_include(nvcc)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force: bool = False, verbose: bool = False, extra_nvcc: list[str] | None = None) -> str:
    """Compile every CUDA/C++ source and link the library; returns its path."""
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, extra_nvcc or []), srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-shared", "-o", tmp, *objs, *ARCH, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
