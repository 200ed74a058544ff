"""Builds the GB300 kernel set in-tree with nvcc (sm_103a only).

Outputs (git-ignored):
  flow_gb300/libflow_gb300.so   the kernel set + C ABI of include/flow_gb300.h
  flow_gb300/flow.gb300         the C host driver (host/flow_main.c)

Usage: ``python -m flow_gb300.build`` or ``flow_gb300.build.build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libflow_gb300.so")
ARCH_LIB = os.path.join(PKG, "libflow_gb300_arch.so")
DRIVER = os.path.join(PKG, "flow.gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "-I" + os.path.join(ROOT, "include")]

# Per-translation-unit flags.  stages.cu reproduces the reference's IEEE
# evaluation order, so it must not contract a*b+c into fused multiply-adds.
UNIT_FLAGS = {
    "stages.cu": ["--fmad=false"],
}

SOURCES = ["stages.cu", "interface.cu", "fused.cu", "batched.cu", "profile.cu", "peaks.cu",
           "noalloc.cu", "selftest.cu", "init.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 kernel set needs the CUDA toolkit")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src), __file__] + _headers()
    if _stale(obj, deps):
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *UNIT_FLAGS.get(src, []), "-c",
               os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles every CUDA unit (in parallel) and links the shared library."""
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "lib64")
        cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "shared", "-Xlinker", "-rpath," + cuda_lib,
               "-o", LIB, *objs]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    _build_driver(verbose)
    return LIB


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(_nvcc()))


def _build_driver(verbose: bool) -> None:
    """The GPU arch layer (C, cudart) and the C host driver."""
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(_cuda_home(), "include")]
    cuda_lib = os.path.join(_cuda_home(), "lib64")
    link_cuda = ["-L" + cuda_lib, "-Wl,-rpath," + cuda_lib, "-lcudart"]
    arch_src = os.path.join(PKG, "host", "arch_gb300.c")
    if _stale(ARCH_LIB, [arch_src, LIB] + _headers()):
        # The arch layer's problem set-up calls the kernel set's device
        # rasteriser (gb300_fill_boxes).
        cmd = ["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", *inc, arch_src, "-o", ARCH_LIB,
               "-L" + PKG, "-lflow_gb300", "-Wl,-rpath,$ORIGIN", *link_cuda, "-pthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    src = os.path.join(PKG, "host", "flow_main.c")
    if not _stale(DRIVER, [src, LIB, ARCH_LIB] + _headers()):
        return
    cmd = ["gcc", "-O2", "-std=gnu99", *inc, src, "-o", DRIVER, "-L" + PKG,
           "-lflow_gb300", "-lflow_gb300_arch", "-Wl,-rpath,$ORIGIN", *link_cuda, "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
