"""In-tree build of libcfgpu.so (the CUDA hot path behind the C ABI).

nvcc compiles each translation unit for sm_103a in parallel and links one
shared library next to this file.  FP64 device code is compiled with
--fmad=false (every fused multiply-add in the kernels is an explicit fma),
and host code with -ffp-contract=off, so that the FP64 path is reproducible
bit for bit across machines.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcfgpu.so")
SOURCES = ["cf_api.cu", "cf_fields.cu", "cf_project.cu", "cf_cg32.cu", "cf_adjoint.cu", "cf_noalloc.cu", "cf_mg.cu"]
HEADERS = ["cf_internal.cuh", "cf_ctx.cuh", "cf_adv32.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcfgpu.so")


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    files.append(os.path.join(ROOT, "include", "cajitafluids_gb300.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile and link libcfgpu.so; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


EXAMPLE_SRC = os.path.join(HERE, "cpp", "advection_gb300.cpp")
EXAMPLE_HDR = os.path.join(HERE, "cpp", "CajitaFluidsGB300.hpp")
EXAMPLE = os.path.join(HERE, "advection_gb300")


def build_example(force: bool = False) -> str:
    """The C++ driver over the reference-shaped interface (links libcfgpu.so)."""
    lib = build_library()
    if (not force and os.path.exists(EXAMPLE)
            and all(os.path.getmtime(f) <= os.path.getmtime(EXAMPLE) for f in (EXAMPLE_SRC, EXAMPLE_HDR, lib))):
        return EXAMPLE
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-ffp-contract=off", f"-I{ROOT}", EXAMPLE_SRC,
           f"-L{HERE}", "-lcfgpu", "-Wl,-rpath,$ORIGIN", "-o", EXAMPLE + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"example build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(EXAMPLE + ".tmp", EXAMPLE)
    return EXAMPLE


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
    print(build_example(force=True))
