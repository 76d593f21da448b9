"""Builds the CPU oracle (test infrastructure only) into oracle/_build/, and,
where the reference's sources are present, the reference driver into
oracle/_ref/.

gcc with -ffp-contract=off: the oracle's floating-point order is part of its
contract (explicit fma() only), so the compiler must not fuse anything.

The reference driver (oracle/ref_driver.cpp) compiles the reference's own
headers (src/*.hpp of CUP-ECS/cajitafluids) unchanged, against the serial
Kokkos/Cajita/MPI stand-ins in oracle/refshim, with the same flags: the
reference's expressions are then evaluated as written, one rounding per
operation.  The reference's sources are read from CF_REFERENCE_SRC (default
/root/reference/src); when they are absent (a machine without the
reference) nothing is built and build_reference() returns None.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcforacle.so")
SRC = [os.path.join(HERE, "cf_oracle.c")]
HDR = [os.path.join(HERE, "cf_oracle.h")]
CFLAGS = ["-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas"]


def build_oracle(force: bool = False) -> str:
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) <= t for f in SRC + HDR):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = [os.environ.get("CC", "gcc")] + CFLAGS + ["-o", tmp] + SRC + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


REF_BUILD = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_BUILD, "libcfref.so")
REF_DRIVER = os.path.join(HERE, "ref_driver.cpp")
REF_SHIM = os.path.join(HERE, "refshim")
REF_HEADERS = ("Solver.hpp", "Mesh.hpp", "ProblemManager.hpp", "TimeIntegrator.hpp", "Interpolation.hpp",
               "VelocityCorrector.hpp", "BoundaryConditions.hpp", "InflowSource.hpp", "BodyForce.hpp")


def reference_src() -> str:
    return os.environ.get("CF_REFERENCE_SRC", "/root/reference/src")


def build_reference(force: bool = False):
    """libcfref.so from the reference's unchanged headers, or None when the
    reference's sources are not on this machine."""
    src = reference_src()
    refs = [os.path.join(src, h) for h in REF_HEADERS]
    if not all(os.path.exists(f) for f in refs):
        return None
    deps = refs + [REF_DRIVER] + [os.path.join(REF_SHIM, f) for f in os.listdir(REF_SHIM)]
    if not force and os.path.exists(REF_LIB):
        t = os.path.getmtime(REF_LIB)
        if all(os.path.getmtime(f) <= t for f in deps):
            return REF_LIB
    os.makedirs(REF_BUILD, exist_ok=True)
    tmp = REF_LIB + ".tmp"
    # the stand-ins come first on the include path: they provide Kokkos,
    # Cajita, MPI and the Silo writer; everything else is the reference's
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", f"-I{REF_SHIM}", f"-I{src}", "-o", tmp, REF_DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference driver build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
