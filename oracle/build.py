"""Builds the CPU oracle (test infrastructure only) into oracle/_build/.

gcc with -ffp-contract=off: the oracle's floating-point order is part of its
contract (explicit fma() only), so the compiler must not fuse anything.
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


if __name__ == "__main__":
    print(build_oracle(force=True))
