"""cajitafluids_gb300: the cajitafluids per-timestep hot path on one GB300.

The compute path is libcfgpu.so (hand-written CUDA for sm_103a behind the C
ABI in include/cajitafluids_gb300.h).  This package holds the CUDA sources
(csrc/), the in-tree build (build.py), the ctypes binding (_lib.py), a
context handle (api.py), the header-only C++ mirror of the reference's
Solver / ProblemManager / TimeIntegrator / VelocityCorrector interfaces
(cpp/) and the seeded benchmark workloads (workloads.py).
"""
from .api import CfError, Context, SolverOptions  # noqa: F401

__all__ = ["CfError", "Context", "SolverOptions"]
