"""The C++ mirror of the reference interfaces (cajitafluids_gb300/cpp/):
the advection driver built on createSolver/Solver<2> runs on the GPU and its
final fields equal the oracle's, bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from oracle import Oracle

pytestmark = pytest.mark.gpu


def _read_dump(path):
    with open(path, "rb") as f:
        magic, nx, ny = np.frombuffer(f.read(12), dtype=np.int32)
        assert magic == 0x42474643
        rest = np.frombuffer(f.read(), dtype=np.float64)
    sizes = [nx * ny, (nx + 1) * ny, nx * (ny + 1), nx * ny]
    shapes = [(ny, nx), (ny, nx + 1), (ny + 1, nx), (ny, nx)]
    out, k = {}, 0
    for name, sz, sh in zip(("q", "u", "v", "p"), sizes, shapes):
        out[name] = rest[k:k + sz].reshape(sh)
        k += sz
    return out


@pytest.mark.parametrize("precon", [None, "Diagonal"])
def test_cpp_driver_matches_oracle(built, tmp_path, precon):
    """Default preconditioner (PFMG, the reference CLI's default, served by
    the multigrid V-cycle) and the diagonal one."""
    from cajitafluids_gb300.build import build_example
    exe = build_example()
    n, steps = 40, 6
    out = os.path.join(tmp_path, "fields.bin")
    cmd = [exe, "-n", str(n), "--steps", str(steps), "--linear", "--tol", "1e-9", "--inflow", "0.45",
           "0.10", "0.10", "0.05", "0.0", "3.0", "1.0", "-d", "0.005", "--out", out]
    if precon:
        cmd += ["-p", precon]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = _read_dump(out)
    o = Oracle(n, n, source=((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0), density=0.1,
               precon_mg=precon is None)
    o.setup(0.005, tol=1e-9, max_iter=100000)
    for _ in range(steps):
        o.step(0.005, 1, tol=1e-9, max_iter=100000)
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(o.get(f), got[f]), f


def test_cpp_driver_rejects_unsupported_backend_and_solver(built):
    from cajitafluids_gb300.build import build_example
    exe = build_example()
    r = subprocess.run([exe, "-n", "8", "--steps", "1", "--device", "serial"], capture_output=True, text=True)
    assert r.returncode == 1 and "not part of this build" in r.stderr
    r = subprocess.run([exe, "-n", "8", "--steps", "1", "-p", "Euclid"], capture_output=True, text=True)
    assert r.returncode == 1 and "not implemented" in r.stderr
