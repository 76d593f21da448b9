"""The output path (src/SiloWriter.hpp): the cell-centred velocity the writer
interpolates (interpolateVelocity<2, 1> at cell centres) equals the oracle's
linear sample bit for bit, and the C++ mirror's SiloWriter<2> writes the mesh,
"quantity" and "velocity" variables of the state it was given."""
import os
import subprocess

import numpy as np
import pytest

from helpers import load_state, make_pair, pair_round, random_state

pytestmark = pytest.mark.gpu


def read_cfraw(path):
    with open(path, "rb") as f:
        raw = f.read()
    assert raw[:8] == b"CFSILO01"
    nx, ny, cycle = np.frombuffer(raw[8:20], dtype=np.int32)
    time, dt = np.frombuffer(raw[20:36], dtype=np.float64)
    rest = np.frombuffer(raw[36:], dtype=np.float64)
    X, Y = rest[:nx + 1], rest[nx + 1:nx + ny + 2]
    k = nx + ny + 2
    n = nx * ny
    q, u, v = (rest[k + i * n:k + (i + 1) * n].reshape(ny, nx) for i in range(3))
    assert rest.size == k + 3 * n
    return {"nx": int(nx), "ny": int(ny), "cycle": int(cycle), "time": float(time), "dt": float(dt), "X": X,
            "Y": Y, "quantity": q, "u": u, "v": v}


def cell_centres(nx, ny, dx, lo=(0.0, 0.0)):
    gi, gj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    # the coordinate of cell (i, j) as the kernels form it: gl + (idx + 1/2) dx, gl = lo - 3 dx
    x = (lo[0] - 3.0 * dx) + ((gi + 3).astype(np.float64) + 0.5) * dx
    y = (lo[1] - 3.0 * dx) + ((gj + 3).astype(np.float64) + 0.5) * dx
    return np.stack([x.ravel(), y.ravel()], axis=1)


@pytest.mark.parametrize("nx,ny,periodic,precision", [(40, 40, (False, False), "fp64"), (64, 32, (True, True), "fp64"),
                                                      (33, 20, (True, False), "fp64"), (48, 48, (False, False), "mixed")])
def test_cell_velocity_matches_oracle(built, nx, ny, periodic, precision):
    rng = np.random.default_rng(nx + ny)
    o, c = make_pair(nx, ny, periodic=periodic, precision=precision)
    st = random_state(o, rng)
    if precision == "mixed":
        # a mixed context keeps u, v as double-float pairs
        st["u"], st["v"] = pair_round(st["u"]), pair_round(st["v"])
    load_state(o, c, st)
    o.fill_ghosts()
    uc, vc = c.cell_velocity()
    xy = cell_centres(nx, ny, c.dx)
    assert np.array_equal(uc.ravel(), o.sample("u", 1, xy))
    assert np.array_equal(vc.ravel(), o.sample("v", 1, xy))
    # a uniform flow is reproduced at every cell centre; cells next to a wall
    # also touch its zero ghosts, with a weight that is zero only up to the
    # rounding of the cell-centre coordinate
    for f, val in (("u", 0.75), ("v", -1.25)):
        c.upload(f, np.full(o.shape(f), val))
    uc, vc = c.cell_velocity()
    assert np.all(uc[1:-1, 1:-1] == 0.75) and np.all(vc[1:-1, 1:-1] == -1.25)
    assert np.allclose(uc, 0.75, rtol=1e-14) and np.allclose(vc, -1.25, rtol=1e-14)


def test_cpp_silo_writer(built, tmp_path):
    from cajitafluids_gb300.build import build_example
    from oracle import Oracle
    exe = build_example()
    n, steps = 32, 4
    out = os.path.join(tmp_path, "fields.bin")
    r = subprocess.run([exe, "-n", str(n), "--steps", str(steps), "-w", "2", "--tol", "1e-9", "-d", "0.005",
                        "--inflow", "0.45", "0.10", "0.10", "0.05", "0.0", "3.0", "1.0", "--out", out,
                        "--write-dir", str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    files = sorted(f for f in os.listdir(tmp_path) if f.endswith(".cfraw"))
    # cycle 0 is written before setup and again after the first step (as
    # Solver::solve does, src/Solver.hpp:156,169-173); then every -w 2 steps
    assert files == ["CajitaFluids00000.cfraw", "CajitaFluids00002.cfraw"]
    first = read_cfraw(os.path.join(tmp_path, files[0]))
    assert first["nx"] == n and first["ny"] == n and first["cycle"] == 0
    assert np.allclose(first["X"], np.arange(n + 1) / n) and np.allclose(first["Y"], np.arange(n + 1) / n)
    last = read_cfraw(os.path.join(tmp_path, files[-1]))
    assert last["cycle"] == 2 and last["dt"] == 0.005
    # the same steps on the oracle: quantity and cell velocities bit for bit
    o = Oracle(n, n, source=((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0), density=0.1, precon_mg=True)
    o.setup(0.005, tol=1e-9, max_iter=100000)
    for _ in range(3):
        o.step(0.005, 3, tol=1e-9, max_iter=100000)
    assert np.array_equal(last["quantity"], o.get("q"))
    o.fill_ghosts()
    xy = cell_centres(n, n, 1.0 / n)
    assert np.array_equal(last["u"].ravel(), o.sample("u", 1, xy))
    assert np.array_equal(last["v"].ravel(), o.sample("v", 1, xy))
