"""Host logic of the C++ mirror (cajitafluids_gb300/cpp/), checked without a
GPU: the header compiles against the C ABI, Mesh<2> follows the reference's
geometry and its uniform-cell check (src/Mesh.hpp:41-103), the time step is
limited as src/Solver.hpp:96-106 does, InflowSource<2> builds its bounding box
(src/InflowSource.hpp:30-60), and createSolver rejects the CPU backends before
any device work.  No compute call is made."""
import math
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include <cstring>
#include "cajitafluids_gb300/cpp/CajitaFluidsGB300.hpp"
using namespace CajitaFluids;

int main(int argc, char** argv) {
    if (argc > 1 && std::strcmp(argv[1], "mesh") == 0) {
        Mesh<2> m({0.0, 0.0, 1.0, 1.0}, {512, 512}, 3);
        auto lo = m.minDomainGlobalCellIndex();
        auto hi = m.maxDomainGlobalCellIndex();
        std::printf("%.17g %d %d %d %d %d\n", m.cellSize(), lo[0], lo[1], hi[0], hi[1], m.haloCellWidth());
        try {
            Mesh<2> bad({0.0, 0.0, 1.0, 2.0}, {8, 8}, 3);
            std::printf("accepted\n");
        } catch (const std::logic_error& e) {
            std::printf("%s\n", e.what());
        }
        return 0;
    }
    if (argc > 1 && std::strcmp(argv[1], "dt") == 0) {
        // args: dt n ux uy fx fy
        double dt = std::atof(argv[2]);
        int n = std::atoi(argv[3]);
        InflowSource<2> src({0.2, 0.45}, {0.02, 0.1}, {std::atof(argv[4]), std::atof(argv[5])}, 3.0);
        BodyForce<2> body(std::atof(argv[6]), std::atof(argv[7]));
        std::printf("%.17g\n", limitTimeStep(dt, 1.0 / n, src, body));
        return 0;
    }
    if (argc > 1 && std::strcmp(argv[1], "source") == 0) {
        InflowSource<2> src({0.2, 0.45}, {0.02, 0.1}, {1.0, -2.0}, 3.0);
        std::printf("%.17g %.17g %.17g %.17g %.17g %.17g %d\n", src._bounding_box[0], src._bounding_box[1],
                    src._bounding_box[2], src._bounding_box[3], src._velocity[0], src._velocity[1], src._mode);
        return 0;
    }
    return 2;
}
"""


@pytest.fixture(scope="module")
def prog(built, tmp_path_factory):
    from cajitafluids_gb300.build import HERE
    d = tmp_path_factory.mktemp("cppmirror")
    src = os.path.join(d, "mirror_host.cpp")
    exe = os.path.join(d, "mirror_host")
    with open(src, "w") as f:
        f.write(PROGRAM)
    cxx = os.environ.get("CXX", "g++")
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-Wall", "-Wextra", "-Werror", f"-I{ROOT}", src, f"-L{HERE}",
                        "-lcfgpu", f"-Wl,-rpath,{HERE}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, *args):
    r = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return r.stdout.split("\n")


def test_mesh_geometry_and_uniform_cells(prog):
    """MeshTest.BasicParameters (tests/tstMesh.cpp:16-40): 512 cells on the
    unit box; a box whose sides are not a whole number of square cells is
    rejected with the reference's message."""
    out = _run(prog, "mesh")
    dx, lo0, lo1, hi0, hi1, halo = out[0].split()
    assert float(dx) == 1.0 / 512
    assert (int(lo0), int(lo1), int(hi0), int(hi1), int(halo)) == (0, 0, 511, 511, 3)
    assert out[1] == "Extent not evenly divisible by uniform cell size"


@pytest.mark.parametrize("dt,n,vel,force", [
    (0.05, 64, (3.0, 1.0), (0.0, -9.81)),     # limited by inflow + sqrt(|f| dx)
    (0.05, 64, (-1.0, -4.0), (0.0, 0.0)),     # limited by |V|
    (0.001, 64, (3.0, 1.0), (0.0, -9.81)),    # already below the limit
    (0.05, 64, (0.0, 0.0), (0.0, 0.0)),       # no speed: unchanged
])
def test_time_step_limit(prog, dt, n, vel, force):
    """Solver::Solver (src/Solver.hpp:96-106): umax = max(|U|, |V|) +
    sqrt(|f| dx); dt is replaced by dx / umax when it is larger."""
    got = float(_run(prog, "dt", dt, n, vel[0], vel[1], force[0], force[1])[0])
    dx = 1.0 / n
    umax = max(abs(vel[0]), abs(vel[1])) + math.sqrt(math.hypot(*force) * dx)
    expect = dx / umax if umax > 0 and dt > dx / umax else dt
    assert got == expect


def test_inflow_source_bounding_box(prog):
    """InflowSource<2> stores [x0, y0, x0 + w, y0 + h] and the velocity; the
    reference's clamp mode is the default."""
    vals = _run(prog, "source")[0].split()
    assert [float(v) for v in vals[:6]] == [0.2, 0.45, 0.2 + 0.02, 0.45 + 0.1, 1.0, -2.0]
    assert vals[6] == "0"


def test_driver_rejects_cpu_backends(built):
    """createSolver (src/Solver.hpp:283-350): the Serial / OpenMP / HIP
    backends are not part of this build, and an unknown name is an invalid
    backend; both are refused before a context is created."""
    from cajitafluids_gb300.build import build_example
    exe = build_example()
    for dev, msg in (("serial", "not part of this build"), ("openmp", "not part of this build"),
                     ("bogus", "invalid backend")):
        r = subprocess.run([exe, "-n", "8", "--steps", "1", "--device", dev], capture_output=True, text=True,
                           timeout=60)
        assert r.returncode == 1 and msg in r.stderr, (dev, r.stderr)
