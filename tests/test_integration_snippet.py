"""The createSolver branch (cajitafluids_gb300/cpp/gb300_solver_branch.hpp,
the code a maintainer pastes into the reference's src/Solver.hpp) compiles
against the C ABI header and links against the library, with the reference's own types
(SolverBase, BoundaryCondition<2>, InflowSource<2>, BodyForce<2>) taken from
the C++ mirror and Kokkos::Array standing in as std::array.  Checked without a
GPU: nothing is run."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PRELUDE = r"""
#include <algorithm>
#include <array>
#include <memory>
#include <stdexcept>
#include <string>
#include "cajitafluids_gb300/cpp/CajitaFluidsGB300.hpp"
namespace Kokkos {
template <class T, std::size_t N>
using Array = std::array<T, N>;
}
using namespace CajitaFluids;
"""

EPILOGUE = r"""
int main(int argc, char**) {
    if (argc > 5) {  // never taken: the object is only built
        BoundaryCondition<2> bc;
        InflowSource<2> src({0.2, 0.45}, {0.02, 0.1}, {1.0, 0.0}, 3.0);
        BodyForce<2> body(0.0, -9.81);
        std::shared_ptr<SolverBase> s =
            std::make_shared<GB300Solver>(Kokkos::Array<double, 4>{0, 0, 1, 1}, std::array<int, 2>{64, 64}, 1.0,
                                          bc, src, body, 1e-3, std::string("PCG"), std::string("PFMG"));
        s->solve(0.1, 10);
    }
    return 0;
}
"""


def test_create_solver_branch_compiles(built, tmp_path):
    from cajitafluids_gb300.build import HERE
    with open(os.path.join(ROOT, "cajitafluids_gb300", "cpp", "gb300_solver_branch.hpp")) as f:
        body = f.read()
    src = os.path.join(tmp_path, "gb300_solver.cpp")
    with open(src, "w") as f:
        f.write(PRELUDE + body + EPILOGUE)
    exe = os.path.join(tmp_path, "gb300_solver")
    cxx = os.environ.get("CXX", "g++")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wno-unused-private-field", f"-I{ROOT}", f"-I{ROOT}/include",
                        src, f"-L{HERE}", "-lcfgpu", f"-Wl,-rpath,{HERE}", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
