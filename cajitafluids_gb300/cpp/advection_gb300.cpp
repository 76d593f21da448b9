// Driver mirroring examples/advection.cpp of CUP-ECS/cajitafluids on the
// GB300 path: all-SOLID walls, zero initial state, one inflow block, body
// force (0, -g), createSolver + solve (examples/advection.cpp:438-461).
//
// Defaults are the reference's (:168-189): PCG with the PFMG preconditioner
// name, served here by the geometric multigrid V-cycle.
//
// Extra options: --steps N runs exactly N steps after setup instead of
// t_final / dt; --linear samples the advected field linearly; --tol sets the
// solver tolerance; --out FILE writes the final owned fields as raw FP64
// ("CFGB" magic, nx, ny, then q, u, v, p in x-fastest order); --write-dir DIR
// turns on the SiloWriter output (DIR/CajitaFluids%05d.cfraw every -w steps,
// as Solver::solve writes Silo files).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "CajitaFluidsGB300.hpp"

template <std::size_t Dim>
struct MeshInitFunc {
    double _q, _u[Dim];
    MeshInitFunc(double q, std::array<double, Dim> u) : _q(q) {
        _u[0] = u[0];
        _u[1] = u[1];
    }
    KOKKOS_INLINE_FUNCTION bool operator()(Cajita::Cell, CajitaFluids::Field::Quantity, const int*, const double*,
                                           double& quantity) const {
        quantity = _q;
        return true;
    }
    KOKKOS_INLINE_FUNCTION bool operator()(Cajita::Face<Cajita::Dim::I>, CajitaFluids::Field::Velocity, const int*,
                                           const double*, double& xvelocity) const {
        xvelocity = _u[0];
        return true;
    }
    KOKKOS_INLINE_FUNCTION bool operator()(Cajita::Face<Cajita::Dim::J>, CajitaFluids::Field::Velocity, const int*,
                                           const double*, double& yvelocity) const {
        yvelocity = _u[1];
        return true;
    }
};

static void dump(const char* path, const CajitaFluids::ProblemManager<2>& pm) {
    FILE* f = fopen(path, "wb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    auto q = pm.get(Cajita::Cell(), CajitaFluids::Field::Quantity(), CajitaFluids::Version::Current());
    auto u = pm.get(Cajita::Face<Cajita::Dim::I>(), CajitaFluids::Field::Velocity(), CajitaFluids::Version::Current());
    auto v = pm.get(Cajita::Face<Cajita::Dim::J>(), CajitaFluids::Field::Velocity(), CajitaFluids::Version::Current());
    auto p = pm.pressure();
    int hdr[3] = {0x42474643, q.nx, q.ny};
    fwrite(hdr, sizeof(int), 3, f);
    for (auto* h : {&q, &u, &v, &p}) fwrite(h->data.data(), sizeof(double), h->data.size(), f);
    fclose(f);
}

int main(int argc, char** argv) {
    std::string device = "gb300", solver = "PCG", precon = "PFMG", out, write_dir;
    double t_final = 4.0, delta_t = 0.005, density = 0.1, gravity = 0.0, quantity = 3.0, tol = 1.0e-6;
    int n = 128, write_freq = 20, steps = -1, order = 3;
    std::array<double, 2> inLocation{{0.2, 0.45}}, inSize{{0.02, 0.1}}, inVelocity{{1.0, 0.0}};
    for (int k = 1; k < argc; ++k) {
        std::string a = argv[k];
        auto next = [&]() -> const char* {
            if (k + 1 >= argc) {
                fprintf(stderr, "missing value for %s\n", a.c_str());
                exit(2);
            }
            return argv[++k];
        };
        if (a == "-n") n = atoi(next());
        else if (a == "-t") t_final = atof(next());
        else if (a == "-d") delta_t = atof(next());
        else if (a == "-g") gravity = atof(next());
        else if (a == "-m") solver = next();
        else if (a == "-p") precon = next();
        else if (a == "-w") write_freq = atoi(next());
        else if (a == "--device") device = next();
        else if (a == "--steps") steps = atoi(next());
        else if (a == "--linear") order = 1;
        else if (a == "--tol") tol = atof(next());
        else if (a == "--out") out = next();
        else if (a == "--write-dir") write_dir = next();
        else if (a == "--inflow") {
            inLocation = {{atof(next()), atof(next())}};
            inSize = {{atof(next()), atof(next())}};
            inVelocity = {{atof(next()), atof(next())}};
            quantity = atof(next());
        } else {
            fprintf(stderr, "unknown option %s\n", a.c_str());
            return 2;
        }
    }
    if (n <= 0 || write_freq <= 0) {
        fprintf(stderr, "bad arguments\n");
        return 2;
    }
    try {
        CajitaFluids::BoundaryCondition<2> bc;
        bc.boundary_type = {CajitaFluids::BoundaryType::SOLID, CajitaFluids::BoundaryType::SOLID,
                            CajitaFluids::BoundaryType::SOLID, CajitaFluids::BoundaryType::SOLID};
        CajitaFluids::InflowSource<2> source(inLocation, inSize, inVelocity, quantity);
        CajitaFluids::BodyForce<2> body(0.0, -gravity);
        MeshInitFunc<2> initializer(0.0, {0.0, 0.0});
        if (device != "gb300" && device != "cuda") {
            auto s = CajitaFluids::createSolver(device, {0, 0, 1.0, 1.0}, {n, n}, density, initializer, bc, source,
                                                body, delta_t, solver, precon);
        }
        CajitaFluids::Solver<2> s({0, 0, 1.0, 1.0}, {n, n}, density, initializer, bc, source, body, delta_t, solver,
                                  precon, false, {false, false}, order);
        s.setTolerance(tol, 100000);
        if (!write_dir.empty()) s.setOutputDirectory(write_dir);
        if (steps < 0) {
            s.solve(t_final, write_freq);
        } else {
            // Solver::solve's loop (src/Solver.hpp:149-177) for a fixed step count
            if (s.siloWriter()) s.siloWriter()->siloWrite("Mesh", 0, s.time(), s.timeStep());
            s.setup();
            for (int k = 0; k < steps; ++k) {
                s.step();
                if (s.siloWriter() && 0 == k % write_freq) s.siloWriter()->siloWrite("Mesh", k, s.time(), s.timeStep());
            }
        }
        const cf_solve_stats& st = s.lastStats();
        printf("done: t = %.6f dt = %.6e iterations %d div_l2 %.3e status %d\n", s.time(), s.timeStep(),
               st.iterations, st.div_l2, st.status);
        if (!out.empty()) dump(out.c_str(), *s.problemManager());
    } catch (const std::exception& e) {
        fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
