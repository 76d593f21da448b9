// Reference driver: the reference's own Solver<2> (src/Solver.hpp with
// Mesh, ProblemManager, TimeIntegrator, Interpolation, VelocityCorrector,
// BoundaryConditions, InflowSource and BodyForce), compiled unchanged from
// the reference's sources against the serial Kokkos/Cajita/MPI stand-ins in
// oracle/refshim, behind a small C ABI for the tests.
//
// TEST INFRASTRUCTURE ONLY: it pins the oracle (oracle/cf_oracle.c) to the
// reference's code.  Only oracle/build.py builds it, into oracle/_ref/, and
// only when the reference's sources are present; nothing in the product
// links or loads it.
//
// The run goes through the reference's public API: createSolver("serial",
// ...) with the "Reference" solver (Cajita's ReferenceConjugateGradient with
// the diagonal preconditioner VelocityCorrector builds, tolerance 1e-6 and
// 2000 iterations as src/VelocityCorrector.hpp:103-104 hard-codes them),
// then setup() and step() (src/Solver.hpp:125-147) or solve(t_final,
// write_freq) (:149-177).  The initial state is set through the
// ProblemManager's init functor (src/ProblemManager.hpp:186-263).
#include <Solver.hpp>

#include <cstdio>
#include <cstring>
#include <exception>

namespace {

using PM = CajitaFluids::ProblemManager<2, Kokkos::Serial, Kokkos::HostSpace>;
constexpr int kHalo = 3;  // src/Solver.hpp:78

// init functor: owned values from row-major arrays (NULL = zero)
struct InitFromArrays {
    int nx, ny;
    const double *q, *u, *v;
    bool operator()(Cajita::Cell, CajitaFluids::Field::Quantity, const int index[2], const double[2],
                    double& val) const {
        val = q ? q[(size_t)(index[1] - kHalo) * nx + (index[0] - kHalo)] : 0.0;
        return true;
    }
    bool operator()(Cajita::Face<Cajita::Dim::I>, CajitaFluids::Field::Velocity, const int index[2],
                    const double[2], double& val) const {
        val = u ? u[(size_t)(index[1] - kHalo) * (nx + 1) + (index[0] - kHalo)] : 0.0;
        return true;
    }
    bool operator()(Cajita::Face<Cajita::Dim::J>, CajitaFluids::Field::Velocity, const int index[2],
                    const double[2], double& val) const {
        val = v ? v[(size_t)(index[1] - kHalo) * nx + (index[0] - kHalo)] : 0.0;
        return true;
    }
};

template <class View>
void copy_owned(const View& f, int ox, int oy, double* out) {
    for (int j = 0; j < oy; ++j)
        for (int i = 0; i < ox; ++i) out[(size_t)j * ox + i] = f(i + kHalo, j + kHalo, 0);
}

}  // namespace

extern "C" {

typedef struct {
    int nx, ny;
    double lo[2], hi[2];
    int bc[4];  // boundary_type [left, bottom, right, top]: 0 SOLID, 1 FREE
    double src_loc[2], src_size[2], src_vel[2], src_q;
    double force[2];
    double density, dt;
} cfref_params;

// mode 0: setup() then nsteps step(); mode 1: solve(t_final, write_freq).
// Outputs: owned q (ny x nx), u (ny x nx+1), v (ny+1 x nx), p (ny x nx),
// the iteration count and status of every pressure solve (up to
// max_solves; *nsolves gets the number of solves) and the number of
// SiloWriter writes.  Returns 0, or -1 with a message in err.
int cfref_run(const cfref_params* prm, const double* q0, const double* u0, const double* v0, int mode, int nsteps,
              double t_final, int write_freq, double* q, double* u, double* v, double* p, int* iters, int* status,
              int max_solves, int* nsolves, int* writes, char* err, int errlen) {
    try {
        Cajita::refshim::solve_log().clear();
        CajitaFluids::refshim::silo_writes() = 0;
        CajitaFluids::refshim::last_problem_manager() = nullptr;
        const int nx = prm->nx, ny = prm->ny;
        Kokkos::Array<double, 4> box;
        box[0] = prm->lo[0];
        box[1] = prm->lo[1];
        box[2] = prm->hi[0];
        box[3] = prm->hi[1];
        CajitaFluids::BoundaryCondition<2> bc;
        for (int k = 0; k < 4; ++k) bc.boundary_type[k] = prm->bc[k];
        CajitaFluids::InflowSource<2> source({prm->src_loc[0], prm->src_loc[1]}, {prm->src_size[0], prm->src_size[1]},
                                             {prm->src_vel[0], prm->src_vel[1]}, prm->src_q);
        CajitaFluids::BodyForce<2> body(prm->force[0], prm->force[1]);
        Cajita::DimBlockPartitioner<2> partitioner;
        InitFromArrays init{nx, ny, q0, u0, v0};
        auto solver = CajitaFluids::createSolver("serial", MPI_COMM_WORLD, box, std::array<int, 2>{nx, ny},
                                                 partitioner, prm->density, init, bc, source, body, prm->dt,
                                                 std::string("Reference"), std::string("Diagonal"));
        if (mode == 0) {
            solver->setup();
            for (int s = 0; s < nsteps; ++s) solver->step();
        } else {
            solver->solve(t_final, write_freq);
        }
        const PM* pm = static_cast<const PM*>(CajitaFluids::refshim::last_problem_manager());
        if (!pm) throw std::runtime_error("no ProblemManager was registered");
        using CajitaFluids::Field::Quantity;
        using CajitaFluids::Field::Velocity;
        using CajitaFluids::Version::Current;
        copy_owned(pm->get(Cajita::Cell(), Quantity(), Current()), nx, ny, q);
        copy_owned(pm->get(Cajita::Face<Cajita::Dim::I>(), Velocity(), Current()), nx + 1, ny, u);
        copy_owned(pm->get(Cajita::Face<Cajita::Dim::J>(), Velocity(), Current()), nx, ny + 1, v);
        const auto& x = Cajita::refshim::last_solution();
        if (x.size() == (size_t)nx * ny) std::memcpy(p, x.data(), x.size() * sizeof(double));
        const auto& log = Cajita::refshim::solve_log();
        *nsolves = (int)log.size();
        for (int k = 0; k < (int)log.size() && k < max_solves; ++k) {
            iters[k] = log[k].iterations;
            status[k] = log[k].status;
        }
        *writes = CajitaFluids::refshim::silo_writes();
        return 0;
    } catch (const std::exception& e) {
        std::snprintf(err, errlen, "%s", e.what());
        return -1;
    }
}

// One stage of the reference's own functors on one entity, for the input
// known-answer tests: kind 0 cell inflow, 1/2 I/J-face inflow, 3/4 I/J-face
// body force, 5/6 I/J-face wall condition, 7 build_matrix.  value is read
// and written in place (for 7: the five matrix entries, initialised as
// initializeMatrixValues does before the call).
int cfref_functor(const cfref_params* prm, int kind, int gi, int gj, double x, double y, double* value) {
    CajitaFluids::BoundaryCondition<2> bc;
    for (int k = 0; k < 4; ++k) bc.boundary_type[k] = prm->bc[k];
    bc.min[0] = 0;
    bc.min[1] = 0;
    bc.max[0] = prm->nx - 1;  // src/Solver.hpp:109-110 with src/Mesh.hpp:74-78
    bc.max[1] = prm->ny - 1;
    CajitaFluids::InflowSource<2> source({prm->src_loc[0], prm->src_loc[1]}, {prm->src_size[0], prm->src_size[1]},
                                         {prm->src_vel[0], prm->src_vel[1]}, prm->src_q);
    CajitaFluids::BodyForce<2> body(prm->force[0], prm->force[1]);
    Kokkos::View<double***> a("entity", 1, 1, kind == 7 ? 5 : 1);
    const int nv = kind == 7 ? 5 : 1;
    for (int k = 0; k < nv; ++k) a(0, 0, k) = value[k];
    const double dt = prm->dt, area = 0.0;
    switch (kind) {
        case 0: source(Cajita::Cell(), a, 0, 0, x, y, dt, area); break;
        case 1: source(Cajita::Face<Cajita::Dim::I>(), a, 0, 0, x, y, dt, area); break;
        case 2: source(Cajita::Face<Cajita::Dim::J>(), a, 0, 0, x, y, dt, area); break;
        case 3: body(Cajita::Face<Cajita::Dim::I>(), a, 0, 0, x, y, dt, area); break;
        case 4: body(Cajita::Face<Cajita::Dim::J>(), a, 0, 0, x, y, dt, area); break;
        case 5: bc(Cajita::Face<Cajita::Dim::I>(), a, gi, gj, 0, 0); break;
        case 6: bc(Cajita::Face<Cajita::Dim::J>(), a, gi, gj, 0, 0); break;
        case 7: {
            double scale = value[5];
            bc.build_matrix(gi, gj, 0, 0, a, scale);
            break;
        }
        default: return -1;
    }
    for (int k = 0; k < nv; ++k) value[k] = a(0, 0, k);
    return 0;
}

}  // extern "C"
