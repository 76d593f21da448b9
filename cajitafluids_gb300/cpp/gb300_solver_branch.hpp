// The "gb300" device branch a maintainer adds to the reference's
// createSolver (src/Solver.hpp:283-350).  It is pasted into src/Solver.hpp
// beside the Kokkos solvers, where SolverBase, BoundaryCondition<2>,
// InflowSource<2>, BodyForce<2> and Kokkos::Array are already declared; it
// drives the whole step through the C ABI of include/cajitafluids_gb300.h.
#include <cajitafluids_gb300.h>

class GB300Solver : public SolverBase {
  public:
    GB300Solver(const Kokkos::Array<double, 4>& box, const std::array<int, 2>& n, double density,
                const BoundaryCondition<2>& bc, const InflowSource<2>& src, const BodyForce<2>& body,
                double dt, const std::string& solver, const std::string& precon)
        : _dt(dt), _solver(solver), _precon(precon) {
        cf_grid_desc d{n[0], n[1], {box[0], box[1]}, {box[2], box[3]}, {0, 0}, CF_PREC_FP64, 0};
        check(cf_ctx_create(&d, &_ctx));
        check(cf_set_bc(_ctx, bc.boundary_type.data()));
        std::array<double, 2> loc{src._bounding_box[0], src._bounding_box[1]};
        std::array<double, 2> size{src._bounding_box[2] - loc[0], src._bounding_box[3] - loc[1]};
        check(cf_set_source(_ctx, loc.data(), size.data(), src._velocity.data(), src._quantity, 0));
        check(cf_set_body_force(_ctx, body._force.data(), 0));
        check(cf_set_density(_ctx, density));
        _opts = {_solver.c_str(), _precon.c_str(), 1.0e-6, 0.0, 2000, 0.0, 0};
    }
    // upload the initial Kokkos state once: CUDA views are LayoutLeft (i fastest)
    template <class View> void upload(int field, const View& host_owned) {
        check(cf_upload(_ctx, field, host_owned.data(), host_owned.stride(0), host_owned.stride(1)));
    }
    void setup() override { check(cf_setup(_ctx, _dt, &_opts, &_stats)); }
    void step() override { check(cf_step(_ctx, _dt, 3, &_opts, &_stats)); }
    // Solver::solve, :149-177: the steps between two write points in one
    // device-side loop (cf_steps); the C++ mirror's Solver::solve does this
    // with the reference's step count, prints and writes
    void solve(double t_final, int write_freq) override {
        setup();
        int total = 0;  // the reference loop's step count: time grows one dt at a time
        for (double tm = _time; total == 0 || tm < t_final; ++total) tm += _dt;
        for (int t = 0; t < total; ) {
            int n = (t % write_freq == 0) ? 1 : std::min(total, (t / write_freq + 1) * write_freq) - t;
            int bad = 0;
            check(cf_steps(_ctx, n, _dt, 3, &_opts, &_stats, &bad));
            for (int k = 0; k < n; ++k) _time += _dt;
            t += n;
        }
    }
    ~GB300Solver() { cf_ctx_destroy(_ctx); }

  private:
    void check(int rc) { if (rc != CF_OK && rc != CF_ERR_NOT_CONVERGED)
                             throw std::runtime_error(cf_last_error(_ctx)); }
    cf_ctx* _ctx = nullptr;
    double _dt, _time = 0.0;
    std::string _solver, _precon;
    cf_solver_opts _opts;
    cf_solve_stats _stats;
};

// in createSolver(...):
//     else if ( 0 == device.compare( "gb300" ) )
//         return std::make_shared<GB300Solver>( global_bounding_box, global_num_cell, density,
//                                               bc, source, body, delta_t, matrix_solver, preconditioner );
