// CajitaFluids on one GB300: a header-only C++ mirror of the reference's
// host interfaces (namespace CajitaFluids) over the C ABI of libcfgpu.so.
//
// Mirrored (CUP-ECS/cajitafluids paths):
//   BoundaryType, BoundaryCondition<2>     src/BoundaryConditions.hpp:30-135
//   InflowSource<2>                        src/InflowSource.hpp:30-98
//   BodyForce<2>                           src/BodyForce.hpp:30-69
//   Version::{Current,Next}, Field::{Quantity,Velocity}
//                                          src/ProblemManager.hpp:35-85
//   Mesh<2>                                src/Mesh.hpp:41-151
//   ProblemManager<2>                      src/ProblemManager.hpp:93-419
//   TimeIntegrator::step<2>                src/TimeIntegrator.hpp:120-177
//   VelocityCorrectorBase,
//   createVelocityCorrector                src/VelocityCorrector.hpp:37-42, 297-339
//   SolverBase, Solver<2>, createSolver    src/Solver.hpp:41-350
//
// Differences a caller sees: there is no MPI communicator or Cajita
// partitioner (one GPU holds the whole grid), the device string is "gb300"
// ("cuda" is accepted as a synonym), field access through get() returns
// host copies of the owned region, and errors are thrown as
// std::runtime_error carrying the ABI's message (the reference throws
// std::runtime_error for an invalid backend, src/Solver.hpp:305-348).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/cajitafluids_gb300.h"

#ifndef KOKKOS_INLINE_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#endif

// Entity tags with the reference's spelling, so init functors written for
// the Kokkos path (Cajita::Cell, Cajita::Face<Cajita::Dim::I>) compile as is.
namespace Cajita {
namespace Dim {
enum Values { I = 0, J = 1, K = 2 };
}
struct Cell {};
template <int D>
struct Face {};
}  // namespace Cajita

namespace CajitaFluids {

inline void check(cf_ctx* ctx, int rc, const char* what) {
    if (rc == CF_OK) return;
    std::string msg = std::string(what) + " failed (" + std::to_string(rc) + ")";
    if (ctx) msg += ": " + std::string(cf_last_error(ctx));
    throw std::runtime_error(msg);
}

struct BoundaryType {
    enum Values { SOLID = CF_BC_SOLID, FREE = CF_BC_FREE };
};

template <std::size_t NumSpaceDim>
struct BoundaryCondition;

template <>
struct BoundaryCondition<2> {
    std::array<int, 4> boundary_type{{BoundaryType::SOLID, BoundaryType::SOLID, BoundaryType::SOLID,
                                      BoundaryType::SOLID}};
    std::array<int, 2> min{{0, 0}};
    std::array<int, 2> max{{0, 0}};
};

template <std::size_t NumSpaceDim>
struct InflowSource;

template <>
struct InflowSource<2> {
    InflowSource(std::array<double, 2> location, std::array<double, 2> size, std::array<double, 2> velocity,
                 double quantity)
        : _location(location), _size(size), _quantity(quantity) {
        _bounding_box = {location[0], location[1], location[0] + size[0], location[1] + size[1]};
        _velocity = velocity;
    }
    std::array<double, 2> _location, _size;
    std::array<double, 4> _bounding_box;
    double _quantity;
    std::array<double, 2> _velocity;
    int _mode = 0;  // 0: clamp (reference), 1: rate (extension)
};

template <std::size_t NumSpaceDim>
struct BodyForce;

template <>
struct BodyForce<2> {
    BodyForce(double fx, double fy) : _force{{fx, fy}} {}
    std::array<double, 2> _force;
    bool _density_scaled = false;  // extension
};

namespace Version {
struct Current {};
struct Next {};
}  // namespace Version
namespace Field {
struct Quantity {};
struct Velocity {};
}  // namespace Field

// Uniform mesh with ghost depth halo_cell_width (src/Mesh.hpp:41-103).
template <int Dim>
class Mesh;

template <>
class Mesh<2> {
  public:
    Mesh(const std::array<double, 4>& global_bounding_box, const std::array<int, 2>& global_num_cell,
         int halo_cell_width, std::array<bool, 2> periodic = {{false, false}})
        : _box(global_bounding_box), _n(global_num_cell), _halo(halo_cell_width), _periodic(periodic) {
        if (halo_cell_width != 3) throw std::logic_error("the GB300 path uses ghost depth 3 (src/Solver.hpp:78)");
        _dx = (_box[2] - _box[0]) / _n[0];
        for (int d = 0; d < 2; ++d) {
            double extent = _n[d] * _dx;
            if (std::abs(extent - (_box[d + 2] - _box[d])) > 10.0 * 2.220446049250313e-16)
                throw std::logic_error("Extent not evenly divisible by uniform cell size");
        }
    }
    double cellSize() const { return _dx; }
    std::array<int, 2> minDomainGlobalCellIndex() const { return {{0, 0}}; }
    std::array<int, 2> maxDomainGlobalCellIndex() const { return {{_n[0] - 1, _n[1] - 1}}; }
    int rank() const { return 0; }
    int haloCellWidth() const { return _halo; }
    const std::array<int, 2>& numCell() const { return _n; }
    const std::array<double, 4>& boundingBox() const { return _box; }
    const std::array<bool, 2>& periodic() const { return _periodic; }

  private:
    std::array<double, 4> _box;
    std::array<int, 2> _n;
    int _halo;
    std::array<bool, 2> _periodic;
    double _dx;
};

// Owned-region host copy of one field, indexed (i, j) like a Kokkos view.
struct HostField {
    int nx = 0, ny = 0;
    std::vector<double> data;
    double& operator()(int i, int j) { return data[(size_t)j * nx + i]; }
    double operator()(int i, int j) const { return data[(size_t)j * nx + i]; }
};

// State storage on the GPU (src/ProblemManager.hpp:93-419).  Current/Next
// live on the device; advance() happens inside the advection call.
template <std::size_t NumSpaceDim>
class ProblemManager;

template <>
class ProblemManager<2> {
  public:
    template <class InitFunc>
    ProblemManager(const std::shared_ptr<Mesh<2>>& mesh, const InitFunc& create_functor, bool mixed = false,
                   int device = 0)
        : _mesh(mesh) {
        cf_grid_desc d{};
        d.nx = mesh->numCell()[0];
        d.ny = mesh->numCell()[1];
        d.lo[0] = mesh->boundingBox()[0];
        d.lo[1] = mesh->boundingBox()[1];
        d.hi[0] = mesh->boundingBox()[2];
        d.hi[1] = mesh->boundingBox()[3];
        d.periodic[0] = mesh->periodic()[0];
        d.periodic[1] = mesh->periodic()[1];
        d.precision = mixed ? CF_PREC_MIXED : CF_PREC_FP64;
        d.device = device;
        check(nullptr, cf_ctx_create(&d, &_ctx), "cf_ctx_create");
        initialize(create_functor);
    }
    ~ProblemManager() {
        if (_ctx) cf_ctx_destroy(_ctx);
    }
    ProblemManager(const ProblemManager&) = delete;
    ProblemManager& operator=(const ProblemManager&) = delete;

    // src/ProblemManager.hpp:186-263: the functor sees local indices and the
    // coordinate loc0 + dx * local index of each owned entity.
    template <class InitFunctor>
    void initialize(const InitFunctor& f) {
        const int h = 3;
        const double dx = _mesh->cellSize();
        const double lo[2] = {_mesh->boundingBox()[0] - h * dx, _mesh->boundingBox()[1] - h * dx};
        auto fill = [&](int field, double ox, double oy, auto tag, auto fieldtag) {
            int ex, ey;
            check(_ctx, cf_owned_extent(_ctx, field, &ex, &ey), "cf_owned_extent");
            std::vector<double> a((size_t)ex * ey);
            for (int j = 0; j < ey; ++j)
                for (int i = 0; i < ex; ++i) {
                    int idx[2] = {i + h, j + h};
                    double x[2] = {lo[0] + ox * dx + dx * idx[0], lo[1] + oy * dx + dx * idx[1]};
                    double v = 0.0;
                    f(tag, fieldtag, idx, x, v);
                    a[(size_t)j * ex + i] = v;
                }
            check(_ctx, cf_upload(_ctx, field, a.data(), 1, ex), "cf_upload");
        };
        fill(CF_FIELD_QUANTITY, 0.5, 0.5, Cajita::Cell(), Field::Quantity());
        fill(CF_FIELD_U, 0.0, 0.5, Cajita::Face<Cajita::Dim::I>(), Field::Velocity());
        fill(CF_FIELD_V, 0.5, 0.0, Cajita::Face<Cajita::Dim::J>(), Field::Velocity());
    }

    const std::shared_ptr<Mesh<2>>& mesh() const { return _mesh; }

    HostField get(Cajita::Cell, Field::Quantity, Version::Current) const { return download(CF_FIELD_QUANTITY); }
    HostField get(Cajita::Face<Cajita::Dim::I>, Field::Velocity, Version::Current) const {
        return download(CF_FIELD_U);
    }
    HostField get(Cajita::Face<Cajita::Dim::J>, Field::Velocity, Version::Current) const {
        return download(CF_FIELD_V);
    }
    void set(Cajita::Cell, Field::Quantity, const HostField& f) { upload(CF_FIELD_QUANTITY, f); }
    void set(Cajita::Face<Cajita::Dim::I>, Field::Velocity, const HostField& f) { upload(CF_FIELD_U, f); }
    void set(Cajita::Face<Cajita::Dim::J>, Field::Velocity, const HostField& f) { upload(CF_FIELD_V, f); }
    HostField pressure() const { return download(CF_FIELD_PRESSURE); }

    // ProblemManager::gather(Current): on-device ghost fill
    void gather(Version::Current) const { check(_ctx, cf_fill_ghosts(_ctx), "cf_fill_ghosts"); }
    // ProblemManager::advance: the swap is part of the advection call
    template <class E, class F>
    void advance(E, F) {}

    cf_ctx* ctx() const { return _ctx; }

  private:
    HostField download(int field) const {
        HostField h;
        check(_ctx, cf_owned_extent(_ctx, field, &h.nx, &h.ny), "cf_owned_extent");
        h.data.resize((size_t)h.nx * h.ny);
        check(_ctx, cf_download(_ctx, field, h.data.data(), 1, h.nx), "cf_download");
        return h;
    }
    void upload(int field, const HostField& f) {
        check(_ctx, cf_upload(_ctx, field, f.data.data(), 1, f.nx), "cf_upload");
    }
    std::shared_ptr<Mesh<2>> _mesh;
    cf_ctx* _ctx = nullptr;
};

namespace TimeIntegrator {
// src/TimeIntegrator.hpp:120-177 (gather, advect q/u/v, advance); the final
// sample is cubic as in the reference unless value_order = 1.
template <std::size_t NumSpaceDims>
void step(ProblemManager<2>& pm, const double delta_t, const BoundaryCondition<2>& /*bc*/, int value_order = 3) {
    check(pm.ctx(), cf_advect(pm.ctx(), delta_t, value_order), "cf_advect");
}
}  // namespace TimeIntegrator

class VelocityCorrectorBase {
  public:
    virtual ~VelocityCorrectorBase() = default;
    virtual void correctVelocity() = 0;
};

// VelocityCorrector on the GPU (src/VelocityCorrector.hpp:51-295).  The
// reference hard-codes tol 1e-6 and max_iter 2000 (:103-104); both are
// parameters here, with those defaults.
class VelocityCorrector : public VelocityCorrectorBase {
  public:
    VelocityCorrector(const std::shared_ptr<ProblemManager<2>>& pm, const BoundaryCondition<2>& bc, double density,
                      double delta_t, std::string solver, std::string precon, double tol = 1.0e-6,
                      int max_iter = 2000)
        : _pm(pm), _dt(delta_t), _solver(std::move(solver)), _precon(std::move(precon)) {
        cf_ctx* c = pm->ctx();
        check(c, cf_set_bc(c, bc.boundary_type.data()), "cf_set_bc");
        check(c, cf_set_density(c, density), "cf_set_density");
        _opts.solver = _solver.c_str();
        _opts.precon = _precon.c_str();
        _opts.tol = tol;
        _opts.abs_tol = 0.0;
        _opts.max_iter = max_iter;
        _opts.inner_tol = 0.0;
        _opts.max_outer = 0;
        // reject unsupported solver names at construction, as the reference's
        // factory does when HYPRE does not know them
        if (_solver != "Reference" && _solver != "PCG")
            throw std::runtime_error("pressure solver '" + _solver + "' is not implemented");
        if (_solver == "PCG" && _precon != "Diagonal" && _precon != "Jacobi" && _precon != "None" &&
            _precon != "none" && _precon != "PFMG" && _precon != "SMG" && _precon != "MG")
            throw std::runtime_error("preconditioner '" + _precon + "' is not implemented");
    }
    void correctVelocity() override {
        int rc = cf_project(_pm->ctx(), _dt, &_opts, &_last);
        if (rc != CF_OK && rc != CF_ERR_NOT_CONVERGED) check(_pm->ctx(), rc, "cf_project");
    }
    cf_solver_opts& options() { return _opts; }
    const cf_solve_stats& lastStats() const { return _last; }

  private:
    std::shared_ptr<ProblemManager<2>> _pm;
    double _dt;
    std::string _solver, _precon;
    cf_solver_opts _opts{};
    cf_solve_stats _last{};
};

template <std::size_t NumSpaceDims>
std::shared_ptr<VelocityCorrectorBase> createVelocityCorrector(const std::shared_ptr<ProblemManager<2>>& pm,
                                                               BoundaryCondition<2>& bc, const double density,
                                                               const double delta_t, std::string solver,
                                                               std::string precon) {
    return std::make_shared<VelocityCorrector>(pm, bc, density, delta_t, std::move(solver), std::move(precon));
}

// src/SiloWriter.hpp: the per-step output.  libsilo is not part of this
// build, so siloWrite writes the same mesh and variables that writeFile hands
// to Silo (:61-214: DBPutQuadmesh node coordinates, DBPutQuadvar1 "quantity"
// and DBPutQuadvar "velocity" (u, v) interpolated to cell centres, zone-
// centred, owned cells, x fastest) into one raw little-endian file per call:
//   "CFSILO01" | int32 nx, ny, cycle | float64 time, dt |
//   float64 X[nx+1] | Y[ny+1] | quantity[nx*ny] | u[nx*ny] | v[nx*ny]
// named <dir>/CajitaFluids%05d.cfraw (the reference's master-file name,
// :386-387, with the raw extension).
template <std::size_t NumSpaceDims>
class SiloWriter;

template <>
class SiloWriter<2> {
  public:
    SiloWriter(const std::shared_ptr<ProblemManager<2>>& pm, std::string dir = "data")
        : _pm(pm), _dir(std::move(dir)) {}

    void siloWrite(const char* /*name*/, int time_step, double time, double dt) {
        cf_ctx* c = _pm->ctx();
        const auto& mesh = *_pm->mesh();
        const int nx = mesh.numCell()[0], ny = mesh.numCell()[1];
        const double h = mesh.cellSize();
        std::vector<double> q((size_t)nx * ny), u(q.size()), v(q.size()), X(nx + 1), Y(ny + 1);
        for (int i = 0; i <= nx; ++i) X[i] = mesh.boundingBox()[0] + i * h;
        for (int j = 0; j <= ny; ++j) Y[j] = mesh.boundingBox()[1] + j * h;
        check(c, cf_download(c, CF_FIELD_QUANTITY, q.data(), 1, nx), "cf_download");
        check(c, cf_cell_velocity(c, u.data(), v.data(), 1, nx), "cf_cell_velocity");
        char path[4096];
        snprintf(path, sizeof(path), "%s/CajitaFluids%05d.cfraw", _dir.c_str(), time_step);
        FILE* f = fopen(path, "wb");
        if (!f) throw std::runtime_error(std::string("cannot open ") + path);
        const int32_t hdr[3] = {nx, ny, time_step};
        const double tv[2] = {time, dt};
        bool ok = fwrite("CFSILO01", 1, 8, f) == 8 && fwrite(hdr, sizeof(int32_t), 3, f) == 3 &&
                  fwrite(tv, sizeof(double), 2, f) == 2 && fwrite(X.data(), sizeof(double), X.size(), f) == X.size() &&
                  fwrite(Y.data(), sizeof(double), Y.size(), f) == Y.size();
        for (const auto* a : {&q, &u, &v}) ok = ok && fwrite(a->data(), sizeof(double), a->size(), f) == a->size();
        if (fclose(f) != 0 || !ok) throw std::runtime_error(std::string("write failed: ") + path);
    }

  private:
    std::shared_ptr<ProblemManager<2>> _pm;
    std::string _dir;
};

class SolverBase {
  public:
    virtual ~SolverBase() = default;
    virtual void setup(void) = 0;
    virtual void step(void) = 0;
    virtual void solve(const double t_final, const int write_freq) = 0;
};

// src/Solver.hpp:96-106: dt is limited to one cell per step at the inflow
// speed plus sqrt(|f| dx); the limited step is fixed for the run, because the
// pressure matrix is built with it.
inline double limitTimeStep(double delta_t, double cell_size, const InflowSource<2>& source,
                            const BodyForce<2>& body) {
    double forcemax = std::sqrt(body._force[0] * body._force[0] + body._force[1] * body._force[1]);
    double umax = std::fmax(std::fabs(source._velocity[0]), std::fabs(source._velocity[1])) +
                  std::sqrt(forcemax * cell_size);
    if ((umax > 0) && (delta_t > cell_size / umax)) return cell_size / umax;
    return delta_t;
}

// src/Solver.hpp:55-279.
template <std::size_t NumSpaceDim>
class Solver;

template <>
class Solver<2> : public SolverBase {
  public:
    template <class InitFunc>
    Solver(const std::array<double, 4>& global_bounding_box, const std::array<int, 2>& global_num_cell,
           const double density, const InitFunc& create_functor, const BoundaryCondition<2>& bc,
           const InflowSource<2>& source, const BodyForce<2>& body, const double delta_t,
           const std::string& matrix_solver, const std::string& preconditioner, bool mixed = false,
           std::array<bool, 2> periodic = {{false, false}}, int value_order = 3)
        : _density(density), _bc(bc), _source(source), _body(body), _dt(delta_t), _time(0.0), _order(value_order) {
        _mesh = std::make_shared<Mesh<2>>(global_bounding_box, global_num_cell, 3, periodic);
        _dt = limitTimeStep(delta_t, _mesh->cellSize(), source, body);
        if (_dt != delta_t)
            std::cerr << "Reducting timestep to " << _dt << " given mesh size and inflow velocity.\n";
        _bc.min = _mesh->minDomainGlobalCellIndex();
        _bc.max = _mesh->maxDomainGlobalCellIndex();
        _pm = std::make_shared<ProblemManager<2>>(_mesh, create_functor, mixed);
        cf_ctx* c = _pm->ctx();
        check(c, cf_set_source(c, source._location.data(), source._size.data(), source._velocity.data(),
                               source._quantity, source._mode),
              "cf_set_source");
        check(c, cf_set_body_force(c, body._force.data(), body._density_scaled ? 1 : 0), "cf_set_body_force");
        _vc = std::make_shared<VelocityCorrector>(_pm, _bc, _density, _dt, matrix_solver, preconditioner);
    }

    void setup() override {
        check(_pm->ctx(), cf_add_inputs(_pm->ctx(), _dt), "cf_add_inputs");
        _vc->correctVelocity();
    }
    // advect (with the input stage fused into the advection kernel), then project
    void step() override {
        int rc = cf_step(_pm->ctx(), _dt, _order, &_vc->options(), &_last);
        if (rc != CF_OK && rc != CF_ERR_NOT_CONVERGED) check(_pm->ctx(), rc, "cf_step");
        _time += _dt;
    }
    // src/Solver.hpp:149-177, writing through SiloWriter when an output
    // directory is set (setOutputDirectory).  The same steps, prints and
    // writes as the reference's do-while loop; the steps between two output
    // points go to the device in one cf_steps call (no host synchronisation
    // between them).
    void solve(const double t_final, const int write_freq) override {
        int num_step = (int)(t_final / _dt);
        if (_silo) _silo->siloWrite("Mesh", 0, _time, _dt);
        setup();
        // the loop's step count: time accumulates one dt at a time until t_final
        int total = 0;
        for (double tm = _time; total == 0 || tm < t_final; ++total) tm += _dt;
        int t = 0;
        while (t < total) {
            if (0 == t % write_freq) {
                printf("Step %d / %d at time = %f\n", t, num_step, _time);
                steps(1);
                if (_silo) _silo->siloWrite("Mesh", t, _time, _dt);
                t += 1;
            } else {
                const int next = std::min(total, (t / write_freq + 1) * write_freq);
                steps(next - t);
                t = next;
            }
        }
    }
    // n steps in one device-side loop (cf_steps)
    void steps(int n) {
        int bad = 0;
        int rc = cf_steps(_pm->ctx(), n, _dt, _order, &_vc->options(), &_last, &bad);
        if (rc != CF_OK && rc != CF_ERR_NOT_CONVERGED) check(_pm->ctx(), rc, "cf_steps");
        for (int k = 0; k < n; ++k) _time += _dt;
    }
    void setOutputDirectory(const std::string& dir) { _silo = std::make_shared<SiloWriter<2>>(_pm, dir); }
    const std::shared_ptr<SiloWriter<2>>& siloWriter() const { return _silo; }

    // the reference hard-codes tol 1e-6 / max_iter 2000 (src/VelocityCorrector.hpp:103-104)
    void setTolerance(double tol, int max_iter) {
        _vc->options().tol = tol;
        _vc->options().max_iter = max_iter;
    }
    const std::shared_ptr<ProblemManager<2>>& problemManager() const { return _pm; }
    const cf_solve_stats& lastStats() const { return _last; }
    double timeStep() const { return _dt; }
    double time() const { return _time; }

  private:
    double _density;
    BoundaryCondition<2> _bc;
    InflowSource<2> _source;
    BodyForce<2> _body;
    double _dt, _time;
    int _order;
    std::shared_ptr<Mesh<2>> _mesh;
    std::shared_ptr<ProblemManager<2>> _pm;
    std::shared_ptr<VelocityCorrector> _vc;
    std::shared_ptr<SiloWriter<2>> _silo;
    cf_solve_stats _last{};
};

// src/Solver.hpp:283-350; "gb300" (or "cuda") selects this GPU path.
template <class InitFunc>
std::shared_ptr<SolverBase> createSolver(const std::string& device, const std::array<double, 4>& global_bounding_box,
                                         const std::array<int, 2>& global_num_cell, const double density,
                                         const InitFunc& create_functor, const BoundaryCondition<2>& bc,
                                         const InflowSource<2>& source, const BodyForce<2>& body,
                                         const double delta_t, const std::string& matrix_solver,
                                         const std::string& preconditioner) {
    if (device == "gb300" || device == "cuda")
        return std::make_shared<Solver<2>>(global_bounding_box, global_num_cell, density, create_functor, bc, source,
                                           body, delta_t, matrix_solver, preconditioner);
    if (device == "serial" || device == "openmp" || device == "hip")
        throw std::runtime_error("backend '" + device + "' is not part of this build");
    throw std::runtime_error("invalid backend");
}

}  // namespace CajitaFluids
