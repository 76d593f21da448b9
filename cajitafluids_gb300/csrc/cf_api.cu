// C ABI of libcfgpu (declared in include/cajitafluids_gb300.h).
//
// Context creation restates the Solver / Mesh / ProblemManager constructors
// (src/Solver.hpp:69-123, src/Mesh.hpp:41-103, src/ProblemManager.hpp:127-180):
// uniform square cells, ghost depth 3, zero-initialised ghosts, and the
// curr/next double buffering that ProblemManager::advance swaps.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include <cstring>
#include <new>
#include <vector>

#include "../../include/cajitafluids_gb300.h"
#include "cf_ctx.cuh"

namespace cf {

int fail(cf_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_check(cf_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return CF_OK;
    return fail(c, CF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Matrix tables: initializeMatrixValues + build_matrix
// (src/VelocityCorrector.hpp:116-144, src/BoundaryConditions.hpp:57-97) and
// the Jacobi preconditioner 1 / A_00 (:174-179).
void build_stencil(const cf_ctx* c, double dt, int precon_none, Stencil* st) {
    const Phys& p = c->ph;
    double scale = dt / ((c->density * p.dx) * p.dx);
    for (int b = 0; b < 16; ++b) {
        double d = 4.0 * scale;
        if ((b & 1) && p.bc[0] == CF_BC_SOLID) d = d - scale;
        if ((b & 2) && p.bc[2] == CF_BC_SOLID) d = d - scale;
        if ((b & 4) && p.bc[1] == CF_BC_SOLID) d = d - scale;
        if ((b & 8) && p.bc[3] == CF_BC_SOLID) d = d - scale;
        st->diag[b] = d;
        st->minv[b] = precon_none ? 1.0 : 1.0 / d;
        st->diag32[b] = (float)d;
        st->minv32[b] = precon_none ? 1.0f : (float)(1.0 / d);
    }
    st->ms = -1.0 * scale;
    st->ms32 = (float)st->ms;
}

}  // namespace cf

using namespace cf;

namespace {

size_t round_up(size_t v, size_t m) { return (v + m - 1) / m * m; }

template <typename T>
int alloc_grid(cf_ctx* c, Grid<T>& g, int ex, int ey) {
    const int col0 = CF_COL0;  // local column 3 lands on a 32-element boundary
    int pitch = (int)round_up((size_t)col0 + ex, 32);
    void* base = nullptr;
    size_t bytes = (size_t)pitch * ey * sizeof(T);
    cudaError_t e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) return fail(c, CF_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    c->allocs.push_back(base);
    cudaMemsetAsync(base, 0, bytes, c->stream);
    g.o = reinterpret_cast<T*>(base) + col0;
    g.pitch = pitch;
    g.ex = ex;
    g.ey = ey;
    return CF_OK;
}

// Host-side failure injection for tests: when positive, the n-th device
// allocation from now on fails as if cudaMalloc had run out of memory.
static int g_fail_alloc_in = 0;

template <typename T>
int alloc_dev(cf_ctx* c, T*& ptr, size_t n) {
    if (g_fail_alloc_in > 0 && --g_fail_alloc_in == 0)
        return fail(c, CF_ERR_NOMEM, "cudaMalloc of %zu bytes failed: injected failure", n * sizeof(T));
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, n * sizeof(T) + 256);
    if (e != cudaSuccess) return fail(c, CF_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
    c->allocs.push_back(base);
    cudaMemsetAsync(base, 0, n * sizeof(T) + 256, c->stream);
    ptr = reinterpret_cast<T*>(base);
    return CF_OK;
}

int owned(const cf_ctx* c, int field, int* ex, int* ey) {
    const Phys& p = c->ph;
    switch (field) {
        case CF_FIELD_QUANTITY:
        case CF_FIELD_PRESSURE:
            *ex = p.nx;
            *ey = p.ny;
            return CF_OK;
        case CF_FIELD_U:
            *ex = p.per_x ? p.nx : p.nx + 1;
            *ey = p.ny;
            return CF_OK;
        case CF_FIELD_V:
            *ex = p.nx;
            *ey = p.per_y ? p.ny : p.ny + 1;
            return CF_OK;
    }
    return CF_ERR_INVALID;
}

int sync(cf_ctx* c, const char* what) { return cuda_check(c, cudaStreamSynchronize(c->stream), what); }

int parse_opts(cf_ctx* c, const cf_solver_opts* o, SolveOpts* so) {
    const char* solver = (o && o->solver) ? o->solver : "PCG";
    const char* precon = (o && o->precon) ? o->precon : "Diagonal";
    if (strcmp(solver, "Reference") != 0 && strcmp(solver, "PCG") != 0)
        return fail(c, CF_ERR_UNSUPPORTED, "pressure solver '%s' is not implemented (use Reference or PCG)", solver);
    so->precon_none = 0;
    so->precon_mg = 0;
    if (strcmp(solver, "PCG") == 0) {
        if (!strcmp(precon, "None") || !strcmp(precon, "none"))
            so->precon_none = 1;
        else if (!strcmp(precon, "PFMG") || !strcmp(precon, "SMG") || !strcmp(precon, "MG"))
            so->precon_mg = 1;
        else if (strcmp(precon, "Diagonal") != 0 && strcmp(precon, "Jacobi") != 0)
            return fail(c, CF_ERR_UNSUPPORTED,
                        "preconditioner '%s' is not implemented (use Diagonal, Jacobi, PFMG, SMG, MG or None)", precon);
    }
    so->tol = o ? o->tol : 1.0e-6;
    so->abs_tol = o ? o->abs_tol : 0.0;
    so->max_iter = o ? o->max_iter : 2000;
    so->inner_tol = (o && o->inner_tol > 0.0) ? o->inner_tol : 0.1;
    so->max_outer = (o && o->max_outer > 0) ? o->max_outer : 200;
    if (!(so->tol >= 0.0) || !(so->abs_tol >= 0.0) || so->max_iter < 0 || !(so->inner_tol < 1.0))
        return fail(c, CF_ERR_INVALID, "invalid solver options");
    return CF_OK;
}

int status_code(int st) {
    switch (st) {
        case ST_CONVERGED: return CF_OK;
        case ST_MAXIT: return CF_ERR_NOT_CONVERGED;
        case ST_TIMEOUT: return CF_ERR_TIMEOUT;
        default: return CF_ERR_NUMERIC;
    }
}

void fill_stats(const SolveResult& r, cf_solve_stats* s) {
    if (!s) return;
    s->iterations = r.iterations;
    s->outer_iterations = r.outer;
    s->status = r.status;
    s->b_norm = sqrt(r.bb);
    s->r_norm = sqrt(r.rr);
    s->div_l2 = r.div_l2;
    s->div_linf = r.div_linf;
}

int do_project(cf_ctx* c, double dt, const cf_solver_opts* opts, cf_solve_stats* stats) {
    SolveOpts so{};
    int rc = parse_opts(c, opts, &so);
    if (rc) return rc;
    if (!(dt > 0.0) || !isfinite(dt)) return fail(c, CF_ERR_INVALID, "dt must be positive and finite");
    SolveResult r{};
    rc = project(c, dt, so, &r);
    if (rc) return rc;
    fill_stats(r, stats);
    rc = status_code(r.status);
    if (rc == CF_ERR_NOT_CONVERGED)
        fail(c, rc, "pressure solve stopped at max_iter (%d iterations, |r|/|b| = %g)", r.iterations,
             r.bb > 0 ? sqrt(r.rr / r.bb) : 0.0);
    else if (rc)
        fail(c, rc, "pressure solve failed (%s) after %d iterations",
             r.status == ST_NAN ? "NaN" : (r.status == ST_TIMEOUT ? "device wait timed out" : "breakdown"),
             r.iterations);
    return rc;
}

int record_advect(cf_ctx* c) {
    int rc = cuda_check(c, cudaEventSynchronize(c->ev[3]), "advect timing");
    float ms = 0.f;
    if (!rc && cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]) == cudaSuccess) {
        c->pd.advect_ms += ms;
        c->pd.advect_calls += 1;
    }
    return rc;
}

#define CF_GUARD_BEGIN try {
#define CF_GUARD_END                                                   \
    }                                                                  \
    catch (const std::bad_alloc&) {                                    \
        return fail(ctx, CF_ERR_NOMEM, "host allocation failed");     \
    }                                                                  \
    catch (...) {                                                      \
        return fail(ctx, CF_ERR_INVALID, "unexpected host exception"); \
    }

}  // namespace

namespace cf {
// One Solver::step (src/Solver.hpp:135-147) enqueued on the context's stream:
// ghost fills, advection (inputs fused unless the force is density-scaled),
// then the projection, deferred when the resident graph serves it (the
// caller synchronises and collects; a resident projection adds to the
// device tally when it does not converge).  params_ready: the projection's
// parameters were written by an earlier enqueued step with the same options.
int enqueue_step(cf_ctx* ctx, double dt, int value_order, const SolveOpts& so, SolveResult* r, bool* deferred,
                 bool params_ready) {
    const bool fuse = !ctx->ph.force_density;
    if (!ctx->prof && !ctx->direct && resident_projection()) {
        // the whole step as one graph (ghost fill, advection, inputs, projection)
        *deferred = true;
        return step_resident(ctx, dt, value_order, fuse ? 1 : 0, so, params_ready);
    }
    int rc = cuda_check(ctx, launch_fill_ghosts(ctx), "fill ghosts");
    if (ctx->prof) cudaEventRecord(ctx->ev[2], ctx->stream);
    if (!rc) rc = cuda_check(ctx, launch_advect(ctx, dt, value_order, fuse ? 1 : 0), "advect");
    if (ctx->prof) {
        cudaEventRecord(ctx->ev[3], ctx->stream);
        rc = rc ? rc : record_advect(ctx);
    }
    if (!rc && !fuse) rc = cuda_check(ctx, launch_add_inputs(ctx, dt), "add inputs");
    if (!rc) rc = project_async(ctx, dt, so, r, deferred, params_ready);
    return rc;
}

int parse_solver_opts(cf_ctx* ctx, const cf_solver_opts* opts, SolveOpts* so) { return parse_opts(ctx, opts, so); }

int alloc_grid64(cf_ctx* c, Grid<double>& g, int ex, int ey) { return alloc_grid(c, g, ex, ey); }
}  // namespace cf

extern "C" {

int cf_abi_version(void) { return CF_ABI_VERSION; }

int cf_ctx_create(const cf_grid_desc* d, cf_ctx** out) {
    if (!d || !out) return CF_ERR_INVALID;
    *out = nullptr;
    if (d->nx <= 0 || d->ny <= 0 || d->nx > (1 << 16) || d->ny > (1 << 16)) return CF_ERR_INVALID;
    if (d->precision != CF_PREC_FP64 && d->precision != CF_PREC_MIXED) return CF_ERR_INVALID;
    if (!(d->hi[0] > d->lo[0]) || !(d->hi[1] > d->lo[1])) return CF_ERR_INVALID;
    // src/Mesh.hpp:49-64: uniform cell size from x, every extent divisible by it
    double dx = (d->hi[0] - d->lo[0]) / d->nx;
    for (int k = 0; k < 2; ++k) {
        int n = k == 0 ? d->nx : d->ny;
        double extent = n * dx;
        if (fabs(extent - (d->hi[k] - d->lo[k])) > 10.0 * DBL_EPSILON) return CF_ERR_MESH;
    }
    cf_ctx* ctx = nullptr;
    try {
        ctx = new cf_ctx();
    } catch (...) {
        return CF_ERR_NOMEM;
    }
    cf_ctx* c = ctx;
    c->device = d->device;
    // CF_GRAPHS=0 in the environment: contexts start with every kernel of the
    // solve launched on its own (as cf_set_graphs(ctx, 0)), for profilers
    // that list kernel launches one by one
    if (const char* e = getenv("CF_GRAPHS")) c->direct = atoi(e) == 0 ? 1 : 0;
    int rc = cuda_check(c, cudaSetDevice(d->device), "cudaSetDevice");
    if (!rc) rc = cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream create");
    if (rc) {
        delete c;
        return rc;
    }
    Phys& p = c->ph;
    p.nx = d->nx;
    p.ny = d->ny;
    p.per_x = d->periodic[0] ? 1 : 0;
    p.per_y = d->periodic[1] ? 1 : 0;
    p.dx = dx;
    p.rdx = 1.0 / dx;
    static const double off[3][2] = {{0.5, 0.5}, {0.0, 0.5}, {0.5, 0.0}};
    for (int k = 0; k < 2; ++k) p.gl[k] = d->lo[k] - 3.0 * dx;
    for (int e = 0; e < 3; ++e)
        for (int k = 0; k < 2; ++k) {
            double t = 0.0 + off[e][k];
            p.low[e][k] = p.gl[k] + t * dx;
        }
    for (int k = 0; k < 4; ++k) p.bc[k] = CF_BC_SOLID;
    c->precision = d->precision;
    c->density = 1.0;

    int nx = p.nx, ny = p.ny;
    for (int s = 0; s < 2 && !rc; ++s) {
        if (c->precision == CF_PREC_FP64)
            rc = alloc_grid(c, c->q64[s], nx + 2 * CF_HALO, ny + 2 * CF_HALO);
        else
            rc = alloc_grid(c, c->q32[s], nx + 2 * CF_HALO, ny + 2 * CF_HALO);
        if (!rc) rc = alloc_grid(c, c->u[s], nx + 2 * CF_HALO + 1, ny + 2 * CF_HALO);
        if (!rc) rc = alloc_grid(c, c->v[s], nx + 2 * CF_HALO, ny + 2 * CF_HALO + 1);
    }
    c->vpitch = (int)round_up(nx, 32);
    size_t vn = (size_t)c->vpitch * ny;
    if (!rc) rc = alloc_dev(c, c->x.a, vn);
    if (c->precision == CF_PREC_FP64) {
        if (!rc) rc = alloc_dev(c, c->r.a, vn);
        if (!rc) rc = alloc_dev(c, c->pa.a, vn);
        if (!rc) rc = alloc_dev(c, c->pb.a, vn);
        if (!rc) rc = alloc_dev(c, c->qv.a, vn);
    } else {
        if (!rc) rc = alloc_dev(c, c->b.a, vn);
        if (!rc) rc = alloc_dev(c, c->xb.a, vn);
        // the old faces on the reduction units' west columns and south rows
        // (pairs), saved by the divergence for the gradient's fused norms
        if (!rc)
            rc = alloc_dev(c, c->bnd,
                           (size_t)((nx + CF_UNIT_COLS - 1) / CF_UNIT_COLS) * ny +
                               (size_t)((ny + CF_BAND_ROWS - 1) / CF_BAND_ROWS) * nx);
        // FP32 vectors with a one-cell ghost ring, owned column 0 on 16 bytes
        c->p32 = (int)round_up((size_t)nx + 8, 32);
        size_t n32 = (size_t)c->p32 * (ny + 2);
        float** bases[3] = {&c->r32b, &c->pa32b, &c->pb32b};
        cf::Vec32* vecs[3] = {&c->r32, &c->pa32, &c->pb32};
        for (int k = 0; k < 3 && !rc; ++k) {
            rc = alloc_dev(c, *bases[k], n32);
            vecs[k]->a = *bases[k] + c->p32 + 4;
            vecs[k]->pitch = c->p32;
        }
    }
    if (cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || c->sms < 1)
        c->sms = 1;
    c->G = (nx + CF_UNIT_COLS - 1) / CF_UNIT_COLS;
    c->B = (ny + CF_BAND_ROWS - 1) / CF_BAND_ROWS;
    c->n_units = c->G * c->B;
    if (!rc) rc = alloc_dev(c, c->partials, 4 * (size_t)c->n_units);
    if (!rc) rc = alloc_dev(c, c->S, 1);
    if (!rc) rc = alloc_dev(c, c->d_out, 4);
    c->staging_elems = (size_t)(nx + 1) * (ny + 1);
    if (!rc) rc = alloc_dev(c, c->staging, c->staging_elems);
    if (!rc) rc = cuda_check(c, cudaMallocHost(&c->hS, sizeof(SolverState)), "cudaMallocHost");
    if (!rc) rc = cuda_check(c, cudaMallocHost(&c->hP, sizeof(SolverState)), "cudaMallocHost");
    if (!rc) rc = cuda_check(c, cudaMallocHost(&c->hPa, sizeof(SolverState)), "cudaMallocHost");
    if (!rc) rc = alloc_dev(c, c->d_tally, 4);
    if (!rc) rc = cuda_check(c, cudaMallocHost(&c->h_out, 4 * sizeof(double)), "cudaMallocHost");
    if (!rc && c->precision == CF_PREC_MIXED) rc = cg32_setup(c);
    for (int k = 0; k < 8 && !rc; ++k) rc = cuda_check(c, cudaEventCreate(&c->ev[k]), "event create");
    if (!rc) rc = sync(c, "context init");
    if (rc) {
        cf_ctx_destroy(c);
        return rc;
    }
    *out = c;
    return CF_OK;
}

int cf_ctx_destroy(cf_ctx* ctx) {
    if (!ctx) return CF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (cudaEvent_t e : ctx->ev)
        if (e) cudaEventDestroy(e);
    cf_adjoint_free(ctx);
    if (ctx->g64) cudaGraphExecDestroy(ctx->g64);
    if (ctx->g32) cudaGraphExecDestroy(ctx->g32);
    if (ctx->gmg) cudaGraphExecDestroy(ctx->gmg);
    if (ctx->gmg_pre) cudaGraphExecDestroy(ctx->gmg_pre);
    for (cudaGraphExec_t g : ctx->rgx)
        if (g) cudaGraphExecDestroy(g);
    for (cudaGraphExec_t g : ctx->sgx)
        if (g) cudaGraphExecDestroy(g);
    cf::mg_free(ctx);
    for (void* p : ctx->allocs) cudaFree(p);
    if (ctx->hS) cudaFreeHost(ctx->hS);
    if (ctx->hP) cudaFreeHost(ctx->hP);
    if (ctx->hPa) cudaFreeHost(ctx->hPa);
    if (ctx->h_out) cudaFreeHost(ctx->h_out);
    if (ctx->stream2) {
        cudaStreamSynchronize(ctx->stream2);
        cudaStreamDestroy(ctx->stream2);
    }
    if (ctx->ev_adv) cudaEventDestroy(ctx->ev_adv);
    if (ctx->ev_uv) cudaEventDestroy(ctx->ev_uv);
    if (ctx->ev_q) cudaEventDestroy(ctx->ev_q);
    if (ctx->ev_press) cudaEventDestroy(ctx->ev_press);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return CF_OK;
}

const char* cf_last_error(const cf_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int cf_owned_extent(const cf_ctx* ctx, int field, int* ex, int* ey) {
    if (!ctx || !ex || !ey) return CF_ERR_INVALID;
    return owned(ctx, field, ex, ey);
}

int cf_cell_size(const cf_ctx* ctx, double* dx) {
    if (!ctx || !dx) return CF_ERR_INVALID;
    *dx = ctx->ph.dx;
    return CF_OK;
}

int cf_set_bc(cf_ctx* ctx, const int type[4]) {
    if (!ctx || !type) return CF_ERR_INVALID;
    for (int k = 0; k < 4; ++k)
        if (type[k] != CF_BC_SOLID && type[k] != CF_BC_FREE) return fail(ctx, CF_ERR_INVALID, "boundary type must be SOLID or FREE");
    for (int k = 0; k < 4; ++k) ctx->ph.bc[k] = type[k];
    return CF_OK;
}

int cf_set_source(cf_ctx* ctx, const double location[2], const double size[2], const double velocity[2],
                  double quantity, int mode) {
    if (!ctx || !location || !size || !velocity) return CF_ERR_INVALID;
    if (mode != 0 && mode != 1) return fail(ctx, CF_ERR_INVALID, "source mode must be 0 (clamp) or 1 (rate)");
    Phys& p = ctx->ph;
    p.bbox[0] = location[0];  // src/InflowSource.hpp:78-88
    p.bbox[1] = location[1];
    p.bbox[2] = location[0] + size[0];
    p.bbox[3] = location[1] + size[1];
    p.src_vel[0] = velocity[0];
    p.src_vel[1] = velocity[1];
    p.src_q = quantity;
    p.src_mode = mode;
    // index ranges of the box test x0 <= x < x1 on each entity's coordinates,
    // x = gl + (idx + offset) dx exactly as the kernels evaluate it
    static const double off[3][2] = {{0.5, 0.5}, {0.0, 0.5}, {0.5, 0.0}};
    for (int e = 0; e < 3; ++e)
        for (int a = 0; a < 2; ++a) {
            const int n = (a == 0 ? p.nx : p.ny) + 2 * CF_HALO + 1;
            int lo = 0, hi = 0;
            for (int idx = 0; idx < n; ++idx) {
                double t = (double)idx + off[e][a];
                double x = p.gl[a] + t * p.dx;
                if (x >= p.bbox[a] && x < p.bbox[a + 2]) {
                    if (hi == 0) lo = idx;
                    hi = idx + 1;
                }
            }
            p.box[e][2 * a] = lo;
            p.box[e][2 * a + 1] = hi;
        }
    return CF_OK;
}

int cf_set_body_force(cf_ctx* ctx, const double force[2], int density_scaled) {
    if (!ctx || !force) return CF_ERR_INVALID;
    ctx->ph.force[0] = force[0];
    ctx->ph.force[1] = force[1];
    ctx->ph.force_density = density_scaled ? 1 : 0;
    return CF_OK;
}

int cf_set_warm_start(cf_ctx* ctx, int on) {
    if (!ctx) return CF_ERR_INVALID;
    ctx->warm = on ? 1 : 0;
    return CF_OK;
}

int cf_set_graphs(cf_ctx* ctx, int on) {
    if (!ctx) return CF_ERR_INVALID;
    ctx->direct = on ? 0 : 1;
    return CF_OK;
}

int cf_test_stall_wait(cf_ctx* ctx, int on) {
    if (!ctx) return CF_ERR_INVALID;
    ctx->test_stall = on ? 1 : 0;
    return CF_OK;
}

int cf_test_advect_unstaged(cf_ctx* ctx, int on) {
    if (!ctx) return CF_ERR_INVALID;
    ctx->test_unstaged = on ? 1 : 0;
    return CF_OK;
}

int cf_test_apply_general(cf_ctx* ctx, int on) {
    if (!ctx) return CF_ERR_INVALID;
    ctx->test_general_apply = on ? 1 : 0;
    return CF_OK;
}

int cf_set_density(cf_ctx* ctx, double density) {
    if (!ctx) return CF_ERR_INVALID;
    if (!(density > 0.0) || !isfinite(density)) return fail(ctx, CF_ERR_INVALID, "density must be positive");
    ctx->density = density;
    return CF_OK;
}

int cf_set_quirks(cf_ctx* ctx, unsigned flags) {
    if (!ctx) return CF_ERR_INVALID;
    if (flags & ~(CF_FIX_Q1 | CF_FIX_Q3)) return fail(ctx, CF_ERR_INVALID, "unknown quirk flags");
    ctx->ph.quirks = flags;
    return CF_OK;
}

int cf_upload(cf_ctx* ctx, int field, const double* host, ptrdiff_t si, ptrdiff_t sj) {
    if (!ctx || !host) return CF_ERR_INVALID;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    int ox, oy;
    if (field == CF_FIELD_PRESSURE || owned(ctx, field, &ox, &oy))
        return fail(ctx, CF_ERR_INVALID, "field %d cannot be uploaded", field);
    if (si <= 0 || sj <= 0) return fail(ctx, CF_ERR_INVALID, "strides must be positive");
    int s = ctx->cur;
    bool q32 = field == CF_FIELD_QUANTITY && ctx->precision == CF_PREC_MIXED;
    // a mixed context's u, v are stored as double-float pairs: the FP64
    // values land in place and are split there
    const bool pairs = field != CF_FIELD_QUANTITY && ctx->precision == CF_PREC_MIXED;
    Grid<double> g = field == CF_FIELD_QUANTITY ? ctx->q64[s] : (field == CF_FIELD_U ? ctx->u[s] : ctx->v[s]);
    int rc;
    if (si == 1 && !q32) {
        rc = cuda_check(ctx, cudaMemcpy2DAsync(&g.at(CF_HALO, CF_HALO), g.pitch * sizeof(double), host, sj * sizeof(double),
                                               ox * sizeof(double), oy, cudaMemcpyDefault, ctx->stream), "upload");
        if (!rc && pairs) rc = cuda_check(ctx, launch_to_pairs(ctx, field, s), "split");
        if (rc) return rc;
        return sync(ctx, "upload");
    }
    // general layout: stage contiguous (x fastest) owned values
    if (si == 1) {
        rc = cuda_check(ctx, cudaMemcpy2DAsync(ctx->staging, ox * sizeof(double), host, sj * sizeof(double),
                                               ox * sizeof(double), oy, cudaMemcpyDefault, ctx->stream), "upload");
    } else {
        std::vector<double> tmp((size_t)ox * oy);
        for (int j = 0; j < oy; ++j)
            for (int i = 0; i < ox; ++i) tmp[(size_t)j * ox + i] = host[i * si + j * sj];
        rc = cuda_check(ctx, cudaMemcpyAsync(ctx->staging, tmp.data(), tmp.size() * sizeof(double), cudaMemcpyDefault,
                                             ctx->stream), "upload");
        if (!rc) rc = sync(ctx, "upload");
    }
    if (rc) return rc;
    if (q32) {
        rc = cuda_check(ctx, launch_convert_q(ctx, 1, s), "convert");
    } else {
        rc = cuda_check(ctx, cudaMemcpy2DAsync(&g.at(CF_HALO, CF_HALO), g.pitch * sizeof(double), ctx->staging,
                                               ox * sizeof(double), ox * sizeof(double), oy, cudaMemcpyDeviceToDevice,
                                               ctx->stream), "upload");
        if (!rc && pairs) rc = cuda_check(ctx, launch_to_pairs(ctx, field, s), "split");
    }
    if (rc) return rc;
    return sync(ctx, "upload");
    CF_GUARD_END
}

int cf_download(cf_ctx* ctx, int field, double* host, ptrdiff_t si, ptrdiff_t sj) {
    if (!ctx || !host) return CF_ERR_INVALID;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    int ox, oy;
    if (owned(ctx, field, &ox, &oy)) return fail(ctx, CF_ERR_INVALID, "unknown field %d", field);
    if (si <= 0 || sj <= 0) return fail(ctx, CF_ERR_INVALID, "strides must be positive");
    int s = ctx->cur;
    const double* src;
    size_t spitch;
    int rc = CF_OK;
    if (field == CF_FIELD_PRESSURE && ctx->p_df) {
        // the last mixed projection left its solution as double-float pairs
        rc = cuda_check(ctx, pressure_to_f64(ctx, ctx->staging), "convert");
        src = ctx->staging;
        spitch = ox;
    } else if (field == CF_FIELD_PRESSURE) {
        src = ctx->x.a;
        spitch = ctx->vpitch;
    } else if (field == CF_FIELD_QUANTITY && ctx->precision == CF_PREC_MIXED) {
        rc = cuda_check(ctx, launch_convert_q(ctx, 0, s), "convert");
        src = ctx->staging;
        spitch = ox;
    } else if (ctx->precision == CF_PREC_MIXED) {
        // u, v pairs to FP64
        rc = cuda_check(ctx, launch_from_pairs(ctx, field, s, ctx->staging), "convert");
        src = ctx->staging;
        spitch = ox;
    } else {
        Grid<double> g = field == CF_FIELD_QUANTITY ? ctx->q64[s] : (field == CF_FIELD_U ? ctx->u[s] : ctx->v[s]);
        src = &g.at(CF_HALO, CF_HALO);
        spitch = g.pitch;
    }
    if (rc) return rc;
    if (si == 1) {
        rc = cuda_check(ctx, cudaMemcpy2DAsync(host, sj * sizeof(double), src, spitch * sizeof(double), ox * sizeof(double),
                                               oy, cudaMemcpyDefault, ctx->stream), "download");
        if (rc) return rc;
        return sync(ctx, "download");
    }
    std::vector<double> tmp((size_t)ox * oy);
    rc = cuda_check(ctx, cudaMemcpy2DAsync(tmp.data(), ox * sizeof(double), src, spitch * sizeof(double),
                                           ox * sizeof(double), oy, cudaMemcpyDefault, ctx->stream), "download");
    if (!rc) rc = sync(ctx, "download");
    if (rc) return rc;
    for (int j = 0; j < oy; ++j)
        for (int i = 0; i < ox; ++i) host[i * si + j * sj] = tmp[(size_t)j * ox + i];
    return CF_OK;
    CF_GUARD_END
}

int cf_download_ghosted(cf_ctx* ctx, int field, double* host, int* ex, int* ey) {
    if (!ctx || !ex || !ey) return CF_ERR_INVALID;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    int s = ctx->cur;
    int rc;
    if (field == CF_FIELD_QUANTITY && ctx->precision == CF_PREC_MIXED) {
        const Grid<float>& g = ctx->q32[s];
        *ex = g.ex;
        *ey = g.ey;
        if (!host) return CF_OK;
        std::vector<float> tmp((size_t)g.ex * g.ey);
        rc = cuda_check(ctx, cudaMemcpy2DAsync(tmp.data(), g.ex * sizeof(float), g.o, g.pitch * sizeof(float),
                                               g.ex * sizeof(float), g.ey, cudaMemcpyDeviceToHost, ctx->stream), "download");
        if (!rc) rc = sync(ctx, "download");
        if (rc) return rc;
        for (size_t k = 0; k < tmp.size(); ++k) host[k] = tmp[k];
        return CF_OK;
    }
    if (field != CF_FIELD_QUANTITY && field != CF_FIELD_U && field != CF_FIELD_V)
        return fail(ctx, CF_ERR_INVALID, "field %d has no ghosted array", field);
    Grid<double> g = field == CF_FIELD_QUANTITY ? ctx->q64[s] : (field == CF_FIELD_U ? ctx->u[s] : ctx->v[s]);
    if (field != CF_FIELD_QUANTITY && ctx->precision == CF_PREC_MIXED && host) {
        // u, v pairs: FP64 copies of the ghosted arrays
        Grid<double> gu, gv;
        if ((rc = velocity_f64(ctx, &gu, &gv))) return rc;
        g = field == CF_FIELD_U ? gu : gv;
    }
    *ex = g.ex;
    *ey = g.ey;
    if (!host) return CF_OK;
    rc = cuda_check(ctx, cudaMemcpy2DAsync(host, g.ex * sizeof(double), g.o, g.pitch * sizeof(double),
                                           g.ex * sizeof(double), g.ey, cudaMemcpyDefault, ctx->stream), "download");
    if (rc) return rc;
    return sync(ctx, "download");
    CF_GUARD_END
}

int cf_fill_ghosts(cf_ctx* ctx) {
    if (!ctx) return CF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return cuda_check(ctx, launch_fill_ghosts(ctx), "fill ghosts");
}

int cf_advect(cf_ctx* ctx, double dt, int value_order) {
    if (!ctx) return CF_ERR_INVALID;
    if (value_order != 1 && value_order != 3) return fail(ctx, CF_ERR_INVALID, "value_order must be 1 or 3");
    if (!isfinite(dt)) return fail(ctx, CF_ERR_INVALID, "dt must be finite");
    cudaSetDevice(ctx->device);
    int rc = cuda_check(ctx, launch_fill_ghosts(ctx), "fill ghosts");
    if (ctx->prof) cudaEventRecord(ctx->ev[2], ctx->stream);
    if (!rc) rc = cuda_check(ctx, launch_advect(ctx, dt, value_order, 0), "advect");
    if (ctx->prof) {
        cudaEventRecord(ctx->ev[3], ctx->stream);
        rc = rc ? rc : record_advect(ctx);
    }
    return rc;
}

int cf_add_inputs(cf_ctx* ctx, double dt) {
    if (!ctx) return CF_ERR_INVALID;
    if (!isfinite(dt)) return fail(ctx, CF_ERR_INVALID, "dt must be finite");
    cudaSetDevice(ctx->device);
    return cuda_check(ctx, launch_add_inputs(ctx, dt), "add inputs");
}

int cf_project(cf_ctx* ctx, double dt, const cf_solver_opts* opts, cf_solve_stats* stats) {
    if (!ctx) return CF_ERR_INVALID;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    return do_project(ctx, dt, opts, stats);
    CF_GUARD_END
}

int cf_setup(cf_ctx* ctx, double dt, const cf_solver_opts* opts, cf_solve_stats* stats) {
    if (!ctx) return CF_ERR_INVALID;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    int rc = cf_add_inputs(ctx, dt);
    if (rc) return rc;
    return do_project(ctx, dt, opts, stats);
    CF_GUARD_END
}

int cf_step(cf_ctx* ctx, double dt, int value_order, const cf_solver_opts* opts, cf_solve_stats* stats) {
    if (!ctx) return CF_ERR_INVALID;
    if (value_order != 1 && value_order != 3) return fail(ctx, CF_ERR_INVALID, "value_order must be 1 or 3");
    if (!(dt > 0.0) || !isfinite(dt)) return fail(ctx, CF_ERR_INVALID, "dt must be positive and finite");
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    SolveOpts so{};
    int rc = parse_opts(ctx, opts, &so);
    if (rc) return rc;
    const bool fuse = !ctx->ph.force_density;
    rc = cuda_check(ctx, launch_fill_ghosts(ctx), "fill ghosts");
    if (ctx->prof) cudaEventRecord(ctx->ev[2], ctx->stream);
    if (!rc) rc = cuda_check(ctx, launch_advect(ctx, dt, value_order, fuse ? 1 : 0), "advect");
    if (ctx->prof) {
        cudaEventRecord(ctx->ev[3], ctx->stream);
        rc = rc ? rc : record_advect(ctx);
    }
    if (!rc && !fuse) rc = cuda_check(ctx, launch_add_inputs(ctx, dt), "add inputs");
    if (rc) return rc;
    return do_project(ctx, dt, opts, stats);
    CF_GUARD_END
}

// Solver::solve's step loop (src/Solver.hpp:149-177) on the device: nsteps
// advections and projections enqueued back to back, the projections'
// parameters written once, one synchronisation at the end.  Each projection
// adds to a device tally when it does not converge.
int cf_steps(cf_ctx* ctx, int nsteps, double dt, int value_order, const cf_solver_opts* opts,
             cf_solve_stats* stats, int* unconverged) {
    if (!ctx || nsteps < 0) return CF_ERR_INVALID;
    if (value_order != 1 && value_order != 3) return fail(ctx, CF_ERR_INVALID, "value_order must be 1 or 3");
    if (!(dt > 0.0) || !isfinite(dt)) return fail(ctx, CF_ERR_INVALID, "dt must be positive and finite");
    if (unconverged) *unconverged = 0;
    if (nsteps == 0) return CF_OK;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    SolveOpts so{};
    int rc = parse_opts(ctx, opts, &so);
    if (rc) return rc;
    if (ctx->prof || ctx->direct || !resident_projection()) {
        // host-polled projections: one step at a time
        int bad = 0, worst = CF_OK;
        for (int k = 0; k < nsteps; ++k) {
            int r = cf_step(ctx, dt, value_order, opts, stats);
            if (r == CF_ERR_NOT_CONVERGED || r == CF_ERR_NUMERIC || r == CF_ERR_TIMEOUT) {
                ++bad;
                worst = r;
            } else if (r) {
                return r;
            }
        }
        if (unconverged) *unconverged = bad;
        return worst;
    }
    rc = cuda_check(ctx, cudaMemsetAsync(ctx->d_tally, 0, 3 * sizeof(int), ctx->stream), "tally");
    SolveResult r{};
    bool deferred = false;
    for (int k = 0; k < nsteps && !rc; ++k) rc = enqueue_step(ctx, dt, value_order, so, &r, &deferred, k > 0);
    int tally[3] = {0, 0, 0};
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpyAsync(tally, ctx->d_tally, sizeof(tally), cudaMemcpyDeviceToHost, ctx->stream),
                        "tally");
    const int rc1 = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "steps");
    if (rc) return rc;
    if (rc1) return rc1;
    if (deferred) project_collect(ctx, &r, nsteps, tally[2]);
    fill_stats(r, stats);
    if (unconverged) *unconverged = tally[0];
    if (tally[0] == 0) return CF_OK;
    const int code = status_code(tally[1]);
    return fail(ctx, code, "%d of %d pressure solves did not converge (worst status %d)", tally[0], nsteps, tally[1]);
    CF_GUARD_END
}

// The second stream, the events and (mixed) the quantity's download staging
// of cf_step_host.  Each member is created into a local and stored only once
// it exists, so a failure leaves the members made so far valid and the rest
// null; the next call creates only what is missing.
static int step_host_resources(cf_ctx* ctx, bool mixed) {
    if (!ctx->stream2) {
        cudaStream_t s = nullptr;
        int rc = cuda_check(ctx, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream create");
        if (rc) return rc;
        ctx->stream2 = s;
    }
    cudaEvent_t* evs[3] = {&ctx->ev_adv, &ctx->ev_uv, &ctx->ev_q};
    for (cudaEvent_t* ev : evs) {
        if (*ev) continue;
        cudaEvent_t e = nullptr;
        int rc = cuda_check(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event create");
        if (rc) return rc;
        *ev = e;
    }
    if (mixed && !ctx->staging2) {
        double* p = nullptr;
        int rc = alloc_dev(ctx, p, (size_t)ctx->ph.nx * ctx->ph.ny);
        if (rc) return rc;
        ctx->staging2 = p;
    }
    if (mixed && !ctx->staging_uv) {
        double* p = nullptr;
        int rc = alloc_dev(ctx, p, 2 * (size_t)(ctx->ph.nx + 1) * (ctx->ph.ny + 1));
        if (rc) return rc;
        ctx->staging_uv = p;
    }
    return CF_OK;
}

int cf_test_fail_alloc(int nth) {
    g_fail_alloc_in = nth > 0 ? nth : 0;
    return CF_OK;
}

// Solver::step with host buffers in and out (owned arrays, x fastest,
// contiguous).  Every copy is asynchronous on the context streams; the
// quantity, final after the advection, is copied out on a second stream while
// the projection runs; one synchronisation at the end.
int cf_step_host(cf_ctx* ctx, double dt, int value_order, const cf_solver_opts* opts, cf_solve_stats* stats,
                 const double* q_in, const double* u_in, const double* v_in, double* q_out, double* u_out,
                 double* v_out) {
    if (!ctx || !q_in || !u_in || !v_in) return CF_ERR_INVALID;
    if (value_order != 1 && value_order != 3) return fail(ctx, CF_ERR_INVALID, "value_order must be 1 or 3");
    if (!(dt > 0.0) || !isfinite(dt)) return fail(ctx, CF_ERR_INVALID, "dt must be positive and finite");
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    SolveOpts so{};
    int rc = parse_opts(ctx, opts, &so);
    if (rc) return rc;
    const bool mixed = ctx->precision == CF_PREC_MIXED;
    const int nx = ctx->ph.nx, ny = ctx->ph.ny;
    // lazy set-up: each member is created on its own when it is missing, so a
    // call that failed part way (out of memory, say) leaves the others valid
    // and the next call creates what is still missing
    rc = step_host_resources(ctx, mixed);
    if (rc) return rc;
    // on an error after copies were queued, wait for both streams before
    // returning, so that no copy touches the caller's buffers after the call
    auto drain = [ctx](int code) {
        cudaStreamSynchronize(ctx->stream2);
        cudaStreamSynchronize(ctx->stream);
        return code;
    };
    // Uploads into the current buffers: u and v first on the main stream; the
    // quantity once they are in (they share the link), on the second stream,
    // while the velocities' own advection runs on the main one.
    const int s0 = ctx->cur;
    for (int f = CF_FIELD_U; f <= CF_FIELD_V && !rc; ++f) {
        int ox, oy;
        owned(ctx, f, &ox, &oy);
        Grid<double> g = f == CF_FIELD_U ? ctx->u[s0] : ctx->v[s0];
        rc = cuda_check(ctx, cudaMemcpy2DAsync(&g.at(CF_HALO, CF_HALO), g.pitch * sizeof(double),
                                               f == CF_FIELD_U ? u_in : v_in, ox * sizeof(double), ox * sizeof(double),
                                               oy, cudaMemcpyDefault, ctx->stream),
                        "upload");
        // mixed: the FP64 values to the pairs the context keeps, in place
        if (!rc && mixed) rc = cuda_check(ctx, launch_to_pairs(ctx, f, s0), "split");
    }
    if (!rc) rc = cuda_check(ctx, cudaEventRecord(ctx->ev_uv, ctx->stream), "event");
    if (!rc) rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->stream2, ctx->ev_uv, 0), "event wait");
    if (!rc && mixed) {
        rc = cuda_check(ctx, cudaMemcpyAsync(ctx->staging, q_in, sizeof(double) * (size_t)nx * ny, cudaMemcpyDefault,
                                             ctx->stream2), "upload");
        if (!rc) rc = cuda_check(ctx, launch_convert_q(ctx, 1, s0, ctx->stream2), "convert");
    } else if (!rc) {
        const Grid<double>& g = ctx->q64[s0];
        rc = cuda_check(ctx, cudaMemcpy2DAsync(&g.at(CF_HALO, CF_HALO), g.pitch * sizeof(double), q_in,
                                               nx * sizeof(double), nx * sizeof(double), ny, cudaMemcpyDefault,
                                               ctx->stream2),
                        "upload");
    }
    if (!rc) rc = cuda_check(ctx, launch_fill_ghosts(ctx, GHOSTS_Q, ctx->stream2), "fill ghosts");
    if (!rc) rc = cuda_check(ctx, cudaEventRecord(ctx->ev_q, ctx->stream2), "event");
    // advection and inputs (src/Solver.hpp:135-147): u and v, then q once it is in
    const bool fuse = !ctx->ph.force_density;
    if (!rc) rc = cuda_check(ctx, launch_fill_ghosts(ctx, GHOSTS_UV), "fill ghosts");
    if (!rc) rc = cuda_check(ctx, launch_advect(ctx, dt, value_order, fuse ? 1 : 0, 1, 2, true, false), "advect");
    if (!rc) rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_q, 0), "event wait");
    if (!rc) rc = cuda_check(ctx, launch_advect(ctx, dt, value_order, fuse ? 1 : 0, 0, 1, false, true), "advect");
    if (!rc && !fuse) rc = cuda_check(ctx, launch_add_inputs(ctx, dt), "add inputs");
    if (rc) return drain(rc);
    const int s1 = ctx->cur;
    // the quantity is final now: copy it out beside the projection
    if (q_out) {
        rc = cuda_check(ctx, cudaEventRecord(ctx->ev_adv, ctx->stream), "event");
        if (!rc) rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->stream2, ctx->ev_adv, 0), "event wait");
        if (!rc && mixed) {
            rc = cuda_check(ctx, launch_q_to_f64(ctx, s1, ctx->staging2, ctx->stream2), "convert");
            if (!rc)
                rc = cuda_check(ctx, cudaMemcpyAsync(q_out, ctx->staging2, sizeof(double) * (size_t)nx * ny,
                                                     cudaMemcpyDefault, ctx->stream2), "download");
        } else if (!rc) {
            const Grid<double>& g = ctx->q64[s1];
            rc = cuda_check(ctx, cudaMemcpy2DAsync(q_out, nx * sizeof(double), &g.at(CF_HALO, CF_HALO),
                                                   g.pitch * sizeof(double), nx * sizeof(double), ny,
                                                   cudaMemcpyDefault, ctx->stream2),
                            "download");
        }
        if (rc) return drain(rc);
    }
    SolveResult r{};
    bool deferred = false;
    rc = project_async(ctx, dt, so, &r, &deferred);
    // the resident projection records ev_press after the gradient subtraction:
    // u and v go out on the second stream from there, beside the rest of the
    // tail (k_div_norms, unless the gradient took the norms itself)
    cudaStream_t out_stream = ctx->stream;
    if (!rc && deferred && (u_out || v_out)) {
        rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->stream2, ctx->ev_press, 0), "event wait");
        out_stream = ctx->stream2;
    }
    double* outs[3] = {nullptr, u_out, v_out};
    for (int f = 1; f < 3 && !rc; ++f) {
        if (!outs[f]) continue;
        int ox, oy;
        owned(ctx, f, &ox, &oy);
        if (mixed) {
            // the pairs to FP64 in the staging buffer, then one copy out
            double* st = ctx->staging_uv + (f - 1) * (size_t)(ctx->ph.nx + 1) * (ctx->ph.ny + 1);
            rc = cuda_check(ctx, launch_from_pairs(ctx, f, s1, st, out_stream), "convert");
            if (!rc)
                rc = cuda_check(ctx, cudaMemcpyAsync(outs[f], st, sizeof(double) * (size_t)ox * oy, cudaMemcpyDefault,
                                                     out_stream),
                                "download");
            continue;
        }
        const Grid<double>& g = f == CF_FIELD_U ? ctx->u[s1] : ctx->v[s1];
        rc = cuda_check(ctx, cudaMemcpy2DAsync(outs[f], ox * sizeof(double), &g.at(CF_HALO, CF_HALO),
                                               g.pitch * sizeof(double), ox * sizeof(double), oy, cudaMemcpyDefault,
                                               out_stream),
                        "download");
    }
    int rc2 = cuda_check(ctx, cudaStreamSynchronize(ctx->stream2), "step_host");
    int rc1 = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "step_host");
    if (rc) return rc;
    if (rc1) return rc1;
    if (rc2) return rc2;
    if (deferred) project_collect(ctx, &r);
    fill_stats(r, stats);
    rc = status_code(r.status);
    if (rc == CF_ERR_NOT_CONVERGED)
        fail(ctx, rc, "pressure solve stopped at max_iter (%d iterations)", r.iterations);
    else if (rc)
        fail(ctx, rc, "pressure solve failed (status %d) after %d iterations", r.status, r.iterations);
    return rc;
    CF_GUARD_END
}

int cf_div_norms(cf_ctx* ctx, double* l2, double* linf) {
    if (!ctx || !l2 || !linf) return CF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return div_norms(ctx, l2, linf);
}

int cf_test_conversions(cf_ctx* ctx, int n, const double* d, float* f, double* w) {
    if (!ctx || n < 0 || (n > 0 && (!d || !f || !w))) return CF_ERR_INVALID;
    if (n == 0) return CF_OK;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    double *dd = nullptr, *dw = nullptr;
    float* df = nullptr;
    int rc = cuda_check(ctx, cudaMalloc(&dd, sizeof(double) * n), "alloc");
    if (!rc) rc = cuda_check(ctx, cudaMalloc(&dw, sizeof(double) * n), "alloc");
    if (!rc) rc = cuda_check(ctx, cudaMalloc(&df, sizeof(float) * n), "alloc");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(dd, d, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream), "copy");
    if (!rc) rc = cuda_check(ctx, launch_test_convert(ctx, n, dd, df, dw), "convert");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(f, df, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(w, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (!rc) rc = sync(ctx, "conversions");
    cudaFree(dd);
    cudaFree(dw);
    cudaFree(df);
    return rc;
    CF_GUARD_END
}

int cf_test_strip_geometry(int nx, int ny, int tile_w, int tile_h, int strip_rows, int pre, int* fields,
                           int* frame_xy, int cap) {
    if (nx < 1 || ny < 1 || (tile_w != 32 && tile_w != 64) || tile_h < 2 || (tile_h & 1) || strip_rows < 0 ||
        !fields || cap < 0 || (cap > 0 && !frame_xy) || (strip_rows > 0 && tile_w != 64))
        return CF_ERR_INVALID;
    return cf::mg_strip_geometry(nx, ny, tile_w, tile_h, strip_rows, pre, fields, frame_xy, cap);
}

int cf_max_velocity(cf_ctx* ctx, double* umax) {
    if (!ctx || !umax) return CF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    int rc = cuda_check(ctx, launch_max_velocity(ctx, ctx->d_out), "max velocity");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(ctx->h_out, ctx->d_out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (!rc) rc = sync(ctx, "max velocity");
    if (!rc) *umax = ctx->h_out[0];
    return rc;
}

static int points_call(cf_ctx* ctx, int n, const double* xy, double* out, int nout, int kind, int field, int order,
                       double dt) {
    if (n < 0 || (n > 0 && (!xy || !out))) return fail(ctx, CF_ERR_INVALID, "bad point arrays");
    if (n == 0) return CF_OK;
    double *dxy = nullptr, *dout = nullptr;
    int rc = cuda_check(ctx, cudaMalloc(&dxy, sizeof(double) * 2 * n), "cudaMalloc");
    if (!rc) rc = cuda_check(ctx, cudaMalloc(&dout, sizeof(double) * nout * n), "cudaMalloc");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(dxy, xy, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, ctx->stream), "copy");
    if (!rc) {
        cudaError_t e = kind == 0 ? launch_interp_points(ctx, field, order, n, dxy, dout)
                                  : launch_trace_points(ctx, n, dxy, dt, dout);
        rc = cuda_check(ctx, e, "points kernel");
    }
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(out, dout, sizeof(double) * nout * n, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (!rc) rc = sync(ctx, "points");
    cudaFree(dxy);
    cudaFree(dout);
    return rc;
}

int cf_interp_points(cf_ctx* ctx, int field, int order, int n, const double* xy, double* out) {
    if (!ctx) return CF_ERR_INVALID;
    if (field != CF_FIELD_QUANTITY && field != CF_FIELD_U && field != CF_FIELD_V)
        return fail(ctx, CF_ERR_INVALID, "field must be quantity, u or v");
    if (order != 1 && order != 3) return fail(ctx, CF_ERR_INVALID, "order must be 1 or 3");
    if (field == CF_FIELD_QUANTITY && ctx->precision == CF_PREC_MIXED)
        return fail(ctx, CF_ERR_UNSUPPORTED, "FP64 sampling of an FP32 quantity");
    cudaSetDevice(ctx->device);
    return points_call(ctx, n, xy, out, 1, 0, field, order, 0.0);
}

int cf_trace_points(cf_ctx* ctx, int n, const double* xy, double dt, double* out) {
    if (!ctx) return CF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return points_call(ctx, n, xy, out, 2, 1, 0, 1, dt);
}

int cf_cell_velocity(cf_ctx* ctx, double* uc, double* vc, ptrdiff_t si, ptrdiff_t sj) {
    if (!ctx || !uc || !vc) return CF_ERR_INVALID;
    CF_GUARD_BEGIN
    cudaSetDevice(ctx->device);
    if (si <= 0 || sj <= 0) return fail(ctx, CF_ERR_INVALID, "strides must be positive");
    const int nx = ctx->ph.nx, ny = ctx->ph.ny;
    const size_t n = (size_t)nx * ny;
    int rc = CF_OK;
    if (!ctx->outbuf) rc = alloc_dev(ctx, ctx->outbuf, 2 * n);
    if (!rc) rc = cuda_check(ctx, launch_fill_ghosts(ctx), "fill ghosts");
    if (!rc) rc = cuda_check(ctx, launch_cell_velocity(ctx, ctx->outbuf, ctx->outbuf + n), "cell velocity");
    if (rc) return rc;
    double* dst[2] = {uc, vc};
    std::vector<double> tmp;
    if (si != 1) tmp.resize(n);
    for (int f = 0; f < 2; ++f) {
        const double* src = ctx->outbuf + f * n;
        if (si == 1) {
            rc = cuda_check(ctx, cudaMemcpy2DAsync(dst[f], sj * sizeof(double), src, nx * sizeof(double),
                                                   nx * sizeof(double), ny, cudaMemcpyDefault, ctx->stream),
                            "cell velocity copy");
            if (!rc) rc = sync(ctx, "cell velocity copy");
        } else {
            rc = cuda_check(ctx, cudaMemcpyAsync(tmp.data(), src, n * sizeof(double), cudaMemcpyDefault, ctx->stream),
                            "cell velocity copy");
            if (!rc) rc = sync(ctx, "cell velocity copy");
            if (!rc)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) dst[f][i * si + j * sj] = tmp[(size_t)j * nx + i];
        }
        if (rc) return rc;
    }
    return CF_OK;
    CF_GUARD_END
}

long long cf_launch_count(const cf_ctx* ctx) { return ctx ? ctx->launches : -1; }

void* cf_stream(const cf_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int cf_timer_start(cf_ctx* ctx) {
    if (!ctx) return CF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return cuda_check(ctx, cudaEventRecord(ctx->ev[6], ctx->stream), "timer start");
}

int cf_timer_stop(cf_ctx* ctx, double* ms) {
    if (!ctx || !ms) return CF_ERR_INVALID;
    cudaSetDevice(ctx->device);
    int rc = cuda_check(ctx, cudaEventRecord(ctx->ev[7], ctx->stream), "timer stop");
    if (!rc) rc = cuda_check(ctx, cudaEventSynchronize(ctx->ev[7]), "timer stop");
    float f = 0.f;
    if (!rc) rc = cuda_check(ctx, cudaEventElapsedTime(&f, ctx->ev[6], ctx->ev[7]), "timer elapsed");
    *ms = f;
    return rc;
}

int cf_profile_enable(cf_ctx* ctx, int on) {
    if (!ctx) return CF_ERR_INVALID;
    if (on) ctx->pd = cf_profile{};
    ctx->prof = on ? 1 : 0;
    return CF_OK;
}

int cf_profile_read(const cf_ctx* ctx, cf_profile* out) {
    if (!ctx || !out) return CF_ERR_INVALID;
    *out = ctx->pd;
    return CF_OK;
}

int cf_host_alloc(size_t bytes, void** ptr) {
    if (!ptr || bytes == 0) return CF_ERR_INVALID;
    return cudaMallocHost(ptr, bytes) == cudaSuccess ? CF_OK : CF_ERR_NOMEM;
}

int cf_host_free(void* ptr) {
    if (!ptr) return CF_ERR_INVALID;
    return cudaFreeHost(ptr) == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

}  // extern "C"
