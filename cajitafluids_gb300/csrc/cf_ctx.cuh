// Host-side context of one simulation on one GPU (opaque cf_ctx of the C ABI).
#pragma once
#include <string>
#include <vector>

#include <cuda.h>

#include "../../include/cajitafluids_gb300.h"
#include "cf_internal.cuh"

struct cf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cf::Phys ph{};
    int precision = 0;
    double density = 1.0;
    int warm = 0;  // start each projection from the previous pressure (cf_set_warm_start)
    // the adjoint's transposed projections start from the previous reverse
    // step's adjoint pressure (set by cf_backward, which keeps that pressure
    // in a vector of its own between steps)
    int adj_warm = 0;
    // mixed MG-PCG with a reliable update after every iteration (threshold >=
    // 0.5): the inner step only advances x (set per projection from its options)
    int x_only = 0;
    int gmg_xonly = -1;  // x_only of the cached host-polled MG graphs
    // fields, two versions each (src/ProblemManager.hpp:143-165); index cur is
    // Current.  A mixed context keeps q in FP32 (q32) and u, v as double-float
    // pairs: each 8-byte element of u, v holds (hi, lo) = (fl32(w), fl32(w -
    // hi)) of the face velocity w.
    cf::Grid<double> q64[2]{}, u[2]{}, v[2]{};
    cf::Grid<float> q32[2]{};
    cf::Grid<double> vel64[2]{};  // mixed: FP64 copies of u, v for the sampling exports, made on first use
    int cur = 0;

    // solver vectors (owned cells)
    int vpitch = 0;
    cf::Vec64 x{}, r{}, pa{}, pb{}, qv{}, b{};
    // mixed: the second buffer of the double-float solution (the MG-PCG's
    // fused x update writes the updated x there; SolverState::xsel)
    cf::Vec64 xb{};
    double* bnd = nullptr;  // mixed: unit-boundary faces of u and v before the gradient
    // the last mixed projection left the pressure as double-float pairs (in
    // the buffer SolverState::xsel names); a download converts it
    int p_df = 0;
    // FP32 vectors with a one-cell ghost ring: element (i, j) at a[j * p32 + i],
    // storage base = a - p32 - 4 (see cf_cg32.cu)
    cf::Vec32 r32{}, pa32{}, pb32{};
    float *r32b = nullptr, *pa32b = nullptr, *pb32b = nullptr;
    int p32 = 0;
    CUtensorMap map_r{}, map_pa{}, map_pb{};
    int tiles_x = 0, tiles = 0, cta32 = 0, cta32b = 0;
    double* partials = nullptr;  // 4 * n_units
    int G = 0, B = 0, n_units = 0;
    int sms = 1;  // multiprocessors of the device (launch sizing)
    cf::SolverState* S = nullptr;   // device
    cf::SolverState* hS = nullptr;  // pinned host mirror (solver state copied back)
    cf::SolverState* hP = nullptr;  // pinned solver parameters copied in (not overwritten by a projection)
    cf::SolverState* hPa = nullptr; // the same for the adjoint's projections
    int* d_tally = nullptr;         // resident projections: [0] unconverged solves, [1] worst status, [2] trips
    double* d_out = nullptr;        // small device output slots
    double* h_out = nullptr;        // pinned host mirror
    double* staging = nullptr;      // FP64 staging for conversions / strided copies
    size_t staging_elems = 0;

    // CUDA graphs of batches of solver iterations, rebuilt when the stencil changes
    cudaGraphExec_t g64 = nullptr, g32 = nullptr;
    int g64_batch = 0, g32_batch = 0;
    cf::Stencil g64_st{}, g32_st{};

    void* adjoint = nullptr;  // checkpoints and adjoint buffers (cf_adjoint.cu)
    void* mg = nullptr;       // multigrid hierarchy (cf_mg.cu)
    double* outbuf = nullptr; // 2 nx ny doubles for cf_cell_velocity, allocated on first use
    // cf_step_host: a second stream for the quantity's download, which overlaps
    // the projection, and its staging buffer (nx ny doubles), made on first use
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_adv = nullptr;
    cudaEvent_t ev_uv = nullptr, ev_q = nullptr;  // cf_step_host: velocities in, quantity in
    cudaEvent_t ev_press = nullptr;  // recorded by the resident projection right after the gradient subtraction
    double* staging2 = nullptr;
    double* staging_uv = nullptr;  // cf_step_host (mixed): u, v as FP64 for their download
    cudaGraphExec_t gmg = nullptr;      // batch of MG-PCG iterations
    cudaGraphExec_t gmg_pre = nullptr;  // V-cycle + r.z after the residual is (re)formed
    cf::Stencil gmg_st{};
    int gmg_per_iter = 0, gmg_pre_launches = 0;
    // device-resident projection graphs (cf_project.cu): slots 0, 1 for the
    // two state buffers, 2, 3 for the adjoint's two pairs of face arrays
    cudaGraphExec_t rgx[4] = {nullptr, nullptr, nullptr, nullptr};
    cf::Stencil rg_st[4]{};
    cf::Phys rg_ph[4]{};
    int rg_flags[4] = {-1, -1, -1, -1};
    const double* rg_u[4] = {nullptr, nullptr, nullptr, nullptr};  // the u array each slot projects
    // launch counts per graph: projection slots 0-3, whole-step graphs 4, 5
    int rg_head[6] = {}, rg_trip[6] = {}, rg_tail[6] = {};
    int rg_pending = 0;  // count slot of the last resident projection launched
    // whole-step graphs (cf_project.cu step_resident): index = the state
    // buffer the step starts from; ghost fill, advection and inputs, then the
    // resident projection of the other buffer; rebuilt when a key changes
    cudaGraphExec_t sgx[2] = {nullptr, nullptr};
    double sg_dt[2] = {0.0, 0.0};
    int sg_order[2] = {0, 0}, sg_fuse[2] = {-1, -1}, sg_flags[2] = {-1, -1};
    cf::Stencil sg_st[2]{};
    cf::Phys sg_ph[2]{};
    // FP32 z = M^-1 r of the mixed MG-PCG, ghost ring as the other FP32 vectors
    cf::Vec32 z32{};
    float* z32b = nullptr;
    CUtensorMap map_z{};
    long long launches = 0;
    // cf_set_graphs(ctx, 0): every kernel is issued on its own (no CUDA graphs,
    // host-polled projection); the results are the same bits
    int direct = 0;
    // cf_test_stall_wait: the inner FP32 CG's first tile wait of block 0
    // waits on an mbarrier nothing arrives on (timeout-path test)
    int test_stall = 0;
    // cf_test_advect_unstaged: every FP32 advection tile reads its taps from
    // global memory instead of its shared-memory window (same bits)
    int test_unstaged = 0;
    int test_general_apply = 0;  // mixed gradient through k_apply_pressure
    // profiling (cf_profile_enable)
    int prof = 0;
    cf_profile pd{};
    cudaEvent_t ev[8] = {};
    std::string err;
    std::vector<void*> allocs;
};

namespace cf {
// helpers implemented in cf_api.cu
int fail(cf_ctx* c, int code, const char* fmt, ...);
int cuda_check(cf_ctx* c, cudaError_t e, const char* what);
void build_stencil(const cf_ctx* c, double dt, int precon_none, Stencil* st);

// launchers (cf_fields.cu)
// ghost fills: what = GHOSTS_Q | GHOSTS_UV, on stream (null: the context's)
enum { GHOSTS_Q = 1, GHOSTS_UV = 2, GHOSTS_ALL = 3 };
cudaError_t launch_fill_ghosts(cf_ctx* c, int what = GHOSTS_ALL, cudaStream_t stream = nullptr);
// advection of entities [ent0, ent0 + nent) (0 q, 1 u, 2 v); prep: make the
// FP32 velocity copies first (mixed); advance: switch to the new state after
cudaError_t launch_advect(cf_ctx* c, double dt, int order, int fuse_inputs, int ent0 = 0, int nent = 3,
                          bool prep = true, bool advance = true);
cudaError_t launch_add_inputs(cf_ctx* c, double dt);
cudaError_t launch_interp_points(cf_ctx* c, int field, int order, int n, const double* d_xy, double* d_out);
cudaError_t launch_trace_points(cf_ctx* c, int n, const double* d_xy, double dt, double* d_out);
cudaError_t launch_cell_velocity(cf_ctx* c, double* d_uc, double* d_vc);
cudaError_t launch_max_velocity(cf_ctx* c, double* d_out);
cudaError_t launch_test_convert(cf_ctx* c, int n, const double* d, float* f, double* w);
cudaError_t launch_convert_q(cf_ctx* c, int to_device, int version, cudaStream_t stream = nullptr);
// mixed u, v (field CF_FIELD_U / CF_FIELD_V of state version): the owned FP64
// values in place to pairs, or the owned pairs to FP64 in dst (row pitch =
// the owned width)
cudaError_t launch_to_pairs(cf_ctx* c, int field, int version, cudaStream_t stream = nullptr);
cudaError_t launch_from_pairs(cf_ctx* c, int field, int version, double* dst, cudaStream_t stream = nullptr);
// the current u, v as FP64 ghosted arrays (mixed: converted copies)
int velocity_f64(cf_ctx* c, Grid<double>* gu, Grid<double>* gv);
int alloc_grid64(cf_ctx* c, Grid<double>& g, int ex, int ey);
cudaError_t launch_q_to_f64(cf_ctx* c, int version, double* dst, cudaStream_t stream);

// projection (cf_project.cu)
struct SolveOpts {
    double tol, abs_tol, inner_tol;
    int max_iter, max_outer;
    int precon_none;
    int precon_mg;  // geometric multigrid V-cycle (cf_mg.cu)
};
struct SolveResult {
    int iterations, outer, status;
    double bb, rr, div_l2, div_linf;
};
int project(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res);
// one whole step (ghost fill, advection, inputs, resident projection) as one
// graph launch, without a synchronisation (project_collect fills res after
// the caller has synchronised the stream); the context then holds the new
// state.  Used when the resident graphs serve (resident_projection()).
int step_resident(cf_ctx* c, double dt, int order, int fuse, const SolveOpts& o, bool params_ready);
// project without the final synchronisation when the device-resident graph
// serves it (*deferred = true; project_collect fills res after the caller has
// synchronised the stream), else a plain project (*deferred = false)
bool resident_projection();  // device-resident projection graphs in use (CF_RESIDENT=0 turns them off)
int project_async(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res, bool* deferred,
                  bool params_ready = false);
// results of the last deferred resident projection; launch counts for it,
// or (nproj > 0) for nproj projections with trips loop trips in all
void project_collect(cf_ctx* c, SolveResult* res, int nproj = 0, long long trips = 0);
int project_grids(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res, Grid<double> gu, Grid<double> gv,
                  int adjoint);
// the adjoint's projection of gu, gv, deferred like project_async when the
// resident graph serves it
int project_adjoint_async(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res, bool* deferred,
                          bool params_ready, Grid<double> gu, Grid<double> gv);
// one step enqueued without a synchronisation (cf_api.cu)
int enqueue_step(cf_ctx* ctx, double dt, int value_order, const SolveOpts& so, SolveResult* r, bool* deferred,
                 bool params_ready);
int parse_solver_opts(cf_ctx* ctx, const cf_solver_opts* opts, SolveOpts* so);
// FP32 TMA inner CG (cf_cg32.cu)
int cg32_setup(cf_ctx* c);
void cg32_launch_iteration(cf_ctx* c, const Stencil& st);
int cg32_mg_setup(cf_ctx* c);
int cg32_mg_precondition(cf_ctx* c, double scale);  // returns kernels launched
void cg32_launch_pair_mg(cf_ctx* c, const Stencil& st);
int div_norms(cf_ctx* c, double* l2, double* linf);
// mixed: the double-float solution as an FP64 pressure (owned cells, row
// pitch nx) in out
cudaError_t pressure_to_f64(cf_ctx* c, double* out);
// multigrid preconditioner (cf_mg.cu)
int mg_setup(cf_ctx* c);
void mg_free(cf_ctx* c);
// Enqueues one V-cycle, returns kernels launched.  Mixed precision with
// rz_done non-null: the finest post-smoothing kernel also forms rho = r.z,
// the CG scalars and z's periodic ghosts when the level runs fused (*rz_done
// tells whether it did).
int mg_vcycle(cf_ctx* c, double scale0, bool* rz_done = nullptr);
int mg_levels(const cf_ctx* c);
int mg_strip_geometry(int nx, int ny, int tw, int th, int strip_rows, int pre, int* fields, int* frame_xy, int cap);
double* mg_z64(cf_ctx* c);
}  // namespace cf

void cf_adjoint_free(cf_ctx* c);
