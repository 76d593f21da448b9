/*
 * cajitafluids_gb300: C ABI of the GB300-native per-timestep hot path of
 * cajitafluids (RK3 semi-Lagrangian advection, inputs/boundary conditions,
 * pressure projection with a matrix-free Jacobi-PCG Poisson solve).
 *
 * Conventions
 *   - Every function returns int: CF_OK (0) or a negative CF_ERR_* code.
 *     cf_last_error(ctx) describes the last failure on that context.
 *   - No C++ exception crosses this boundary.
 *   - One CUDA stream per context.  Calls on one context are not
 *     thread-safe; distinct contexts are independent.
 *   - All device memory is owned by the context.  Host pointers passed in
 *     are read or written only during the call; every call that touches
 *     host memory returns after the copy has completed.
 *   - Field values are addressed by GLOBAL entity index (gi, gj) of the
 *     owned region, with element (gi, gj) at base[gi * stride_i +
 *     gj * stride_j] (strides in elements), so both Kokkos LayoutLeft and
 *     LayoutRight host mirrors can be passed without a copy.
 *
 * Reference interfaces replaced (paths inside CUP-ECS/cajitafluids):
 *   SolverBase / Solver<2>            src/Solver.hpp:41-48, 55-279
 *   TimeIntegrator::step / advect     src/TimeIntegrator.hpp:81-177
 *   Interpolation::interpolate*       src/Interpolation.hpp:30-54
 *   VelocityCorrectorBase             src/VelocityCorrector.hpp:37-42,
 *     + createVelocityCorrector        src/VelocityCorrector.hpp:297-339
 *   Solver::_addInputs + POD functors src/Solver.hpp:181-263,
 *     BoundaryCondition<2>            src/BoundaryConditions.hpp:50-135
 *     InflowSource<2>                 src/InflowSource.hpp:30-98
 *     BodyForce<2>                    src/BodyForce.hpp:30-69
 *   ProblemManager get/advance/gather src/ProblemManager.hpp:281-403
 *   Mesh geometry                     src/Mesh.hpp:41-103, 119-134
 */
#ifndef CAJITAFLUIDS_GB300_H
#define CAJITAFLUIDS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CF_ABI_VERSION 1

/* return codes */
#define CF_OK 0
#define CF_ERR_INVALID (-1)       /* bad argument (null handle, bad size, ...) */
#define CF_ERR_CUDA (-2)          /* a CUDA runtime call failed */
#define CF_ERR_UNSUPPORTED (-3)   /* valid request that this build does not implement */
#define CF_ERR_NOT_CONVERGED (-4) /* solver stopped at max_iter; state is consistent */
#define CF_ERR_NUMERIC (-5)       /* NaN/Inf or CG breakdown; state is consistent */
#define CF_ERR_NOMEM (-6)         /* device allocation failed */
#define CF_ERR_MESH (-7)          /* extent not evenly divisible (src/Mesh.hpp:49-64) */
#define CF_ERR_TIMEOUT (-9)       /* a bounded device-side wait ran out; state is consistent */

/* fields */
#define CF_FIELD_QUANTITY 0 /* cell-centred advected scalar          */
#define CF_FIELD_U 1        /* x-velocity on I-faces                 */
#define CF_FIELD_V 2        /* y-velocity on J-faces                 */
#define CF_FIELD_PRESSURE 3 /* last projection's pressure (cells)    */

/* boundary types (src/BoundaryConditions.hpp:30-37) */
#define CF_BC_SOLID 0
#define CF_BC_FREE 1

/* precision of a context */
#define CF_PREC_FP64 0  /* all arithmetic and storage in FP64 */
#define CF_PREC_MIXED 1 /* FP32 advection + inner PCG, FP64 outer refinement */

/* quirk switches (default 0 = reproduce the reference) */
#define CF_FIX_Q1 1u /* apply the J-face wall condition to v after projection
                        (reference applies it to u: VelocityCorrector.hpp:260) */
#define CF_FIX_Q3 2u /* RK3 x2 stage uses v1 (Ralston) instead of v0
                        (reference: TimeIntegrator.hpp:57-58) */

/* solver status codes (cf_solve_stats.status) */
#define CF_SOLVE_CONVERGED 0
#define CF_SOLVE_MAX_ITER 1
#define CF_SOLVE_BREAKDOWN 2
#define CF_SOLVE_NAN 3
#define CF_SOLVE_TIMEOUT 4

typedef struct cf_ctx cf_ctx;

/* Mesh + storage description (src/Mesh.hpp:41-103; the reference hard-codes
 * periodic = false, :85-87; periodic axes are an extension). */
typedef struct {
    int nx, ny;          /* global cells per axis */
    double lo[2], hi[2]; /* global bounding box (x0, y0), (x1, y1) */
    int periodic[2];
    int precision;       /* CF_PREC_FP64 or CF_PREC_MIXED */
    int device;          /* CUDA device ordinal */
} cf_grid_desc;

/* Pressure-solver options (src/VelocityCorrector.hpp:96-106, 297-339).
 * solver: "Reference" or "PCG" (both run the GPU preconditioned CG); other
 * HYPRE solver names return CF_ERR_UNSUPPORTED.
 * precon (read for "PCG"; "Reference" always uses the diagonal preconditioner,
 * src/VelocityCorrector.hpp:158-180): "Diagonal" or "Jacobi" -> diagonal
 * (Jacobi) scaling, "None"/"none" -> unpreconditioned CG, "PFMG", "SMG" or
 * "MG" -> one geometric multigrid V-cycle per iteration (cell-centred
 * levels, red-black Gauss-Seidel, bilinear transfers; the reference CLI's
 * default is PCG + PFMG, examples/advection.cpp:186-189; a periodic axis
 * needs an even cell count, else CF_ERR_UNSUPPORTED), other HYPRE names ->
 * CF_ERR_UNSUPPORTED.
 * Convergence: ||r||_2 <= tol * ||b||_2, or, when abs_tol > 0,
 * ||div u||_L2 = ||r||_2 * dx <= abs_tol.  The reference hard-codes
 * tol 1e-6 and max_iter 2000 (:103-104). */
typedef struct {
    const char* solver;
    const char* precon;
    double tol;
    double abs_tol;
    int max_iter;        /* FP64 CG iterations, or total FP32 iterations (mixed) */
    double inner_tol;    /* mixed: FP32 residual reduction that triggers an FP64
                            reliable update (0 = 0.1); with PFMG/SMG/MG, 0.5 or
                            more updates after every iteration (the inner step
                            then only advances x) */
    int max_outer;       /* mixed: limit on FP64 reliable updates (0 = 200) */
} cf_solver_opts;

typedef struct {
    int iterations;       /* CG iterations (mixed: total inner iterations) */
    int outer_iterations; /* mixed: FP64 refinement steps; FP64: 0 */
    int status;           /* CF_SOLVE_* */
    double b_norm;        /* ||b||_2 of the projection right-hand side */
    double r_norm;        /* ||r||_2 at exit (FP64 residual) */
    double div_l2;        /* L2 norm of the stored field's divergence (unit-area cells) */
    double div_linf;      /* max |div u| of the stored field */
} cf_solve_stats;

/* ---- context (replaces Solver ctor + ProblemManager storage) ---- */
/* src/Solver.hpp:69-123, src/ProblemManager.hpp:127-180, src/Mesh.hpp:41-103 */
int cf_ctx_create(const cf_grid_desc* desc, cf_ctx** out);
int cf_ctx_destroy(cf_ctx* ctx);
const char* cf_last_error(const cf_ctx* ctx);
int cf_abi_version(void);
/* owned extent of a field: cells nx*ny, I-faces (nx+1-px)*ny, J-faces nx*(ny+1-py) */
int cf_owned_extent(const cf_ctx* ctx, int field, int* ex, int* ey);
/* mesh accessors: Mesh::cellSize (src/Mesh.hpp:119-122) */
int cf_cell_size(const cf_ctx* ctx, double* dx);

/* ---- inputs: POD functors of src/BoundaryConditions.hpp, InflowSource.hpp, BodyForce.hpp ---- */
/* type[4] in the reference order [left, bottom, right, top] (BoundaryConditions.hpp:68-92) */
int cf_set_bc(cf_ctx* ctx, const int type[4]);
/* InflowSource(location, size, velocity, quantity) (InflowSource.hpp:78-88);
 * mode 0 = clamp q to max(q, Q) (reference), 1 = rate q += Q dt (extension) */
int cf_set_source(cf_ctx* ctx, const double location[2], const double size[2],
                  const double velocity[2], double quantity, int mode);
/* BodyForce(fx, fy) (BodyForce.hpp:62-66); density_scaled (extension) scales the
 * face force by the mean quantity of the two adjacent cells */
int cf_set_body_force(cf_ctx* ctx, const double force[2], int density_scaled);
/* density used by the VelocityCorrector (src/VelocityCorrector.hpp:72-76) */
int cf_set_density(cf_ctx* ctx, double density);
/* Extension: on != 0 starts each projection from the previous pressure (r =
 * b - A p_prev) instead of the reference's cold start x0 = 0
 * (src/VelocityCorrector.hpp:272).  Fewer iterations per step; the result
 * differs from the cold start within the solver tolerance.  The adjoint
 * (cf_forward_checkpointed / cf_backward) returns CF_ERR_UNSUPPORTED while on. */
int cf_set_warm_start(cf_ctx* ctx, int on);
int cf_set_quirks(cf_ctx* ctx, unsigned flags);
/* Launch mode (no counterpart in the reference; Kokkos launches every
 * parallel_for on its own).  on = 1 (default): the pressure solve runs as
 * CUDA graphs (one device-resident graph per projection, or host-polled
 * graph batches).  on = 0: every kernel of the solve is launched on its own
 * and the host polls the solver state between batches, for tools that list
 * kernel launches one by one.  The results are the same bits either way.
 * The environment variable CF_GRAPHS=0 sets every new context to on = 0. */
int cf_set_graphs(cf_ctx* ctx, int on);

/* ---- state (ProblemManager::get / initialize / advance) ---- */
int cf_upload(cf_ctx* ctx, int field, const double* host, ptrdiff_t stride_i, ptrdiff_t stride_j);
int cf_download(cf_ctx* ctx, int field, double* host, ptrdiff_t stride_i, ptrdiff_t stride_j);
/* full ghosted array (local index, x fastest) for halo tests */
int cf_download_ghosted(cf_ctx* ctx, int field, double* host, int* ex, int* ey);
/* ProblemManager::gather(Current) (src/ProblemManager.hpp:394-398): on one GPU,
 * an on-device ghost fill (wrap copy along periodic axes; wall ghosts stay 0) */
int cf_fill_ghosts(cf_ctx* ctx);

/* ---- hot path ---- */
/* TimeIntegrator::step<2> (src/TimeIntegrator.hpp:120-177): gather, advect q, u, v
 * from Current into Next, swap.  value_order = 1 (linear) or 3 (cubic, reference). */
int cf_advect(cf_ctx* ctx, double dt, int value_order);
/* Solver::_addInputs (src/Solver.hpp:181-263) */
int cf_add_inputs(cf_ctx* ctx, double dt);
/* VelocityCorrectorBase::correctVelocity (src/VelocityCorrector.hpp:266-282) */
int cf_project(cf_ctx* ctx, double dt, const cf_solver_opts* opts, cf_solve_stats* stats);
/* Solver::setup (src/Solver.hpp:125-133): add inputs, correct velocity */
int cf_setup(cf_ctx* ctx, double dt, const cf_solver_opts* opts, cf_solve_stats* stats);
/* Solver::step (src/Solver.hpp:135-147): advect, add inputs, correct velocity.
 * The input stage is fused into the advection kernel unless the body force
 * is density scaled. */
int cf_step(cf_ctx* ctx, double dt, int value_order, const cf_solver_opts* opts,
            cf_solve_stats* stats);
/* Solver::step (as cf_step) with host buffers in and out: q_in, u_in, v_in
 * are uploaded into the current state, one step runs, and the new q, u, v are
 * written to q_out, u_out, v_out (any of the outputs may be NULL).  All six
 * arrays are owned regions, x fastest, contiguous (element (i, j) at
 * [j * ex + i], ex from cf_owned_extent).  Copies are asynchronous (page-locked
 * buffers from cf_host_alloc give the full link bandwidth); q_out is copied on
 * a second stream while the projection runs; the call returns after one final
 * synchronisation, so the buffers are only touched during the call. */
int cf_step_host(cf_ctx* ctx, double dt, int value_order, const cf_solver_opts* opts, cf_solve_stats* stats,
                 const double* q_in, const double* u_in, const double* v_in, double* q_out, double* u_out,
                 double* v_out);

/* Solver::solve's step loop (src/Solver.hpp:149-177) on the device: nsteps
 * calls' worth of cf_step enqueued back to back with one synchronisation at
 * the end.  stats: the last step's solve.  *unconverged (may be NULL): how
 * many of the steps' pressure solves did not converge.  Returns CF_OK when
 * all converged, else the code of the worst failure (CF_ERR_NOT_CONVERGED,
 * CF_ERR_NUMERIC, CF_ERR_TIMEOUT); the state has advanced nsteps either way. */
int cf_steps(cf_ctx* ctx, int nsteps, double dt, int value_order, const cf_solver_opts* opts,
             cf_solve_stats* stats, int* unconverged);

/* divergence norms of the current velocity field */
int cf_div_norms(cf_ctx* ctx, double* l2, double* linf);
/* max |u|, |v| over owned faces (for CFL time steps) */
int cf_max_velocity(cf_ctx* ctx, double* umax);

/* ---- adjoint (no counterpart in the reference: new functionality) ----
 * Forward/backward contract of an autograd function over nsteps Solver::step
 * calls (src/Solver.hpp:135-147) from the current state s_0.
 * cf_forward_checkpointed runs the steps, storing the state every ckpt_every
 * steps (sqrt(nsteps) keeps memory at O(sqrt(nsteps)) states); the context
 * ends in s_T.  cf_backward takes dL/dq(T) and optionally dL/du(T), dL/dv(T)
 * (NULL = 0), recomputes each segment from its checkpoint, runs the reverse
 * steps, and writes dL/dq(0), dL/du(0), dL/dv(0) and dL/dQ for the quantity
 * source's Q: its rate (rate form) or its level (clamp form) (any output may
 * be NULL); the context is left
 * in s_T with the pressure at zero.  Host arrays are contiguous owned regions (x fastest).  An FP64
 * context runs the FP64 adjoint; a mixed context checkpoints its own state
 * (FP32 q, velocity pairs), recomputes the mixed forward, and runs the
 * reverse advection in FP32 and the transposed projection with the mixed
 * PCG (FP32 inner iterations, double-float refinement; relative tolerance
 * opts->tol, default 1e-7).  See cf_adjoint.cu for the supported inputs. */
int cf_forward_checkpointed(cf_ctx* ctx, int nsteps, int ckpt_every, double dt, int value_order,
                            const cf_solver_opts* opts, cf_solve_stats* last);
int cf_backward(cf_ctx* ctx, const double* dL_dq_T, const double* dL_du_T, const double* dL_dv_T, double* dL_dq0,
                double* dL_du0, double* dL_dv0, double* dL_drate);

/* ---- test exports (Interpolation / rk3 at arbitrary points) ---- */
/* Interpolation::interpolateField (src/Interpolation.hpp:30-41) of a state field
 * at n physical points xy[2n] */
int cf_interp_points(cf_ctx* ctx, int field, int order, int n, const double* xy, double* out);
/* TimeIntegrator::rk3 (src/TimeIntegrator.hpp:36-77) of n points */
int cf_trace_points(cf_ctx* ctx, int n, const double* xy, double dt, double* out);
/* the device's FP64 -> FP32 (round to nearest even) and FP32 -> FP64
 * conversions of the mixed-precision kernels, applied to d[n]: f = narrowed,
 * w = f widened (no counterpart in the reference) */
int cf_test_conversions(cf_ctx* ctx, int n, const double* d, float* f, double* w);

/* launch geometry of the fused multigrid pre-smoothing (pre != 0) or
 * post-smoothing kernel on an nx x ny level with tile_w x tile_h tiles
 * (tile_w 32 or 64) and register strips of about strip_rows rows (0: tiles
 * only), computed on the host without a device (no counterpart in the
 * reference).  fields[CF_STRIP_FIELDS]: frame blocks, tiles per row, the
 * strip-covered tile rectangle [txa, txb) x [tya, tyb), strips per row and
 * rows of strips, strip height, first written column and row, columns written
 * per strip, column halo, row halo, columns read per strip, row unroll, strips
 * per block, blocks launched.  frame_xy (optional, 2 * cap ints) receives the
 * tile (x, y) of each frame block. */
#define CF_STRIP_FIELDS 18
int cf_test_strip_geometry(int nx, int ny, int tile_w, int tile_h, int strip_rows, int pre, int* fields,
                           int* frame_xy, int cap);

/* Test hook (host-side failure injection, no GPU fault): with nth > 0 the
 * nth device allocation of the library from now on fails as an out-of-memory
 * cudaMalloc would (CF_ERR_NOMEM); 0 switches the injection off. */
int cf_test_fail_alloc(int nth);
/* Test hook (timeout path, no GPU fault): with on != 0, the first tile wait
 * of one CTA of the mixed-precision inner CG waits on an mbarrier that
 * nothing arrives on, with a short limit; it times out, the CTA waits for
 * its own bulk copies in flight and returns, and the projection returns
 * CF_ERR_TIMEOUT.  The context stays usable; 0 switches the hook off. */
int cf_test_stall_wait(cf_ctx* ctx, int on);
/* Test hook: with on != 0, every tile of the mixed-precision advection reads
 * its stencil taps from global memory (the path a tile takes when a trace
 * could leave its shared-memory window) instead of the staged window.  The
 * results are the same bits either way; 0 switches the hook off. */
int cf_test_advect_unstaged(cf_ctx* ctx, int on);
/* Test hook: with on != 0, the mixed-precision pressure gradient updates
 * every face in the one-thread-per-face kernel the FP64 gradient uses
 * instead of the unit-per-warp kernel.  The results are the same bits either
 * way; 0 switches the hook off. */
int cf_test_apply_general(cf_ctx* ctx, int on);

/* ---- output (replaces the device half of SiloWriter::writeFile) ----
 * SiloWriter interpolates the face velocities to cell centres for its
 * "velocity" zonal variable (src/SiloWriter.hpp:177-205:
 * interpolateVelocity<2, 1> at every owned cell centre).  cf_cell_velocity
 * fills uc, vc (nx x ny, element (i, j) at base[i*stride_i + j*stride_j]) with
 * that interpolation of the current velocities (ghosts refreshed first).  The
 * "quantity" variable is cf_download(CF_FIELD_QUANTITY); the mesh is the node
 * coordinates lo + i dx.  The C++ mirror's SiloWriter<2> writes these in the
 * Silo variables' layout to a raw file (libsilo is not part of this build). */
int cf_cell_velocity(cf_ctx* ctx, double* uc, double* vc, ptrdiff_t stride_i, ptrdiff_t stride_j);

/* ---- instrumentation ---- */
/* number of kernels this context has launched (graph nodes included) */
long long cf_launch_count(const cf_ctx* ctx);
/* CUDA stream of the context (cudaStream_t), for event timing by the caller */
void* cf_stream(const cf_ctx* ctx);
/* CUDA-event timer on the context stream: start, then stop returns the
 * device time between the two events in milliseconds (waits for the stop) */
int cf_timer_start(cf_ctx* ctx);
int cf_timer_stop(cf_ctx* ctx, double* ms);

/* Device-time profile kept by the context while enabled.  A projection
 * normally runs as one device-resident CUDA graph (the PCG iterations in a
 * conditional loop on the device, one host synchronisation per projection).
 * While profiling is enabled it runs instead in host-polled CUDA-graph batches
 * (CF_CG_BATCH Jacobi-PCG or 4 multigrid-PCG iterations) with CUDA events
 * around each; only batches in which every iteration ran are counted, so
 * solve_ms / solve_iters is the device time of one PCG iteration (all its
 * kernels).  The two forms compute the same results. */
#define CF_CG_BATCH 32
typedef struct {
    double solve_ms;
    long long solve_iters;
    long long solve_batches;
    double advect_ms;
    long long advect_calls;
    double project_ms;
    long long projects;
    double adj_advect_ms;        /* mixed adjoint: the FP32 reverse advection (k_adj_advect32) */
    long long adj_advect_calls;
    long long adj_projects;      /* the adjoint's transposed projections and their PCG iterations */
    long long adj_iters;
} cf_profile;
/* on != 0 resets the counters and starts recording; 0 stops recording */
int cf_profile_enable(cf_ctx* ctx, int on);
int cf_profile_read(const cf_ctx* ctx, cf_profile* out);

/* page-locked host memory for fast cf_upload / cf_download */
int cf_host_alloc(size_t bytes, void** ptr);
int cf_host_free(void* ptr);

/* ---- allocation-free divergence norms (no counterpart in the reference) ----
 * For callers that own their velocity arrays on the device and cannot
 * allocate device memory where they need the norm: codes whose device
 * memory belongs to their own pool allocator or fixed memory budget, and
 * hooks inside latency-critical loops where cudaMalloc/cudaFree would
 * synchronise the device.  cf_div_norms needs a context, and creating one
 * allocates the whole state.  This entry point allocates nothing (no
 * cudaMalloc, cudaFree or allocating library call); its reduction scratch
 * is a fixed 1 MiB device array inside this library, held by every GPU that
 * loads the library until the process exits.
 *
 * u: device pointer to u(0, 0) of the owned I-faces, u(gi, gj) at
 *    u[gj * u_pitch + gi], (nx + 1 - periodic_x) x ny values; v likewise
 *    for the J-faces, nx x (ny + 1 - periodic_y).  out: device pointer to two
 *    doubles: the L2 norm of div u with unit-area cells and max |div u|,
 *    equal bit for bit to what cf_div_norms returns for an FP64 context
 *    holding the same u and v (a mixed-precision context squares the
 *    divergence in FP32 before its FP64 sum, so its L2 norm can differ in
 *    the last bits).  stream: a cudaStream_t (NULL = default
 *    stream).  The call only enqueues work; read out after the stream.
 * Limits: at most CF_NOALLOC_MAX_UNITS units of 64 x 16 cells (8192 x 8192
 * cells); larger grids return CF_ERR_TOO_LARGE without touching the GPU.
 * The first call on each device looks up the scratch address on that
 * device (make that first call before any stream capture) and keeps it for
 * the rest of the process: that address belongs to the CUDA runtime's
 * primary context of the device, so calls must run with that context
 * current, and not after cudaDeviceReset on that device (the library's
 * device module, and with it the scratch array, may then sit elsewhere).  All calls share
 * the one scratch array: calls that overlap on the GPU (different streams,
 * or threads without ordering) race and give wrong results. */
#define CF_ERR_TOO_LARGE (-8)
#define CF_NOALLOC_MAX_UNITS 65536
int cf_div_norms_noalloc(const double* u, ptrdiff_t u_pitch, const double* v, ptrdiff_t v_pitch, int nx, int ny,
                         int periodic_x, int periodic_y, double dx, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
