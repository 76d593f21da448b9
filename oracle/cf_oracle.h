/*
 * CPU oracle for the cajitafluids per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load this library,
 * and only as the checker or the timed CPU baseline.  The product path
 * (cajitafluids_gb300/) never calls it.
 *
 * Parity status: UNPINNED against the reference's numerics.  The reference
 * (Kokkos + Cabana/Cajita + HYPRE + MPI) cannot be built here, and its own
 * tests pin only mesh geometry and state-array bookkeeping
 * (tests/tstMesh.cpp:16-69, tests/tstProblemManager.cpp:23-98).  Those
 * conventions are pinned by tests/test_oracle_geometry.py.  Everything else
 * is a restatement of the reference's source, cited function by function in
 * cf_oracle.c.
 *
 * The floating-point evaluation order of every formula is fixed and written
 * out in cf_oracle.c (explicit fma(), no contraction), and dot products use
 * a fixed blocked order, so the CUDA FP64 path can be compared bit for bit.
 */
#ifndef CF_ORACLE_H
#define CF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny;              /* global cells per axis */
    double lo[2], hi[2];     /* global bounding box */
    int periodic[2];         /* extension: periodic axes (reference: none) */
    int bc_type[4];          /* [left, bottom, right, top]: 0 SOLID, 1 FREE */
    double src_bbox[4];      /* x0, y0, x1, y1 (x1 = x0 + width) */
    double src_quantity;
    double src_velocity[2];
    int src_mode;            /* 0: clamp (reference), 1: rate q += Q dt */
    double body_force[2];
    int body_density_scaled; /* extension: force scaled by face density */
    double density;
    unsigned quirks;         /* bit 0: fix Q1, bit 1: fix Q3 */
    int precon_none;         /* 1: unpreconditioned CG ("PCG" + "None") */
    int precon_mg;           /* 1: geometric multigrid V-cycle preconditioner */
    int warm_start;          /* extension: start each solve from the previous pressure */
} orc_params;

typedef struct {
    int iterations;
    int status;      /* 0 converged, 1 max_iter, 2 breakdown, 3 nan */
    double bb;       /* ||b||^2 */
    double rr;       /* ||r||^2 at exit */
    double div_l2;   /* L2 norm of the stored field's divergence */
    double div_linf;
} orc_solve_stats;

typedef struct orc_state orc_state;

enum { ORC_Q = 0, ORC_U = 1, ORC_V = 2, ORC_P = 3, ORC_RHS = 4 };

orc_state* orc_create(const orc_params* prm, char* err, int errlen);
void orc_destroy(orc_state* st);
int orc_owned_extent(const orc_state* st, int field, int* ex, int* ey);
int orc_ghosted_extent(const orc_state* st, int field, int* ex, int* ey);
int orc_set_field(orc_state* st, int field, const double* owned);
int orc_get_field(const orc_state* st, int field, double* owned);
int orc_get_ghosted(const orc_state* st, int field, double* full);
int orc_set_ghosted(orc_state* st, int field, const double* full);

void orc_fill_ghosts(orc_state* st);
void orc_advect_step(orc_state* st, double dt, int value_order);
void orc_add_inputs(orc_state* st, double dt);
int orc_project(orc_state* st, double dt, double tol, double abs_tol,
                int max_iter, orc_solve_stats* stats);
int orc_step(orc_state* st, double dt, int value_order, double tol,
             double abs_tol, int max_iter, orc_solve_stats* stats);
void orc_div_norms(const orc_state* st, double* l2, double* linf);

/* test exports */
void orc_sample(const orc_state* st, int field, int order, int n,
                const double* xy, double* out);
void orc_trace(const orc_state* st, int n, const double* xy, double dt,
               double* out);
void orc_matvec(const orc_state* st, double dt, const double* p, double* q);
double orc_canonical_dot(int nx, int ny, const double* a, const double* b);
int orc_mg_apply(orc_state* st, double dt, const double* r, double* z);
int orc_threads(void);

#ifdef __cplusplus
}
#endif
#endif
