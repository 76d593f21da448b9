/*
 * CPU oracle: a plain-C FP64 restatement of the cajitafluids per-timestep
 * hot path (Solver::step, src/Solver.hpp:135-147).
 *
 * TEST INFRASTRUCTURE ONLY (see cf_oracle.h).  Parity unpinned: the
 * reference cannot be built here, so this file restates its source.  Each
 * function names the reference file:line it follows.
 *
 * Evaluation-order contract (shared with the CUDA FP64 kernels, written
 * independently there):
 *   - arithmetic the reference writes out in its own files (the rk3 stages,
 *     the body force, the divergence, the gradient subtraction, the matrix
 *     entries) is evaluated as written: C++ precedence, left to right, one
 *     rounding per operation, no contraction (build with -ffp-contract=off);
 *     the reference's own code compiled the same way gives the same bits
 *     (oracle/refshim and tests/test_reference_pin.py);
 *   - in the parts the reference delegates to Cajita (spline weights and
 *     sums, the conjugate-gradient recurrences), every fused multiply-add is
 *     an explicit fma();
 *   - dot products are summed in a fixed blocked order: the owned cell grid
 *     is cut into units of 64 columns x 16 rows; unit u = band * G + g;
 *     inside a unit, "lane" l (0..31) owns columns 64g+2l and 64g+2l+1 and
 *     accumulates acc = fma(a, b, acc) row by row (row ascending, the two
 *     columns in order); the 32 lane sums are folded by a butterfly
 *     (xor 16, 8, 4, 2, 1); the unit partials are then summed by 256
 *     strided accumulators (s[t] += partial[t + 256k]), each group of 32
 *     folded by the same butterfly, and the 8 group sums added in order.
 */
#include "cf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define HALO 3
#define UNIT_COLS 64
#define BAND_ROWS 16
#define FINAL_THREADS 256

enum { E_CELL = 0, E_FACEI = 1, E_FACEJ = 2 };
enum { SOLID = 0, FREE = 1 };

/* Entity offsets in cell units: Cajita places cells at (i+1/2, j+1/2),
 * I-faces at (i, j+1/2) and J-faces at (i+1/2, j). */
static const double ENT_OFF[3][2] = {{0.5, 0.5}, {0.0, 0.5}, {0.5, 0.0}};

typedef struct {
    double* a;
    int ex, ey; /* ghosted extents */
} grid_t;

struct orc_state {
    orc_params p;
    double dx, rdx;
    double gl[2];       /* low corner of the ghosted local mesh */
    grid_t f[3][2];     /* [field][0 current, 1 next] */
    double *x, *r, *pv, *qv, *z, *rhs, *diag, *minv;
    double* partial;
    int n_units;
};

static inline double* at(const grid_t* g, int i, int j) {
    return g->a + (size_t)j * g->ex + i;
}

static int owned_count(const orc_state* st, int field, int axis) {
    int n = axis == 0 ? st->p.nx : st->p.ny;
    if ((field == ORC_U && axis == 0) || (field == ORC_V && axis == 1))
        return st->p.periodic[axis] ? n : n + 1;
    return n;
}

static int ghost_count(const orc_state* st, int field, int axis) {
    int n = axis == 0 ? st->p.nx : st->p.ny;
    int extra = ((field == ORC_U && axis == 0) || (field == ORC_V && axis == 1)) ? 1 : 0;
    return n + 2 * HALO + extra;
}

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Mesh construction: the uniform cell size and its extent check,
 * src/Mesh.hpp:49-64. */
orc_state* orc_create(const orc_params* prm, char* err, int errlen) {
    if (prm->nx <= 0 || prm->ny <= 0) {
        snprintf(err, errlen, "cell counts must be positive");
        return NULL;
    }
    double dx = (prm->hi[0] - prm->lo[0]) / prm->nx;
    for (int d = 0; d < 2; ++d) {
        int n = d == 0 ? prm->nx : prm->ny;
        double extent = n * dx;
        if (fabs(extent - (prm->hi[d] - prm->lo[d])) > 10.0 * DBL_EPSILON) {
            snprintf(err, errlen, "Extent not evenly divisible by uniform cell size");
            return NULL;
        }
    }
    if (prm->precon_mg && ((prm->periodic[0] && (prm->nx & 1)) || (prm->periodic[1] && (prm->ny & 1)))) {
        snprintf(err, errlen, "multigrid needs an even cell count along periodic axes");
        return NULL;
    }
    orc_state* st = (orc_state*)calloc(1, sizeof(orc_state));
    st->p = *prm;
    st->dx = dx;
    st->rdx = 1.0 / dx;
    for (int d = 0; d < 2; ++d) st->gl[d] = prm->lo[d] - 3.0 * dx;
    for (int fld = 0; fld < 3; ++fld)
        for (int v = 0; v < 2; ++v) {
            grid_t* g = &st->f[fld][v];
            g->ex = ghost_count(st, fld, 0);
            g->ey = ghost_count(st, fld, 1);
            g->a = (double*)calloc((size_t)g->ex * g->ey, sizeof(double));
        }
    size_t n = (size_t)prm->nx * prm->ny;
    st->x = (double*)calloc(n, sizeof(double));
    st->r = (double*)calloc(n, sizeof(double));
    st->pv = (double*)calloc(n, sizeof(double));
    st->qv = (double*)calloc(n, sizeof(double));
    st->z = (double*)calloc(n, sizeof(double));
    st->rhs = (double*)calloc(n, sizeof(double));
    st->diag = (double*)calloc(n, sizeof(double));
    st->minv = (double*)calloc(n, sizeof(double));
    int G = (prm->nx + UNIT_COLS - 1) / UNIT_COLS;
    int B = (prm->ny + BAND_ROWS - 1) / BAND_ROWS;
    st->n_units = G * B;
    st->partial = (double*)calloc((size_t)st->n_units, sizeof(double));
    return st;
}

void orc_destroy(orc_state* st) {
    if (!st) return;
    for (int fld = 0; fld < 3; ++fld)
        for (int v = 0; v < 2; ++v) free(st->f[fld][v].a);
    free(st->x); free(st->r); free(st->pv); free(st->qv); free(st->z);
    free(st->rhs); free(st->diag); free(st->minv); free(st->partial);
    free(st);
}

int orc_owned_extent(const orc_state* st, int field, int* ex, int* ey) {
    if (field >= ORC_Q && field <= ORC_V) {
        *ex = owned_count(st, field, 0);
        *ey = owned_count(st, field, 1);
        return 0;
    }
    if (field == ORC_P || field == ORC_RHS) {
        *ex = st->p.nx;
        *ey = st->p.ny;
        return 0;
    }
    return -1;
}

int orc_ghosted_extent(const orc_state* st, int field, int* ex, int* ey) {
    if (field < ORC_Q || field > ORC_V) return -1;
    *ex = st->f[field][0].ex;
    *ey = st->f[field][0].ey;
    return 0;
}

int orc_set_field(orc_state* st, int field, const double* owned) {
    if (field < ORC_Q || field > ORC_V) return -1;
    int ox = owned_count(st, field, 0), oy = owned_count(st, field, 1);
    grid_t* g = &st->f[field][0];
    for (int j = 0; j < oy; ++j)
        for (int i = 0; i < ox; ++i) *at(g, i + HALO, j + HALO) = owned[(size_t)j * ox + i];
    return 0;
}

int orc_get_field(const orc_state* st, int field, double* owned) {
    if (field == ORC_P || field == ORC_RHS) {
        memcpy(owned, field == ORC_P ? st->x : st->rhs,
               sizeof(double) * (size_t)st->p.nx * st->p.ny);
        return 0;
    }
    if (field < ORC_Q || field > ORC_V) return -1;
    int ox = owned_count(st, field, 0), oy = owned_count(st, field, 1);
    const grid_t* g = &st->f[field][0];
    for (int j = 0; j < oy; ++j)
        for (int i = 0; i < ox; ++i) owned[(size_t)j * ox + i] = *at(g, i + HALO, j + HALO);
    return 0;
}

int orc_get_ghosted(const orc_state* st, int field, double* full) {
    if (field < ORC_Q || field > ORC_V) return -1;
    const grid_t* g = &st->f[field][0];
    memcpy(full, g->a, sizeof(double) * (size_t)g->ex * g->ey);
    return 0;
}

int orc_set_ghosted(orc_state* st, int field, const double* full) {
    if (field < ORC_Q || field > ORC_V) return -1;
    grid_t* g = &st->f[field][0];
    memcpy(g->a, full, sizeof(double) * (size_t)g->ex * g->ey);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Ghost fill: the single-rank form of the advection halo gather
 * (src/ProblemManager.hpp:173-176, 394-398; NodeHaloPattern, depth 3).
 * Along a wall axis there is no neighbour and the ghosts keep the zeros
 * they were given at construction (src/ProblemManager.hpp:149-165).  Along
 * a periodic axis (extension) the ghost copies the wrapped owned entity. */
void orc_fill_ghosts(orc_state* st) {
    for (int fld = 0; fld < 3; ++fld) {
        grid_t* g = &st->f[fld][0];
        int nox = owned_count(st, fld, 0), noy = owned_count(st, fld, 1);
        for (int j = 0; j < g->ey; ++j)
            for (int i = 0; i < g->ex; ++i) {
                int gi = i - HALO, gj = j - HALO;
                int in_x = gi >= 0 && gi < nox, in_y = gj >= 0 && gj < noy;
                if (in_x && in_y) continue;
                if (!in_x) {
                    if (!st->p.periodic[0]) continue;
                    gi = ((gi % nox) + nox) % nox;
                }
                if (!in_y) {
                    if (!st->p.periodic[1]) continue;
                    gj = ((gj % noy) + noy) % noy;
                }
                *at(g, i, j) = *at(g, gi + HALO, gj + HALO);
            }
    }
}

/* ------------------------------------------------------------------ */
/* Interpolation: src/Interpolation.hpp:30-54, which builds Cajita
 * SplineData and calls evaluateSpline + G2P::value.  Restated: the logical
 * coordinate of a point relative to entity index 0 of the ghosted local
 * mesh is xi = (x - x_E(0)) / dx; order 1 uses stencil {k, k+1} with
 * weights {1-t, t}; order 3 is the uniform cubic B-spline on {k-1..k+2}
 * with t = xi - k.  The sum is evaluated separably (rows along x first).
 * Positions beyond the ghosted array are clamped to its edge (the
 * reference reads out of bounds there). */
static inline double entity_coord(const orc_state* st, int ent, int axis, int idx) {
    double t = (double)idx + ENT_OFF[ent][axis];
    return st->gl[axis] + t * st->dx;
}

static void weights(int order, double xi, int ext, int* k0, double* w) {
    if (order == 1) {
        xi = fmin(fmax(xi, 0.0), (double)(ext - 1));
        int k = (int)xi;
        if (k > ext - 2) k = ext - 2;
        double t = xi - (double)k;
        w[0] = 1.0 - t;
        w[1] = t;
        *k0 = k;
    } else {
        xi = fmin(fmax(xi, 1.0), (double)(ext - 2));
        int k = (int)xi;
        if (k > ext - 3) k = ext - 3;
        double t = xi - (double)k;
        double s = 1.0 - t;
        double t2 = t * t;
        double t3 = t2 * t;
        double s3 = (s * s) * s;
        w[0] = s3 * (1.0 / 6.0);
        w[1] = fma(0.5, t3, -t2) + (2.0 / 3.0);
        w[2] = fma(0.5, (t + t2) - t3, 1.0 / 6.0);
        w[3] = t3 * (1.0 / 6.0);
        *k0 = k - 1;
    }
}

static double sample_grid(const orc_state* st, const grid_t* g, int ent, int order,
                          double x, double y) {
    double lx = entity_coord(st, ent, 0, 0), ly = entity_coord(st, ent, 1, 0);
    double xi = (x - lx) * st->rdx;
    double yi = (y - ly) * st->rdx;
    int kx, ky;
    double wx[4], wy[4];
    weights(order, xi, g->ex, &kx, wx);
    weights(order, yi, g->ey, &ky, wy);
    int n = order == 1 ? 2 : 4;
    double val = 0.0;
    for (int b = 0; b < n; ++b) {
        const double* row = at(g, kx, ky + b);
        double rs = wx[0] * row[0];
        for (int a = 1; a < n; ++a) rs = fma(wx[a], row[a], rs);
        val = (b == 0) ? wy[0] * rs : fma(wy[b], rs, val);
    }
    return val;
}

/* RK3 backtrace: src/TimeIntegrator.hpp:36-77.  The x2 stage uses v0
 * (quirk Q3) unless quirk bit 1 selects Ralston's v1. */
static void rk3_trace(const orc_state* st, double dt, const double x0[2], double tr[2]) {
    const grid_t* u = &st->f[ORC_U][0];
    const grid_t* v = &st->f[ORC_V][0];
    double v0[2], v1[2], v2[2], x1[2], x2[2];
    v0[0] = sample_grid(st, u, E_FACEI, 1, x0[0], x0[1]);
    v0[1] = sample_grid(st, v, E_FACEJ, 1, x0[0], x0[1]);
    /* the reference's expressions as written, one rounding per operation:
     * x0 - 0.5 * dt * v0 parses as x0 - ((0.5 * dt) * v0) (:48-49) */
    double h1 = 0.5 * dt;
    x1[0] = x0[0] - h1 * v0[0];
    x1[1] = x0[1] - h1 * v0[1];
    v1[0] = sample_grid(st, u, E_FACEI, 1, x1[0], x1[1]);
    v1[1] = sample_grid(st, v, E_FACEJ, 1, x1[0], x1[1]);
    double h2 = 0.75 * dt;
    const double* vs = (st->p.quirks & 2u) ? v1 : v0;
    x2[0] = x0[0] - h2 * vs[0];
    x2[1] = x0[1] - h2 * vs[1];
    v2[0] = sample_grid(st, u, E_FACEI, 1, x2[0], x2[1]);
    v2[1] = sample_grid(st, v, E_FACEJ, 1, x2[0], x2[1]);
    /* x0 - dt * ((2/9) v0 + (3/9) v1 + (4/9) v2), summed left to right (:62-65) */
    for (int d = 0; d < 2; ++d) {
        double a = (2.0 / 9.0) * v0[d] + (3.0 / 9.0) * v1[d];
        a = a + (4.0 / 9.0) * v2[d];
        tr[d] = x0[d] - dt * a;
    }
}

/* TimeIntegrator::step: gather, advect q/u/v from Current into Next, swap
 * (src/TimeIntegrator.hpp:81-116, 120-177).  The final sample has order
 * value_order (the reference uses 3). */
void orc_advect_step(orc_state* st, double dt, int value_order) {
    orc_fill_ghosts(st);
    static const int ent_of[3] = {E_CELL, E_FACEI, E_FACEJ};
    for (int fld = 0; fld < 3; ++fld) {
        const grid_t* cur = &st->f[fld][0];
        grid_t* nxt = &st->f[fld][1];
        int ox = owned_count(st, fld, 0), oy = owned_count(st, fld, 1);
        int ent = ent_of[fld];
#pragma omp parallel for schedule(static)
        for (int j = 0; j < oy; ++j)
            for (int i = 0; i < ox; ++i) {
                double x0[2], tr[2];
                x0[0] = entity_coord(st, ent, 0, i + HALO);
                x0[1] = entity_coord(st, ent, 1, j + HALO);
                rk3_trace(st, dt, x0, tr);
                *at(nxt, i + HALO, j + HALO) = sample_grid(st, cur, ent, value_order, tr[0], tr[1]);
            }
    }
    for (int fld = 0; fld < 3; ++fld) {
        grid_t t = st->f[fld][0];
        st->f[fld][0] = st->f[fld][1];
        st->f[fld][1] = t;
    }
}

/* ------------------------------------------------------------------ */
/* Solver::_addInputs (src/Solver.hpp:181-263) with InflowSource
 * (src/InflowSource.hpp:33-77), BodyForce (src/BodyForce.hpp:44-60) and
 * the face wall conditions (src/BoundaryConditions.hpp:102-129). */
static inline int in_box(const orc_params* p, double x, double y) {
    return x >= p->src_bbox[0] && x < p->src_bbox[2] && y >= p->src_bbox[1] &&
           y < p->src_bbox[3];
}

static double cell_value(const orc_state* st, int gi, int gj) {
    int nx = st->p.nx, ny = st->p.ny;
    if (gi < 0 || gi >= nx) {
        if (!st->p.periodic[0]) return 0.0;
        gi = ((gi % nx) + nx) % nx;
    }
    if (gj < 0 || gj >= ny) {
        if (!st->p.periodic[1]) return 0.0;
        gj = ((gj % ny) + ny) % ny;
    }
    return *at(&st->f[ORC_Q][0], gi + HALO, gj + HALO);
}

void orc_add_inputs(orc_state* st, double dt) {
    const orc_params* p = &st->p;
    grid_t* q = &st->f[ORC_Q][0];
    grid_t* u = &st->f[ORC_U][0];
    grid_t* v = &st->f[ORC_V][0];
    int nx = p->nx, ny = p->ny;
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = 0; gi < nx; ++gi) {
            double x = entity_coord(st, E_CELL, 0, gi + HALO);
            double y = entity_coord(st, E_CELL, 1, gj + HALO);
            double* qq = at(q, gi + HALO, gj + HALO);
            if (in_box(p, x, y)) {
                if (p->src_mode == 0) {
                    if (*qq < p->src_quantity) *qq = p->src_quantity;
                } else {
                    *qq = *qq + p->src_quantity * dt; /* rate form (extension) */
                }
            }
        }
    int oxu = owned_count(st, ORC_U, 0);
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = 0; gi < oxu; ++gi) {
            double x = entity_coord(st, E_FACEI, 0, gi + HALO);
            double y = entity_coord(st, E_FACEI, 1, gj + HALO);
            double* uu = at(u, gi + HALO, gj + HALO);
            if (in_box(p, x, y) && fabs(*uu) < fabs(p->src_velocity[0])) *uu = p->src_velocity[0];
            /* ux += _force[0] * delta_t (src/BodyForce.hpp:52); the
             * density-scaled form (extension) scales the force first */
            if (p->body_density_scaled) {
                double rho = (cell_value(st, gi - 1, gj) + cell_value(st, gi, gj)) * 0.5;
                *uu = *uu + (p->body_force[0] * rho) * dt;
            } else {
                *uu = *uu + p->body_force[0] * dt;
            }
            if (!p->periodic[0]) {
                if (gi <= 0 && p->bc_type[0] == SOLID) *uu = 0.0;
                if (gi > nx - 1 && p->bc_type[2] == SOLID) *uu = 0.0;
            }
        }
    int oyv = owned_count(st, ORC_V, 1);
    for (int gj = 0; gj < oyv; ++gj)
        for (int gi = 0; gi < nx; ++gi) {
            double x = entity_coord(st, E_FACEJ, 0, gi + HALO);
            double y = entity_coord(st, E_FACEJ, 1, gj + HALO);
            double* vv = at(v, gi + HALO, gj + HALO);
            if (in_box(p, x, y) && fabs(*vv) < fabs(p->src_velocity[1])) *vv = p->src_velocity[1];
            if (p->body_density_scaled) {
                double rho = (cell_value(st, gi, gj - 1) + cell_value(st, gi, gj)) * 0.5;
                *vv = *vv + (p->body_force[1] * rho) * dt;
            } else {
                *vv = *vv + p->body_force[1] * dt; /* src/BodyForce.hpp:61 */
            }
            if (!p->periodic[1]) {
                if (gj <= 0 && p->bc_type[1] == SOLID) *vv = 0.0;
                if (gj > ny - 1 && p->bc_type[3] == SOLID) *vv = 0.0;
            }
        }
}

/* ------------------------------------------------------------------ */
/* Canonical dot product (see the header comment of this file). */
static double fold32(double* s) {
    double tmp[32];
    for (int m = 16; m >= 1; m >>= 1) {
        for (int l = 0; l < 32; ++l) tmp[l] = s[l] + s[l ^ m];
        memcpy(s, tmp, sizeof(tmp));
    }
    return s[0];
}

static double final_tree(const double* partial, int n) {
    double s[FINAL_THREADS];
    for (int t = 0; t < FINAL_THREADS; ++t) {
        s[t] = 0.0;
        for (int u = t; u < n; u += FINAL_THREADS) s[t] = s[t] + partial[u];
    }
    double w[FINAL_THREADS / 32];
    for (int k = 0; k < FINAL_THREADS / 32; ++k) w[k] = fold32(s + 32 * k);
    double tot = w[0];
    for (int k = 1; k < FINAL_THREADS / 32; ++k) tot = tot + w[k];
    return tot;
}

static double canon_dot_buf(int nx, int ny, const double* a, const double* b, double* partial) {
    int G = (nx + UNIT_COLS - 1) / UNIT_COLS;
    int B = (ny + BAND_ROWS - 1) / BAND_ROWS;
    int U = G * B;
#pragma omp parallel for schedule(static)
    for (int u = 0; u < U; ++u) {
        int g = u % G, band = u / G;
        double lane[32];
        for (int l = 0; l < 32; ++l) lane[l] = 0.0;
        int j1 = (band + 1) * BAND_ROWS;
        if (j1 > ny) j1 = ny;
        for (int j = band * BAND_ROWS; j < j1; ++j) {
            const double* ar = a + (size_t)j * nx;
            const double* br = b + (size_t)j * nx;
            for (int l = 0; l < 32; ++l) {
                int c = g * UNIT_COLS + 2 * l;
                if (c < nx) lane[l] = fma(ar[c], br[c], lane[l]);
                if (c + 1 < nx) lane[l] = fma(ar[c + 1], br[c + 1], lane[l]);
            }
        }
        partial[u] = fold32(lane);
    }
    return final_tree(partial, U);
}

double orc_canonical_dot(int nx, int ny, const double* a, const double* b) {
    int G = (nx + UNIT_COLS - 1) / UNIT_COLS;
    int B = (ny + BAND_ROWS - 1) / BAND_ROWS;
    double* partial = (double*)malloc(sizeof(double) * (size_t)G * B);
    double r = canon_dot_buf(nx, ny, a, b, partial);
    free(partial);
    return r;
}

/* ------------------------------------------------------------------ */
/* Projection: VelocityCorrector (src/VelocityCorrector.hpp). */

/* Matrix diagonal: initializeMatrixValues + BoundaryCondition::build_matrix
 * (src/VelocityCorrector.hpp:116-144, src/BoundaryConditions.hpp:57-97).
 * Off-diagonal legs are -scale; a leg that leaves a wall side reads a zero
 * pressure ghost, which is what the reference's zeroed leg gives. */
static void build_diag(orc_state* st, double dt) {
    const orc_params* p = &st->p;
    int nx = p->nx, ny = p->ny;
    double scale = dt / ((p->density * st->dx) * st->dx);
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = 0; gi < nx; ++gi) {
            double c0 = 4.0 * scale;
            if (!p->periodic[0]) {
                if (gi <= 0 && p->bc_type[0] == SOLID) c0 = c0 - scale;
                if (gi > nx - 2 && p->bc_type[2] == SOLID) c0 = c0 - scale;
            }
            if (!p->periodic[1]) {
                if (gj <= 0 && p->bc_type[1] == SOLID) c0 = c0 - scale;
                if (gj > ny - 2 && p->bc_type[3] == SOLID) c0 = c0 - scale;
            }
            st->diag[(size_t)gj * nx + gi] = c0;
            st->minv[(size_t)gj * nx + gi] = p->precon_none ? 1.0 : 1.0 / c0; /* :174-179 */
        }
}

static inline double vec_at(const orc_state* st, const double* a, int gi, int gj) {
    int nx = st->p.nx, ny = st->p.ny;
    if (gi < 0 || gi >= nx) {
        if (!st->p.periodic[0]) return 0.0;
        gi = gi < 0 ? gi + nx : gi - nx;
    }
    if (gj < 0 || gj >= ny) {
        if (!st->p.periodic[1]) return 0.0;
        gj = gj < 0 ? gj + ny : gj - ny;
    }
    return a[(size_t)gj * nx + gi];
}

/* q = A p with the 5-point stencil {C, W, E, S, N}
 * (src/VelocityCorrector.hpp:96-98). */
static void matvec(const orc_state* st, double scale, const double* pv, double* qv) {
    int nx = st->p.nx, ny = st->p.ny;
    double ms = -1.0 * scale;
#pragma omp parallel for schedule(static)
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = 0; gi < nx; ++gi) {
            size_t k = (size_t)gj * nx + gi;
            double acc = st->diag[k] * pv[k];
            acc = fma(ms, vec_at(st, pv, gi - 1, gj), acc);
            acc = fma(ms, vec_at(st, pv, gi + 1, gj), acc);
            acc = fma(ms, vec_at(st, pv, gi, gj - 1), acc);
            acc = fma(ms, vec_at(st, pv, gi, gj + 1), acc);
            qv[k] = acc;
        }
}

void orc_matvec(const orc_state* st, double dt, const double* p, double* q) {
    build_diag((orc_state*)st, dt);
    double scale = dt / ((st->p.density * st->dx) * st->dx);
    matvec(st, scale, p, q);
}

/* _buildRHS: b = -(1/dx) (u(i+1) - u(i) + v(j+1) - v(j))
 * (src/VelocityCorrector.hpp:182-212). */
static void divergence(const orc_state* st, double* b) {
    int nx = st->p.nx, ny = st->p.ny;
    const grid_t* u = &st->f[ORC_U][0];
    const grid_t* v = &st->f[ORC_V][0];
    double scale = 1.0 / st->dx;
#pragma omp parallel for schedule(static)
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = 0; gi < nx; ++gi) {
            int ie = gi + 1, jn = gj + 1;
            if (st->p.periodic[0] && ie == nx) ie = 0;
            if (st->p.periodic[1] && jn == ny) jn = 0;
            double u0 = *at(u, gi + HALO, gj + HALO), u1 = *at(u, ie + HALO, gj + HALO);
            double v0 = *at(v, gi + HALO, gj + HALO), v1 = *at(v, gi + HALO, jn + HALO);
            double t = u1 - u0;
            t = t + v1;
            t = t - v0;
            b[(size_t)gj * nx + gi] = -scale * t;
        }
}

void orc_div_norms(const orc_state* st, double* l2, double* linf) {
    int nx = st->p.nx, ny = st->p.ny;
    size_t n = (size_t)nx * ny;
    double* b = (double*)malloc(sizeof(double) * n);
    divergence(st, b);
    double ss = orc_canonical_dot(nx, ny, b, b);
    double mx = 0.0;
    for (size_t k = 0; k < n; ++k) mx = fmax(mx, fabs(b[k]));
    *l2 = sqrt(ss) * st->dx;
    *linf = mx;
    free(b);
}

/* _applyPressure (src/VelocityCorrector.hpp:214-264), including quirk Q1:
 * the J-face boundary condition is applied to the u array (:260). */
static void apply_pressure(orc_state* st, double dt) {
    const orc_params* p = &st->p;
    int nx = p->nx, ny = p->ny;
    double scale = dt / (p->density * st->dx);
    grid_t* u = &st->f[ORC_U][0];
    grid_t* v = &st->f[ORC_V][0];
    int oxu = owned_count(st, ORC_U, 0);
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = 0; gi < oxu; ++gi) {
            double d = vec_at(st, st->x, gi, gj) - vec_at(st, st->x, gi - 1, gj);
            double* uu = at(u, gi + HALO, gj + HALO);
            *uu = *uu - scale * d; /* u -= scale * (p(i) - p(i-1)), :245 */
            if (!p->periodic[0]) {
                if (gi <= 0 && p->bc_type[0] == SOLID) *uu = 0.0;
                if (gi > nx - 1 && p->bc_type[2] == SOLID) *uu = 0.0;
            }
        }
    int oyv = owned_count(st, ORC_V, 1);
    int fix_q1 = (p->quirks & 1u) != 0;
    for (int gj = 0; gj < oyv; ++gj)
        for (int gi = 0; gi < nx; ++gi) {
            double d = vec_at(st, st->x, gi, gj) - vec_at(st, st->x, gi, gj - 1);
            double* vv = at(v, gi + HALO, gj + HALO);
            *vv = *vv - scale * d; /* :256 */
            if (p->periodic[1]) continue;
            /* the J-face condition, applied to u (reference) or v (fixed) */
            double* tgt = fix_q1 ? vv : at(u, gi + HALO, gj + HALO);
            if (gj <= 0 && p->bc_type[1] == SOLID) *tgt = 0.0;
            if (gj > ny - 1 && p->bc_type[3] == SOLID) *tgt = 0.0;
        }
}

/* ------------------------------------------------------------------ */
/* Geometric multigrid V-cycle preconditioner: the stand-in for the HYPRE
 * PFMG/SMG preconditioners the reference selects by name
 * (src/VelocityCorrector.hpp:324-338; PFMG is the CLI default,
 * examples/advection.cpp:186-189).  Cell-centred levels halve both axes
 * while both are even and at least 16; level l uses the fine stencil with
 * scale / 4^l and the same wall rules.  Smoother: red-black Gauss-Seidel,
 * MG_NU sweeps red-then-black before and black-then-red after the coarse
 * correction; MG_NC such sweep pairs on the coarsest level.  Prolongation:
 * cell-centred bilinear (3/4, 1/4 per axis; a SOLID wall reflects, a FREE
 * wall reads zero, a periodic axis wraps); restriction: its transpose / 4.
 * The cycle is a symmetric operator, as CG needs. */
#define MG_MAX 16
#define MG_NU 2
#define MG_NC 8

typedef struct {
    int nx, ny;
    double scale, ms;
    double diag[16], invd[16];
    double *x, *b, *r;
} mg_level;

static int mg_bits(const orc_params* p, int nx, int ny, int gi, int gj) {
    int b = 0;
    if (!p->periodic[0]) b |= (gi == 0 ? 1 : 0) | (gi == nx - 1 ? 2 : 0);
    if (!p->periodic[1]) b |= (gj == 0 ? 4 : 0) | (gj == ny - 1 ? 8 : 0);
    return b;
}

static double mg_at(const orc_params* p, const double* a, int nx, int ny, int gi, int gj) {
    if (gi < 0 || gi >= nx) {
        if (!p->periodic[0]) return 0.0;
        gi = gi < 0 ? gi + nx : gi - nx;
    }
    if (gj < 0 || gj >= ny) {
        if (!p->periodic[1]) return 0.0;
        gj = gj < 0 ? gj + ny : gj - ny;
    }
    return a[(size_t)gj * nx + gi];
}

/* per-axis weight of coarse index I in the prolongation to fine index f */
static double mg_pw(int f, int I, int nc, int per, int bclo, int bchi) {
    int parent = f >> 1, nb = parent + ((f & 1) ? 1 : -1);
    int nb_in = nb >= 0 && nb < nc;
    if (!nb_in && per) {
        nb = nb < 0 ? nb + nc : nb - nc;
        nb_in = 1;
    }
    double wp = 0.75;
    if (!nb_in && (nb < 0 ? bclo : bchi) == SOLID) wp = 1.0;
    double w = 0.0;
    if (parent == I) w = w + wp;
    if (nb_in && nb == I) w = w + 0.25;
    return w;
}

static void mg_smooth(const orc_params* p, mg_level* L, int color) {
    int nx = L->nx, ny = L->ny;
#pragma omp parallel for schedule(static)
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = (gj + color) & 1; gi < nx; gi += 2) {
            double s = mg_at(p, L->x, nx, ny, gi - 1, gj) + mg_at(p, L->x, nx, ny, gi + 1, gj);
            s = s + mg_at(p, L->x, nx, ny, gi, gj - 1);
            s = s + mg_at(p, L->x, nx, ny, gi, gj + 1);
            size_t k = (size_t)gj * nx + gi;
            double t = fma(L->scale, s, L->b[k]);
            L->x[k] = t * L->invd[mg_bits(p, nx, ny, gi, gj)];
        }
}

static void mg_residual(const orc_params* p, mg_level* L) {
    int nx = L->nx, ny = L->ny;
#pragma omp parallel for schedule(static)
    for (int gj = 0; gj < ny; ++gj)
        for (int gi = 0; gi < nx; ++gi) {
            size_t k = (size_t)gj * nx + gi;
            double ax = L->diag[mg_bits(p, nx, ny, gi, gj)] * L->x[k];
            ax = fma(L->ms, mg_at(p, L->x, nx, ny, gi - 1, gj), ax);
            ax = fma(L->ms, mg_at(p, L->x, nx, ny, gi + 1, gj), ax);
            ax = fma(L->ms, mg_at(p, L->x, nx, ny, gi, gj - 1), ax);
            ax = fma(L->ms, mg_at(p, L->x, nx, ny, gi, gj + 1), ax);
            L->r[k] = L->b[k] - ax;
        }
}

static void mg_restrict(const orc_params* p, const mg_level* F, mg_level* C) {
    int nfx = F->nx, nfy = F->ny, ncx = C->nx, ncy = C->ny;
#pragma omp parallel for schedule(static)
    for (int J = 0; J < ncy; ++J)
        for (int I = 0; I < ncx; ++I) {
            double acc = 0.0;
            for (int fy0 = 2 * J - 1; fy0 <= 2 * J + 2; ++fy0) {
                int fy = fy0;
                if (fy < 0 || fy >= nfy) {
                    if (!p->periodic[1]) continue;
                    fy = fy < 0 ? fy + nfy : fy - nfy;
                }
                double wy = mg_pw(fy, J, ncy, p->periodic[1], p->bc_type[1], p->bc_type[3]);
                double rs = 0.0;
                for (int fx0 = 2 * I - 1; fx0 <= 2 * I + 2; ++fx0) {
                    int fx = fx0;
                    if (fx < 0 || fx >= nfx) {
                        if (!p->periodic[0]) continue;
                        fx = fx < 0 ? fx + nfx : fx - nfx;
                    }
                    double wx = mg_pw(fx, I, ncx, p->periodic[0], p->bc_type[0], p->bc_type[2]);
                    rs = fma(wx, F->r[(size_t)fy * nfx + fx], rs);
                }
                acc = fma(wy, rs, acc);
            }
            C->b[(size_t)J * ncx + I] = 0.25 * acc;
        }
}

/* neighbour coarse index and weights along one axis for fine index f */
static void mg_axis(int f, int nc, int per, int bclo, int bchi, int* I, int* N, double* wI, double* wN) {
    int parent = f >> 1, nb = parent + ((f & 1) ? 1 : -1);
    *I = parent;
    *wI = 0.75;
    *wN = 0.25;
    if (nb < 0 || nb >= nc) {
        if (per) {
            nb = nb < 0 ? nb + nc : nb - nc;
        } else {
            if ((nb < 0 ? bclo : bchi) == SOLID) *wI = 1.0;
            nb = -1;
            *wN = 0.0;
        }
    }
    *N = nb;
}

static void mg_prolong_add(const orc_params* p, const mg_level* C, mg_level* F) {
    int nfx = F->nx, nfy = F->ny, ncx = C->nx, ncy = C->ny;
#pragma omp parallel for schedule(static)
    for (int fy = 0; fy < nfy; ++fy)
        for (int fx = 0; fx < nfx; ++fx) {
            int I, NI, J, NJ;
            double wxI, wxN, wyJ, wyN;
            mg_axis(fx, ncx, p->periodic[0], p->bc_type[0], p->bc_type[2], &I, &NI, &wxI, &wxN);
            mg_axis(fy, ncy, p->periodic[1], p->bc_type[1], p->bc_type[3], &J, &NJ, &wyJ, &wyN);
            double row0 = wxI * C->x[(size_t)J * ncx + I];
            if (NI >= 0) row0 = fma(wxN, C->x[(size_t)J * ncx + NI], row0);
            double v = wyJ * row0;
            if (NJ >= 0) {
                double row1 = wxI * C->x[(size_t)NJ * ncx + I];
                if (NI >= 0) row1 = fma(wxN, C->x[(size_t)NJ * ncx + NI], row1);
                v = fma(wyN, row1, v);
            }
            size_t k = (size_t)fy * nfx + fx;
            F->x[k] = F->x[k] + v;
        }
}

static void mg_vcycle(const orc_params* p, mg_level* lev, int nlev, int l) {
    mg_level* L = &lev[l];
    memset(L->x, 0, sizeof(double) * (size_t)L->nx * L->ny);
    if (l == nlev - 1) {
        for (int s = 0; s < MG_NC; ++s) {
            mg_smooth(p, L, 0);
            mg_smooth(p, L, 1);
        }
        for (int s = 0; s < MG_NC; ++s) {
            mg_smooth(p, L, 1);
            mg_smooth(p, L, 0);
        }
        return;
    }
    for (int s = 0; s < MG_NU; ++s) {
        mg_smooth(p, L, 0);
        mg_smooth(p, L, 1);
    }
    mg_residual(p, L);
    mg_restrict(p, L, &lev[l + 1]);
    mg_vcycle(p, lev, nlev, l + 1);
    mg_prolong_add(p, &lev[l + 1], L);
    for (int s = 0; s < MG_NU; ++s) {
        mg_smooth(p, L, 1);
        mg_smooth(p, L, 0);
    }
}

static void mg_level_tables(const orc_params* p, mg_level* L) {
    for (int b = 0; b < 16; ++b) {
        double d = 4.0 * L->scale;
        if ((b & 1) && p->bc_type[0] == SOLID) d = d - L->scale;
        if ((b & 2) && p->bc_type[2] == SOLID) d = d - L->scale;
        if ((b & 4) && p->bc_type[1] == SOLID) d = d - L->scale;
        if ((b & 8) && p->bc_type[3] == SOLID) d = d - L->scale;
        L->diag[b] = d;
        L->invd[b] = 1.0 / d;
    }
    L->ms = -1.0 * L->scale;
}

/* levels for this grid; level 0 works in place on r (rhs) and z (result) */
static int mg_build(orc_state* st, double scale, mg_level* lev) {
    int nx = st->p.nx, ny = st->p.ny, n = 0;
    for (;;) {
        mg_level* L = &lev[n];
        L->nx = nx;
        L->ny = ny;
        L->scale = n == 0 ? scale : lev[n - 1].scale * 0.25;
        mg_level_tables(&st->p, L);
        size_t cells = (size_t)nx * ny;
        if (n == 0) {
            L->b = st->r;
            L->x = st->z;
            L->r = st->qv;  /* scratch: free while the V-cycle runs */
        } else {
            L->b = (double*)calloc(cells, sizeof(double));
            L->x = (double*)calloc(cells, sizeof(double));
            L->r = (double*)calloc(cells, sizeof(double));
        }
        ++n;
        /* halve while both axes are even and >= 16 and the halved extent
         * stays even along periodic axes (no same-colour neighbours across
         * the wrap, so each half sweep is independent of its order) */
        if (n == MG_MAX || (nx & 1) || (ny & 1) || nx < 16 || ny < 16) break;
        if ((st->p.periodic[0] && ((nx / 2) & 1)) || (st->p.periodic[1] && ((ny / 2) & 1))) break;
        nx /= 2;
        ny /= 2;
    }
    return n;
}

static void mg_free(mg_level* lev, int n) {
    for (int l = 1; l < n; ++l) {
        free(lev[l].b);
        free(lev[l].x);
        free(lev[l].r);
    }
}

/* MG-preconditioned CG: the same recurrences as below with z = V-cycle(r);
 * the V-cycle is skipped once the loop is about to stop. */
static int project_mg(orc_state* st, double scale, double tol, double abs_tol, int max_iter, int* iters,
                      double* bb_out, double* rr_out) {
    int nx = st->p.nx, ny = st->p.ny;
    size_t n = (size_t)nx * ny;
    double area = st->dx * st->dx;
    mg_level lev[MG_MAX];
    int nlev = mg_build(st, scale, lev);
    double rr = canon_dot_buf(nx, ny, st->r, st->r, st->partial);
    double bb = canon_dot_buf(nx, ny, st->rhs, st->rhs, st->partial), rho = 0.0, beta = 0.0;
    double tol2 = tol * tol, abs2 = abs_tol * abs_tol;
    int k = 0, status = 0;
#define MG_CONVERGED(rr) ((rr) <= tol2 * bb || (abs_tol > 0.0 && (rr) * area <= abs2))
    if (bb != 0.0 && !MG_CONVERGED(rr) && max_iter > 0) {
        mg_vcycle(&st->p, lev, nlev, 0);
        rho = canon_dot_buf(nx, ny, st->r, st->z, st->partial);
    }
    if (bb != 0.0) {
        for (;;) {
            if (MG_CONVERGED(rr)) { status = 0; break; }
            if (k >= max_iter) { status = 1; break; }
#pragma omp parallel for schedule(static)
            for (size_t c = 0; c < n; ++c) st->pv[c] = (k == 0) ? st->z[c] : fma(beta, st->pv[c], st->z[c]);
            matvec(st, scale, st->pv, st->qv);
            double pq = canon_dot_buf(nx, ny, st->pv, st->qv, st->partial);
            if (!(pq > 0.0)) { status = isnan(pq) ? 3 : 2; break; }
            double alpha = rho / pq, malpha = -alpha;
#pragma omp parallel for schedule(static)
            for (size_t c = 0; c < n; ++c) {
                st->x[c] = fma(alpha, st->pv[c], st->x[c]);
                st->r[c] = fma(malpha, st->qv[c], st->r[c]);
            }
            rr = canon_dot_buf(nx, ny, st->r, st->r, st->partial);
            k += 1;
            if (isnan(rr)) { status = 3; break; }
            if (MG_CONVERGED(rr) || k >= max_iter) continue;
            mg_vcycle(&st->p, lev, nlev, 0);
            double rho_new = canon_dot_buf(nx, ny, st->r, st->z, st->partial);
            beta = rho_new / rho;
            rho = rho_new;
        }
    }
#undef MG_CONVERGED
    mg_free(lev, nlev);
    *iters = k;
    *bb_out = bb;
    *rr_out = rr;
    return status;
}

/* test export: z = one V-cycle applied to r at time step dt; returns the
 * number of levels */
int orc_mg_apply(orc_state* st, double dt, const double* r, double* z) {
    size_t n = (size_t)st->p.nx * st->p.ny;
    double scale = dt / ((st->p.density * st->dx) * st->dx);
    mg_level lev[MG_MAX];
    int nlev = mg_build(st, scale, lev);
    memcpy(st->r, r, n * sizeof(double));
    mg_vcycle(&st->p, lev, nlev, 0);
    memcpy(z, st->z, n * sizeof(double));
    mg_free(lev, nlev);
    return nlev;
}

/* Jacobi-preconditioned CG, cold start x0 = 0 (src/VelocityCorrector.hpp:
 * 158-180, 266-282; Cajita ReferenceConjugateGradient restated).  Stops
 * when ||r||^2 <= tol^2 ||b||^2, or ||r||^2 dx^2 <= abs_tol^2 when
 * abs_tol > 0, checked before each iteration. */
/* initial residual: cold start x0 = 0, r = b (src/VelocityCorrector.hpp:272);
 * warm start (extension) keeps x from the previous solve, r = b - A x */
static void initial_residual(orc_state* st, double scale) {
    size_t n = (size_t)st->p.nx * st->p.ny;
    if (st->p.warm_start) {
        matvec(st, scale, st->x, st->qv);
        for (size_t k = 0; k < n; ++k) st->r[k] = st->rhs[k] - st->qv[k];
    } else {
        for (size_t k = 0; k < n; ++k) {
            st->r[k] = st->rhs[k];
            st->x[k] = 0.0;
        }
    }
}

int orc_project(orc_state* st, double dt, double tol, double abs_tol, int max_iter,
                orc_solve_stats* stats) {
    if (st->p.precon_mg) {
        double scale = dt / ((st->p.density * st->dx) * st->dx);
        build_diag(st, dt);
        divergence(st, st->rhs);
        initial_residual(st, scale);
        int iters = 0;
        double bb = 0.0, rr = 0.0;
        int status = project_mg(st, scale, tol, abs_tol, max_iter, &iters, &bb, &rr);
        apply_pressure(st, dt);
        if (stats) {
            stats->iterations = iters;
            stats->status = status;
            stats->bb = bb;
            stats->rr = rr;
            orc_div_norms(st, &stats->div_l2, &stats->div_linf);
        }
        return status;
    }
    int nx = st->p.nx, ny = st->p.ny;
    size_t n = (size_t)nx * ny;
    double scale = dt / ((st->p.density * st->dx) * st->dx);
    double area = st->dx * st->dx;
    build_diag(st, dt);
    divergence(st, st->rhs);
    initial_residual(st, scale);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) st->z[k] = st->minv[k] * st->r[k];
    double rho = canon_dot_buf(nx, ny, st->r, st->z, st->partial);
    double rr = canon_dot_buf(nx, ny, st->r, st->r, st->partial);
    double bb = canon_dot_buf(nx, ny, st->rhs, st->rhs, st->partial);
    double beta = 0.0;
    int k = 0, status = 0;
    double tol2 = tol * tol, abs2 = abs_tol * abs_tol;
    if (bb != 0.0) {
        for (;;) {
            if (rr <= tol2 * bb || (abs_tol > 0.0 && rr * area <= abs2)) { status = 0; break; }
            if (k >= max_iter) { status = 1; break; }
#pragma omp parallel for schedule(static)
            for (size_t c = 0; c < n; ++c) {
                double zc = st->minv[c] * st->r[c];
                st->pv[c] = (k == 0) ? zc : fma(beta, st->pv[c], zc);
            }
            matvec(st, scale, st->pv, st->qv);
            double pq = canon_dot_buf(nx, ny, st->pv, st->qv, st->partial);
            if (!(pq > 0.0)) { status = isnan(pq) ? 3 : 2; break; }
            double alpha = rho / pq;
            double malpha = -alpha;
#pragma omp parallel for schedule(static)
            for (size_t c = 0; c < n; ++c) {
                st->x[c] = fma(alpha, st->pv[c], st->x[c]);
                st->r[c] = fma(malpha, st->qv[c], st->r[c]);
                st->z[c] = st->minv[c] * st->r[c];
            }
            double rho_new = canon_dot_buf(nx, ny, st->r, st->z, st->partial);
            rr = canon_dot_buf(nx, ny, st->r, st->r, st->partial);
            beta = rho_new / rho;
            rho = rho_new;
            k += 1;
            if (isnan(rr)) { status = 3; break; }
        }
    }
    apply_pressure(st, dt);
    if (stats) {
        stats->iterations = k;
        stats->status = status;
        stats->bb = bb;
        stats->rr = rr;
        orc_div_norms(st, &stats->div_l2, &stats->div_linf);
    }
    return status;
}

/* Solver::step: advect, add inputs, correct velocity (src/Solver.hpp:135-147). */
int orc_step(orc_state* st, double dt, int value_order, double tol, double abs_tol,
             int max_iter, orc_solve_stats* stats) {
    orc_advect_step(st, dt, value_order);
    orc_add_inputs(st, dt);
    return orc_project(st, dt, tol, abs_tol, max_iter, stats);
}

/* ------------------------------------------------------------------ */
/* test exports */
void orc_sample(const orc_state* st, int field, int order, int n, const double* xy, double* out) {
    static const int ent_of[3] = {E_CELL, E_FACEI, E_FACEJ};
    for (int k = 0; k < n; ++k)
        out[k] = sample_grid(st, &st->f[field][0], ent_of[field], order, xy[2 * k], xy[2 * k + 1]);
}

void orc_trace(const orc_state* st, int n, const double* xy, double dt, double* out) {
    for (int k = 0; k < n; ++k) rk3_trace(st, dt, xy + 2 * k, out + 2 * k);
}
