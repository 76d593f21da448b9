// Hand-written adjoint of Solver::step (FP64) with sqrt(N)-style
// checkpointing: cf_forward_checkpointed / cf_backward.
//
// Forward step (src/Solver.hpp:135-147): s_k = (q, u, v) ->
//   A  advection   (q_a, u_a, v_a) = Adv(q, u, v)         src/TimeIntegrator.hpp:36-177
//   I  inputs      rate source q += Q dt in the box, wall masks on faces
//                                                          src/Solver.hpp:181-263
//   P  projection  u_p = M u_i + (s'/dx) M G A^-1 D u_i   src/VelocityCorrector.hpp:182-264
// Reverse step, given the adjoint lambda_{k+1}:
//   P^T w = M w + (s'/dx) G A^-1 D (M w)   (G = -D^T exactly and A is
//           symmetric, so the transpose is the same pipeline with the mask
//           applied first and none at the end; one more PCG solve)
//   I^T     wall masks; dL/dQ += dt * sum over the box of the quantity adjoint
//   A^T     transpose of the spline samples and of the RK3 trace:
//           pass 1 (one thread per target entity) recomputes the trace and
//           writes scatter records -- stencil start plus weights already
//           multiplied by the value to scatter -- for the advected field and
//           for the velocity taps of the three RK3 stages;
//           pass 2 (one thread per destination entity) gathers, in a fixed
//           order, every record whose stencil covers it, from target slots
//           within 3 indices.  No floating-point atomics: the result is
//           deterministic.  The window holds while no trace or stage moves
//           more than one cell in a step (the reference's own assumption,
//           src/ProblemManager.hpp:167-172); pass 1 checks it and the call
//           returns CF_ERR_UNSUPPORTED otherwise.
//           Along periodic axes the adjoint that lands on ghosts is folded
//           back onto the owned entity each ghost copies; wall ghosts are
//           constants and drop out.
// Supported: FP64 contexts; the rate-form quantity source with zero inflow
// velocity; constant body forces; the projection with CF_FIX_Q1 whenever a
// y-wall is SOLID (the quirk's projection has an inconsistent adjoint
// right-hand side).  Other settings return CF_ERR_UNSUPPORTED.
#include <cuda_runtime.h>
#include <math.h>

#include <cstring>
#include <string>
#include <vector>

#include "cf_ctx.cuh"

namespace cf {

static __constant__ double ADJ_OFF[3][2] = {{0.5, 0.5}, {0.0, 0.5}, {0.5, 0.0}};

struct RecKind {
    int2* base;   // stencil start on the destination grid (local ghosted index)
    double* cx;   // x weights times the scattered value, cx[a * nt + t]
    double* wy;   // y weights, wy[b * nt + t]
    int n;        // weights per axis (2 or 4)
    int nt, tex;  // target slots and target grid x extent
};

struct Samp {
    int kx, ky;
    double wx[4], wy[4];
    double val, gx, gy;
};

// Weights, derivative weights and the sample value / gradient, in the same
// arithmetic as the forward sample (cf_fields.cu; clamps, integer parts and
// int-to-double conversions on the integer pipe, exact).
template <int ORDER>
__device__ void samp(const Grid<double>& g, double lx, double ly, double rdx, double x, double y, Samp& s) {
    constexpr int n = ORDER == 1 ? 2 : 4;
    double xi[2] = {(x - lx) * rdx, (y - ly) * rdx};
    int ext[2] = {g.ex, g.ey};
    double w[2][4], dw[2][4];
    int k0[2];
    bool clamped[2];
    for (int d = 0; d < 2; ++d) {
        double v = xi[d];
        if (ORDER == 1) {
            double lo = 0.0, hi = exact_double(ext[d] - 1);
            clamped[d] = outside_bits(v, lo, hi);
            v = clamp_bits(v, lo, hi);
            int k = trunc_bits(v);
            if (k > ext[d] - 2) k = ext[d] - 2;
            double t = v - exact_double(k);
            w[d][0] = 1.0 - t;
            w[d][1] = t;
            dw[d][0] = -1.0;
            dw[d][1] = 1.0;
            k0[d] = k;
        } else {
            double lo = 1.0, hi = exact_double(ext[d] - 2);
            clamped[d] = outside_bits(v, lo, hi);
            v = clamp_bits(v, lo, hi);
            int k = trunc_bits(v);
            if (k > ext[d] - 3) k = ext[d] - 3;
            double t = v - exact_double(k);
            double sm = 1.0 - t, t2 = t * t, t3 = t2 * t, s3 = (sm * sm) * sm;
            w[d][0] = s3 * (1.0 / 6.0);
            w[d][1] = fma(0.5, t3, -t2) + (2.0 / 3.0);
            w[d][2] = fma(0.5, (t + t2) - t3, 1.0 / 6.0);
            w[d][3] = t3 * (1.0 / 6.0);
            dw[d][0] = -0.5 * sm * sm;
            dw[d][1] = 1.5 * t2 - 2.0 * t;
            dw[d][2] = -1.5 * t2 + t + 0.5;
            dw[d][3] = 0.5 * t2;
            k0[d] = k - 1;
        }
    }
    double val = 0.0, gx = 0.0, gy = 0.0;
    for (int b = 0; b < n; ++b) {
        const double* row = g.o + (size_t)(k0[1] + b) * g.pitch + k0[0];
        double rs = 0.0, rd = 0.0;
        for (int a = 0; a < n; ++a) {
            double f = row[a];
            rs = fma(w[0][a], f, rs);
            rd = fma(dw[0][a], f, rd);
        }
        val = fma(w[1][b], rs, val);
        gx = fma(w[1][b], rd, gx);
        gy = fma(dw[1][b], rs, gy);
    }
    s.kx = k0[0];
    s.ky = k0[1];
    for (int a = 0; a < n; ++a) {
        s.wx[a] = w[0][a];
        s.wy[a] = w[1][a];
    }
    s.val = val;
    s.gx = clamped[0] ? 0.0 : gx * rdx;
    s.gy = clamped[1] ? 0.0 : gy * rdx;
}

struct AdjRec {
    Phys p;
    Grid<double> q, u, v;     // forward state of the step (ghosts filled)
    Grid<double> aq, au, av;  // adjoint of the advected values
    double dt;
    int order;
    RecKind F[3], Su[3][3], Sv[3][3];
    int* err;
};

__device__ __forceinline__ void put_rec(const RecKind& R, int t, int kx, int ky, double val, const double* wx,
                                        const double* wy, int n) {
    R.base[t] = make_int2(kx, ky);
    for (int a = 0; a < n; ++a) {
        R.cx[a * R.nt + t] = val * wx[a];
        R.wy[a * R.nt + t] = wy[a];
    }
}

// pass 1: one thread per owned target entity (blockIdx.z = entity type)
__global__ void k_adj_records(AdjRec a) {
    const Phys& p = a.p;
    const int ent = blockIdx.z;
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    const int ox = p.nx + ((ent == E_FACEI && !p.per_x) ? 1 : 0);
    const int oy = p.ny + ((ent == E_FACEJ && !p.per_y) ? 1 : 0);
    if (gi >= ox || gj >= oy) return;
    const int li = gi + CF_HALO, lj = gj + CF_HALO;
    const Grid<double>& f = ent == E_CELL ? a.q : (ent == E_FACEI ? a.u : a.v);
    const Grid<double>& fa = ent == E_CELL ? a.aq : (ent == E_FACEI ? a.au : a.av);
    const int t = lj * f.ex + li;
    const double fbar = fa.at(li, lj);
    const double x0 = p.gl[0] + ((double)li + ADJ_OFF[ent][0]) * p.dx;
    const double y0 = p.gl[1] + ((double)lj + ADJ_OFF[ent][1]) * p.dx;
    const double dt = a.dt;
    // forward trace (src/TimeIntegrator.hpp:36-77)
    Samp s0u, s0v, s1u, s1v, s2u, s2v, sf;
    const double ulx = p.low[E_FACEI][0], uly = p.low[E_FACEI][1];
    const double vlx = p.low[E_FACEJ][0], vly = p.low[E_FACEJ][1];
    samp<1>(a.u, ulx, uly, p.rdx, x0, y0, s0u);
    samp<1>(a.v, vlx, vly, p.rdx, x0, y0, s0v);
    const double h1 = 0.5 * dt, h2 = 0.75 * dt;
    // the forward's operation order (one rounding per operation)
    double x1 = __dsub_rn(x0, __dmul_rn(h1, s0u.val)), y1 = __dsub_rn(y0, __dmul_rn(h1, s0v.val));
    samp<1>(a.u, ulx, uly, p.rdx, x1, y1, s1u);
    samp<1>(a.v, vlx, vly, p.rdx, x1, y1, s1v);
    const bool ralston = (p.quirks & 2u) != 0;
    double sx = ralston ? s1u.val : s0u.val, sy = ralston ? s1v.val : s0v.val;
    double x2 = __dsub_rn(x0, __dmul_rn(h2, sx)), y2 = __dsub_rn(y0, __dmul_rn(h2, sy));
    samp<1>(a.u, ulx, uly, p.rdx, x2, y2, s2u);
    samp<1>(a.v, vlx, vly, p.rdx, x2, y2, s2v);
    double ax = __dadd_rn(__dmul_rn(2.0 / 9.0, s0u.val), __dmul_rn(3.0 / 9.0, s1u.val));
    ax = __dadd_rn(ax, __dmul_rn(4.0 / 9.0, s2u.val));
    double ay = __dadd_rn(__dmul_rn(2.0 / 9.0, s0v.val), __dmul_rn(3.0 / 9.0, s1v.val));
    ay = __dadd_rn(ay, __dmul_rn(4.0 / 9.0, s2v.val));
    double tx = __dsub_rn(x0, __dmul_rn(dt, ax)), ty = __dsub_rn(y0, __dmul_rn(dt, ay));
    if (a.order == 1)
        samp<1>(f, p.low[ent][0], p.low[ent][1], p.rdx, tx, ty, sf);
    else
        samp<3>(f, p.low[ent][0], p.low[ent][1], p.rdx, tx, ty, sf);
    // the gather window assumes every position moved at most one cell
    double lim = p.dx;
    if (fabs(tx - x0) > lim || fabs(ty - y0) > lim || fabs(x1 - x0) > lim || fabs(y1 - y0) > lim ||
        fabs(x2 - x0) > lim || fabs(y2 - y0) > lim)
        atomicOr(a.err, 1);
    // reverse
    put_rec(a.F[ent], t, sf.kx, sf.ky, fbar, sf.wx, sf.wy, a.order == 1 ? 2 : 4);
    double tbx = fbar * sf.gx, tby = fbar * sf.gy;
    double abx = -dt * tbx, aby = -dt * tby;
    double v0x = (2.0 / 9.0) * abx, v0y = (2.0 / 9.0) * aby;
    double v1x = (3.0 / 9.0) * abx, v1y = (3.0 / 9.0) * aby;
    double v2x = (4.0 / 9.0) * abx, v2y = (4.0 / 9.0) * aby;
    // stage 2 at (x2, y2)
    put_rec(a.Su[ent][2], t, s2u.kx, s2u.ky, v2x, s2u.wx, s2u.wy, 2);
    put_rec(a.Sv[ent][2], t, s2v.kx, s2v.ky, v2y, s2v.wx, s2v.wy, 2);
    double x2bx = s2u.gx * v2x + s2v.gx * v2y, x2by = s2u.gy * v2x + s2v.gy * v2y;
    if (ralston) {
        v1x -= h2 * x2bx;
        v1y -= h2 * x2by;
    } else {
        v0x -= h2 * x2bx;
        v0y -= h2 * x2by;
    }
    // stage 1 at (x1, y1)
    put_rec(a.Su[ent][1], t, s1u.kx, s1u.ky, v1x, s1u.wx, s1u.wy, 2);
    put_rec(a.Sv[ent][1], t, s1v.kx, s1v.ky, v1y, s1v.wx, s1v.wy, 2);
    double x1bx = s1u.gx * v1x + s1v.gx * v1y, x1by = s1u.gy * v1x + s1v.gy * v1y;
    v0x -= h1 * x1bx;
    v0y -= h1 * x1by;
    // stage 0 at (x0, y0)
    put_rec(a.Su[ent][0], t, s0u.kx, s0u.ky, v0x, s0u.wx, s0u.wy, 2);
    put_rec(a.Sv[ent][0], t, s0v.kx, s0v.ky, v0y, s0v.wx, s0v.wy, 2);
}

struct AdjGather {
    Grid<double> out;
    RecKind k[10];
    int nk;
};

// pass 2: one thread per destination entity (ghosted index space)
__global__ void k_adj_gather(AdjGather a) {
    const int di = blockIdx.x * blockDim.x + threadIdx.x;
    const int dj = blockIdx.y * blockDim.y + threadIdx.y;
    if (di >= a.out.ex || dj >= a.out.ey) return;
    double acc = 0.0;
    for (int k = 0; k < a.nk; ++k) {
        const RecKind& R = a.k[k];
        const int tey = R.nt / R.tex;
        const int j0 = max(dj - 3, 0), j1 = min(dj + 3, tey - 1);
        const int i0 = max(di - 3, 0), i1 = min(di + 3, R.tex - 1);
        for (int tj = j0; tj <= j1; ++tj)
            for (int ti = i0; ti <= i1; ++ti) {
                const int t = tj * R.tex + ti;
                const int2 b = R.base[t];
                const int ox = di - b.x, oy = dj - b.y;
                if ((unsigned)ox < (unsigned)R.n && (unsigned)oy < (unsigned)R.n)
                    acc = fma(R.cx[ox * R.nt + t], R.wy[oy * R.nt + t], acc);
            }
    }
    a.out.at(di, dj) = acc;
}

// periodic axes: add the adjoint that landed on ghost copies to the owned entity
__global__ void k_adj_fold(Grid<double> g, int nox, int noy, int per_x, int per_y) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nox || gj >= noy) return;
    double acc = g.at(gi + CF_HALO, gj + CF_HALO);
    for (int ky = -1; ky <= 1; ++ky)
        for (int kx = -1; kx <= 1; ++kx) {
            if (kx == 0 && ky == 0) continue;
            if ((kx && !per_x) || (ky && !per_y)) continue;
            int li = gi + CF_HALO + kx * nox, lj = gj + CF_HALO + ky * noy;
            if (li < 0 || lj < 0 || li >= g.ex || lj >= g.ey) continue;
            acc = acc + g.at(li, lj);
        }
    g.at(gi + CF_HALO, gj + CF_HALO) = acc;
}

// wall masks on faces: axis 0 zeroes u at SOLID x-walls, axis 1 v at SOLID y-walls
__global__ void k_adj_mask(Phys p, Grid<double> u, Grid<double> v) {
    const int axis = blockIdx.z;
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (axis == 0) {
        if (p.per_x || gj >= p.ny) return;
        if (gi == 0 && p.bc[0] == 0) u.at(CF_HALO, gj + CF_HALO) = 0.0;
        if (gi == 1 && p.bc[2] == 0) u.at(p.nx + CF_HALO, gj + CF_HALO) = 0.0;
    } else {
        if (p.per_y || gi >= p.nx) return;
        if (gj == 0 && p.bc[1] == 0) v.at(gi + CF_HALO, CF_HALO) = 0.0;
        if (gj == 1 && p.bc[3] == 0) v.at(gi + CF_HALO, p.ny + CF_HALO) = 0.0;
    }
}

// dL/d(rate) += dt * (sum of the quantity adjoint over the inflow box's
// cells).  One block: the box's cells (local index ranges the host found
// with the forward's coordinate test) in row-major order, thread t taking
// cells t, t + 256, ...; then a fixed-order block sum, so the result is
// deterministic.
constexpr int kBoxThreads = 256;
__global__ void __launch_bounds__(kBoxThreads) k_adj_rate(Phys p, Grid<double> aq, double dt, double* rbar) {
    const int i0 = p.box[E_CELL][0], i1 = p.box[E_CELL][1], j0 = p.box[E_CELL][2], j1 = p.box[E_CELL][3];
    const int w = i1 - i0, n = w > 0 && j1 > j0 ? w * (j1 - j0) : 0;
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += kBoxThreads) s = s + aq.at(i0 + k % w, j0 + k / w);
    __shared__ double ws[kBoxThreads / 32];
    s = warp_fold(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = ws[0];
        for (int k = 1; k < kBoxThreads / 32; ++k) t = t + ws[k];
        *rbar += dt * t;
    }
}

// host side

static void* grid_base(const Grid<double>& g) { return (void*)(g.o - (32 - CF_HALO)); }
static size_t grid_bytes(const Grid<double>& g) { return (size_t)g.pitch * g.ey * sizeof(double); }

struct AdjState {
    bool ready = false;
    int nsteps = 0, every = 0, order = 3;
    double dt = 0.0;
    cf_solver_opts opts{};
    std::string solver, precon;
    std::vector<double*> ckpt;  // each: q, u, v grids back to back
    std::vector<double*> seg;
    double* final_state = nullptr;
    Grid<double> ag[3]{}, bg[3]{};  // adjoint grids (current and gather output)
    RecKind F[3], Su[3][3], Sv[3][3];
    int* d_err = nullptr;
    double* d_rows = nullptr;
    double* d_rbar = nullptr;  // dL/d(rate), accumulated on the device
    double* xa = nullptr;      // the adjoint pressure between reverse steps (the warm start)
    // the forward pass left the last segment's states in seg: the backward's
    // first segment needs no recomputation (cleared once seg is reused)
    bool last_seg_valid = false;
    std::vector<void*> allocs;
};

}  // namespace cf

using namespace cf;

namespace {

size_t state_bytes(cf_ctx* c) { return grid_bytes(c->q64[0]) + grid_bytes(c->u[0]) + grid_bytes(c->v[0]); }

int dalloc(cf_ctx* c, AdjState* A, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(c, CF_ERR_NOMEM, "adjoint: cudaMalloc of %zu bytes failed", bytes);
    A->allocs.push_back(*p);
    return CF_OK;
}

int save_state(cf_ctx* c, double* dst) {
    char* d = (char*)dst;
    const Grid<double>* gs[3] = {&c->q64[c->cur], &c->u[c->cur], &c->v[c->cur]};
    for (auto* g : gs) {
        cudaError_t e = cudaMemcpyAsync(d, grid_base(*g), grid_bytes(*g), cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return cuda_check(c, e, "checkpoint save");
        d += grid_bytes(*g);
    }
    return CF_OK;
}

int load_state(cf_ctx* c, const double* src) {
    const char* s = (const char*)src;
    const Grid<double>* gs[3] = {&c->q64[c->cur], &c->u[c->cur], &c->v[c->cur]};
    for (auto* g : gs) {
        cudaError_t e = cudaMemcpyAsync(grid_base(*g), s, grid_bytes(*g), cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return cuda_check(c, e, "checkpoint load");
        s += grid_bytes(*g);
    }
    return CF_OK;
}

AdjState* adj(cf_ctx* c) { return static_cast<AdjState*>(c->adjoint); }

int check_supported(cf_ctx* c) {
    // a recomputed segment must repeat the forward exactly; a warm start
    // would depend on a pressure the checkpoints do not hold
    if (c->warm) return fail(c, CF_ERR_UNSUPPORTED, "the adjoint needs cold-started projections (warm start is on)");
    const Phys& p = c->ph;
    if (c->precision != CF_PREC_FP64) return fail(c, CF_ERR_UNSUPPORTED, "the adjoint runs on FP64 contexts");
    bool src_active = p.bbox[2] > p.bbox[0] && p.bbox[3] > p.bbox[1];
    if (src_active && p.src_mode == 0 && p.src_q != 0.0)
        return fail(c, CF_ERR_UNSUPPORTED, "adjoint of the clamp-form quantity source (use the rate form)");
    if (src_active && (p.src_vel[0] != 0.0 || p.src_vel[1] != 0.0))
        return fail(c, CF_ERR_UNSUPPORTED, "adjoint of a velocity inflow");
    if (p.force_density) return fail(c, CF_ERR_UNSUPPORTED, "adjoint of a density-scaled body force");
    if (!(p.quirks & CF_FIX_Q1) && !p.per_y && (p.bc[1] == CF_BC_SOLID || p.bc[3] == CF_BC_SOLID))
        return fail(c, CF_ERR_UNSUPPORTED, "adjoint of the Q1 projection quirk (set CF_FIX_Q1)");
    return CF_OK;
}

int setup_records(cf_ctx* c, AdjState* A) {
    if (A->ag[0].o) return CF_OK;
    int rc = CF_OK;
    // adjoint grids share the field layout
    const Grid<double>* shapes[3] = {&c->q64[0], &c->u[0], &c->v[0]};
    for (int k = 0; k < 3 && !rc; ++k)
        for (int w = 0; w < 2 && !rc; ++w) {
            Grid<double>& g = w == 0 ? A->ag[k] : A->bg[k];
            void* base = nullptr;
            rc = dalloc(c, A, &base, grid_bytes(*shapes[k]));
            if (rc) break;
            cudaMemsetAsync(base, 0, grid_bytes(*shapes[k]), c->stream);
            g = *shapes[k];
            g.o = (double*)base + (32 - CF_HALO);
        }
    auto mk = [&](RecKind& R, int ent, int n) {
        const Grid<double>& tg = *shapes[ent];
        R.n = n;
        R.tex = tg.ex;
        R.nt = tg.ex * tg.ey;
        void *b = nullptr, *x = nullptr, *y = nullptr;
        if (!rc) rc = dalloc(c, A, &b, sizeof(int2) * R.nt);
        if (!rc) rc = dalloc(c, A, &x, sizeof(double) * n * R.nt);
        if (!rc) rc = dalloc(c, A, &y, sizeof(double) * n * R.nt);
        if (rc) return;
        cudaMemsetAsync(b, 0x80, sizeof(int2) * R.nt, c->stream);  // empty slots: far-away stencil start
        R.base = (int2*)b;
        R.cx = (double*)x;
        R.wy = (double*)y;
    };
    for (int e = 0; e < 3; ++e) {
        mk(A->F[e], e, 4);
        for (int s = 0; s < 3; ++s) {
            mk(A->Su[e][s], e, 2);
            mk(A->Sv[e][s], e, 2);
        }
    }
    if (!rc) rc = dalloc(c, A, (void**)&A->d_err, sizeof(int));
    if (!rc) rc = dalloc(c, A, (void**)&A->d_rows, sizeof(double) * (c->ph.ny + 1));
    if (!rc) rc = dalloc(c, A, (void**)&A->d_rbar, sizeof(double));
    if (!rc) rc = dalloc(c, A, (void**)&A->xa, sizeof(double) * (size_t)c->vpitch * c->ph.ny);
    return rc;
}

// One reverse step, enqueued without a synchronisation: the transposed
// projection (deferred through its resident graph when that serves it;
// non-convergence and failures are tallied on the device), the inputs'
// transpose with dL/d(rate) accumulated on the device, and the advection's
// transpose (a trace that moved too far sets the device error flag).
int adjoint_step(cf_ctx* c, AdjState* A, const SolveOpts& so, bool params_ready) {
    const Phys& p = c->ph;
    dim3 blk(32, 8);
    int rc;
    // P^T: mask, then the projection pipeline without the final mask
    k_adj_mask<<<dim3((p.nx + 2 + 31) / 32, (p.ny + 2 + 7) / 8, 2), blk, 0, c->stream>>>(p, A->ag[1], A->ag[2]);
    // the solve starts from the previous reverse step's adjoint pressure
    // (zero for the first), kept in A->xa between steps because the
    // forward recomputation reuses the solver's solution vector
    const size_t xbytes = sizeof(double) * (size_t)c->vpitch * p.ny;
    if ((rc = cuda_check(c, cudaMemcpyAsync(c->x.a, A->xa, xbytes, cudaMemcpyDeviceToDevice, c->stream), "adjoint x")))
        return rc;
    SolveResult res{};
    bool deferred = false;
    if ((rc = project_adjoint_async(c, A->dt, so, &res, &deferred, params_ready, A->ag[1], A->ag[2]))) return rc;
    if (!deferred && res.status != ST_CONVERGED && res.status != ST_MAXIT)
        return fail(c, CF_ERR_NUMERIC, "adjoint projection failed (status %d)", res.status);
    if ((rc = cuda_check(c, cudaMemcpyAsync(A->xa, c->x.a, xbytes, cudaMemcpyDeviceToDevice, c->stream), "adjoint x")))
        return rc;
    // I^T: wall masks of the inputs; dL/dQ from the rate source
    k_adj_mask<<<dim3((p.nx + 2 + 31) / 32, (p.ny + 2 + 7) / 8, 2), blk, 0, c->stream>>>(p, A->ag[1], A->ag[2]);
    bool src_active = p.bbox[2] > p.bbox[0] && p.bbox[3] > p.bbox[1];
    if (src_active && p.src_mode == 1) {
        k_adj_rate<<<1, kBoxThreads, 0, c->stream>>>(p, A->ag[0], A->dt, A->d_rbar);
        c->launches += 1;
    }
    // A^T at the forward state of this step (already loaded)
    if ((rc = cuda_check(c, launch_fill_ghosts(c), "fill ghosts"))) return rc;
    for (int e = 0; e < 3; ++e) A->F[e].n = A->order == 1 ? 2 : 4;
    AdjRec ar;
    ar.p = p;
    ar.q = c->q64[c->cur];
    ar.u = c->u[c->cur];
    ar.v = c->v[c->cur];
    ar.aq = A->ag[0];
    ar.au = A->ag[1];
    ar.av = A->ag[2];
    ar.dt = A->dt;
    ar.order = A->order;
    for (int e = 0; e < 3; ++e) {
        ar.F[e] = A->F[e];
        for (int s = 0; s < 3; ++s) {
            ar.Su[e][s] = A->Su[e][s];
            ar.Sv[e][s] = A->Sv[e][s];
        }
    }
    ar.err = A->d_err;
    k_adj_records<<<dim3((p.nx + 1 + 31) / 32, (p.ny + 1 + 7) / 8, 3), blk, 0, c->stream>>>(ar);
    for (int gsel = 0; gsel < 3; ++gsel) {
        AdjGather ag{};
        ag.out = A->bg[gsel];
        if (gsel == 0) {
            ag.k[0] = A->F[0];
            ag.nk = 1;
        } else {
            ag.k[0] = A->F[gsel];
            int m = 1;
            for (int e = 0; e < 3; ++e)
                for (int s = 0; s < 3; ++s) ag.k[m++] = gsel == 1 ? A->Su[e][s] : A->Sv[e][s];
            ag.nk = m;
        }
        k_adj_gather<<<dim3((ag.out.ex + 31) / 32, (ag.out.ey + 7) / 8), blk, 0, c->stream>>>(ag);
        int nox = p.nx + ((gsel == 1 && !p.per_x) ? 1 : 0);
        int noy = p.ny + ((gsel == 2 && !p.per_y) ? 1 : 0);
        if (p.per_x || p.per_y)
            k_adj_fold<<<dim3((nox + 31) / 32, (noy + 7) / 8), blk, 0, c->stream>>>(A->bg[gsel], nox, noy, p.per_x,
                                                                                     p.per_y);
        std::swap(A->ag[gsel], A->bg[gsel]);
    }
    c->launches += 6 + (p.per_x || p.per_y ? 3 : 0);
    return cuda_check(c, cudaGetLastError(), "adjoint advection");
}

// The device tally of a run of enqueued projections: a solve that broke
// down, produced NaN or timed out fails the call (one that stopped at
// max_iter is tolerated, as cf_step's callers here tolerate it).
int check_tally(cf_ctx* c, const int* tally, const char* what) {
    if (tally[0] == 0 || tally[1] == ST_MAXIT) return CF_OK;
    return fail(c, tally[1] == ST_TIMEOUT ? CF_ERR_TIMEOUT : CF_ERR_NUMERIC, "%s: a pressure solve failed (status %d)",
                what, tally[1]);
}

// owned region of an adjoint grid <-> contiguous host array
int adj_io(cf_ctx* c, Grid<double>& g, int field, double* host, bool to_host) {
    int ox = c->ph.nx, oy = c->ph.ny;
    if (field == CF_FIELD_U && !c->ph.per_x) ox += 1;
    if (field == CF_FIELD_V && !c->ph.per_y) oy += 1;
    cudaError_t e = to_host ? cudaMemcpy2DAsync(host, ox * sizeof(double), &g.at(CF_HALO, CF_HALO),
                                                g.pitch * sizeof(double), ox * sizeof(double), oy,
                                                cudaMemcpyDeviceToHost, c->stream)
                            : cudaMemcpy2DAsync(&g.at(CF_HALO, CF_HALO), g.pitch * sizeof(double), host,
                                                ox * sizeof(double), ox * sizeof(double), oy,
                                                cudaMemcpyHostToDevice, c->stream);
    return cuda_check(c, e, "adjoint copy");
}

}  // namespace

extern "C" {

int cf_forward_checkpointed(cf_ctx* ctx, int nsteps, int ckpt_every, double dt, int value_order,
                            const cf_solver_opts* opts, cf_solve_stats* last) {
    if (!ctx) return CF_ERR_INVALID;
    if (nsteps <= 0 || ckpt_every <= 0 || !(dt > 0.0) || (value_order != 1 && value_order != 3))
        return fail(ctx, CF_ERR_INVALID, "bad forward_checkpointed arguments");
    if (ctx->precision != CF_PREC_FP64) return fail(ctx, CF_ERR_UNSUPPORTED, "the adjoint runs on FP64 contexts");
    if (ctx->warm)
        return fail(ctx, CF_ERR_UNSUPPORTED, "the adjoint needs cold-started projections (warm start is on)");
    cudaSetDevice(ctx->device);
    if (!ctx->adjoint) ctx->adjoint = new AdjState();
    AdjState* A = adj(ctx);
    int nck = (nsteps + ckpt_every - 1) / ckpt_every;
    size_t sb = state_bytes(ctx);
    int rc = CF_OK;
    // (re)allocate checkpoint storage when the schedule grows
    if ((int)A->ckpt.size() < nck || (int)A->seg.size() < ckpt_every || !A->final_state) {
        while ((int)A->ckpt.size() < nck && !rc) {
            void* p = nullptr;
            rc = dalloc(ctx, A, &p, sb);
            A->ckpt.push_back((double*)p);
        }
        while ((int)A->seg.size() < ckpt_every && !rc) {
            void* p = nullptr;
            rc = dalloc(ctx, A, &p, sb);
            A->seg.push_back((double*)p);
        }
        if (!A->final_state && !rc) rc = dalloc(ctx, A, (void**)&A->final_state, sb);
        if (rc) return rc;
    }
    A->nsteps = nsteps;
    A->every = ckpt_every;
    A->dt = dt;
    A->order = value_order;
    A->solver = (opts && opts->solver) ? opts->solver : "PCG";
    A->precon = (opts && opts->precon) ? opts->precon : "Diagonal";
    if (opts) A->opts = *opts;
    else {
        A->opts = cf_solver_opts{};
        A->opts.tol = 1e-6;
        A->opts.max_iter = 2000;
    }
    A->opts.solver = A->solver.c_str();
    A->opts.precon = A->precon.c_str();
    A->ready = false;
    SolveOpts so{};
    if ((rc = parse_solver_opts(ctx, &A->opts, &so))) return rc;
    // the steps go back to back on the stream (checkpoint copies between
    // them), one synchronisation at the end
    rc = cuda_check(ctx, cudaMemsetAsync(ctx->d_tally, 0, 3 * sizeof(int), ctx->stream), "tally");
    SolveResult r{};
    bool deferred = false;
    // the last segment's states also go to the segment buffers, so the
    // backward starts its reverse sweep without recomputing them
    const int k_last = (nck - 1) * ckpt_every;
    for (int k = 0; k < nsteps && !rc; ++k) {
        if (k % ckpt_every == 0) rc = save_state(ctx, A->ckpt[k / ckpt_every]);
        if (!rc && k >= k_last) rc = save_state(ctx, A->seg[k - k_last]);
        if (!rc) rc = enqueue_step(ctx, dt, value_order, so, &r, &deferred, k > 0);
        if (!rc && !deferred && r.status != ST_CONVERGED && r.status != ST_MAXIT)
            rc = fail(ctx, CF_ERR_NUMERIC, "pressure solve failed (status %d)", r.status);
    }
    if (!rc) rc = save_state(ctx, A->final_state);
    int tally[3] = {0, 0, 0};
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpyAsync(tally, ctx->d_tally, sizeof(tally), cudaMemcpyDeviceToHost, ctx->stream),
                        "tally");
    const int rc1 = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "forward");
    if (rc) return rc;
    if (rc1) return rc1;
    if (deferred) project_collect(ctx, &r, nsteps, tally[2]);
    if ((rc = check_tally(ctx, tally, "forward"))) return rc;
    A->ready = true;
    A->last_seg_valid = true;
    if (last) {
        *last = cf_solve_stats{};
        last->iterations = r.iterations;
        last->outer_iterations = r.outer;
        last->status = r.status;
        last->b_norm = sqrt(r.bb);
        last->r_norm = sqrt(r.rr);
        last->div_l2 = r.div_l2;
        last->div_linf = r.div_linf;
    }
    return CF_OK;
}

int cf_backward(cf_ctx* ctx, const double* dL_dq_T, const double* dL_du_T, const double* dL_dv_T, double* dL_dq0,
                double* dL_du0, double* dL_dv0, double* dL_drate) {
    if (!ctx) return CF_ERR_INVALID;
    AdjState* A = adj(ctx);
    if (!A || !A->ready) return fail(ctx, CF_ERR_INVALID, "cf_backward needs a preceding cf_forward_checkpointed");
    cudaSetDevice(ctx->device);
    int rc = check_supported(ctx);
    if (!rc) rc = setup_records(ctx, A);
    if (rc) return rc;
    SolveOpts so{};
    so.tol = A->opts.tol;
    so.abs_tol = 0.0;  // the adjoint right-hand side has its own scale
    so.max_iter = A->opts.max_iter;
    so.inner_tol = 0.1;
    so.max_outer = 200;
    so.precon_none = (!strcmp(A->precon.c_str(), "None") || !strcmp(A->precon.c_str(), "none")) ? 1 : 0;
    so.precon_mg = (A->precon == "PFMG" || A->precon == "SMG" || A->precon == "MG") ? 1 : 0;
    if (!(so.tol > 0.0)) so.tol = 1e-12;
    // lambda_T
    for (int k = 0; k < 3; ++k) cudaMemsetAsync(grid_base(A->ag[k]), 0, grid_bytes(A->ag[k]), ctx->stream);
    const double* seeds[3] = {dL_dq_T, dL_du_T, dL_dv_T};
    const int fields[3] = {CF_FIELD_QUANTITY, CF_FIELD_U, CF_FIELD_V};
    for (int k = 0; k < 3 && !rc; ++k)
        if (seeds[k]) rc = adj_io(ctx, A->ag[k], fields[k], const_cast<double*>(seeds[k]), false);
    if (rc) return rc;
    // the forward recomputation, the checkpoint copies and the reverse steps
    // are all enqueued; one synchronisation at the end reads the tally of
    // the pressure solves, the trace check and dL/d(rate)
    SolveOpts fo{};
    if ((rc = parse_solver_opts(ctx, &A->opts, &fo))) return rc;
    cudaMemsetAsync(ctx->d_tally, 0, 3 * sizeof(int), ctx->stream);
    cudaMemsetAsync(A->d_err, 0, sizeof(int), ctx->stream);
    cudaMemsetAsync(A->d_rbar, 0, sizeof(double), ctx->stream);
    cudaMemsetAsync(A->xa, 0, sizeof(double) * (size_t)ctx->vpitch * ctx->ph.ny, ctx->stream);
    ctx->adj_warm = 1;
    const int C = A->every, T = A->nsteps;
    const int nseg = (T + C - 1) / C;
    SolveResult r{};
    bool deferred = false, fwd_params = false, adj_params = false;
    for (int sg = nseg - 1; sg >= 0 && !rc; --sg) {
        const int k0 = sg * C, k1 = (k0 + C < T) ? k0 + C : T;
        const bool stored = sg == nseg - 1 && A->last_seg_valid;
        A->last_seg_valid = false;  // seg is about to be reused
        if (!stored) rc = load_state(ctx, A->ckpt[sg]);
        for (int k = k0; k < k1 && !rc && !stored; ++k) {
            rc = save_state(ctx, A->seg[k - k0]);
            if (!rc && k < k1 - 1) {
                rc = enqueue_step(ctx, A->dt, A->order, fo, &r, &deferred, fwd_params);
                fwd_params = true;
                if (!rc && !deferred && r.status != ST_CONVERGED && r.status != ST_MAXIT)
                    rc = fail(ctx, CF_ERR_NUMERIC, "pressure solve failed (status %d)", r.status);
            }
        }
        for (int k = k1 - 1; k >= k0 && !rc; --k) {
            rc = load_state(ctx, A->seg[k - k0]);
            if (!rc) rc = adjoint_step(ctx, A, so, adj_params);
            adj_params = true;
        }
    }
    int tally[3] = {0, 0, 0}, herr = 0;
    double rbar = 0.0;
    if (!rc) {
        cudaMemcpyAsync(tally, ctx->d_tally, sizeof(tally), cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(&herr, A->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(&rbar, A->d_rbar, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    }
    const int rc1 = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "backward");
    ctx->adj_warm = 0;
    if (rc) return rc;
    if (rc1) return rc1;
    if ((rc = check_tally(ctx, tally, "backward"))) return rc;
    if (herr)
        return fail(ctx, CF_ERR_UNSUPPORTED, "adjoint: a trace moved more than one cell in a step (reduce dt)");
    if (dL_dq0) rc = adj_io(ctx, A->ag[0], CF_FIELD_QUANTITY, dL_dq0, true);
    if (!rc && dL_du0) rc = adj_io(ctx, A->ag[1], CF_FIELD_U, dL_du0, true);
    if (!rc && dL_dv0) rc = adj_io(ctx, A->ag[2], CF_FIELD_V, dL_dv0, true);
    if (!rc) rc = load_state(ctx, A->final_state);
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "backward");
    if (!rc && dL_drate) *dL_drate = rbar;
    return rc;
}

}  // extern "C"

void cf_adjoint_free(cf_ctx* c) {
    AdjState* A = static_cast<AdjState*>(c->adjoint);
    if (!A) return;
    for (void* p : A->allocs) cudaFree(p);
    delete A;
    c->adjoint = nullptr;
}
