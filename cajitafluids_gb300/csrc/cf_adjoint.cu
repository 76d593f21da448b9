// Hand-written adjoint of Solver::step (FP64) with sqrt(N)-style
// checkpointing: cf_forward_checkpointed / cf_backward.
//
// Forward step (src/Solver.hpp:135-147): s_k = (q, u, v) ->
//   A  advection   (q_a, u_a, v_a) = Adv(q, u, v)         src/TimeIntegrator.hpp:36-177
//   I  inputs      quantity source (rate q += Q dt, or clamp q = max(q, Q)) in
//                  the box, velocity inflow, body force, wall masks on faces
//                                                          src/Solver.hpp:181-263
//   P  projection  u_p = M u_i + (s'/dx) M G A^-1 D u_i   src/VelocityCorrector.hpp:182-264
// Reverse step, given the adjoint lambda_{k+1}:
//   P^T w = M w + (s'/dx) G A^-1 D (M w)   (G = -D^T exactly and A is
//           symmetric, so the transpose is the same pipeline with the mask
//           applied first and none at the end; one more PCG solve)
//   I^T     wall masks; the density-scaled force's coupling into the quantity
//           adjoint; dL/dQ += dt * sum over the box of the quantity adjoint
//           (rate form); the replacing inputs (clamp, velocity inflow) are
//           transposed inside A^T, which recomputes the advected value
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
// Mixed contexts (FP32 bulk): the checkpoints hold the mixed state (FP32 q,
// velocity pairs), the recomputation repeats the mixed forward bit for bit,
// the transposed projection runs the mixed PCG on the adjoint face arrays
// held as pairs, and the advection's transpose runs in FP32 without records
// (k_adj_advect32: the forward's FP32 trace recomputed, contributions
// gathered through a register window per warp, deterministic).
// Supported: FP64 and mixed contexts; the quantity source in either form
// (rate: dL/dQ from the box's adjoint; clamp q = max(q, Q): no adjoint flows
// through the cells where the clamp fired, dL/dQ collects it there); the
// velocity inflow (the faces it overwrote pass no adjoint back; the inflow
// velocity itself gets no gradient); constant and density-scaled body forces
// (the latter couples the face adjoints into the quantity's); the projection
// with CF_FIX_Q1 whenever a y-wall is SOLID.  With the quirk the projected
// wall-normal v keeps a value that depends on the constant mode of the
// pressure, which the PCG leaves to its iteration, so the forward map has no
// well-defined derivative there (CF_ERR_UNSUPPORTED).
#include <cuda_runtime.h>
#include <math.h>

#include <cstring>
#include <string>
#include <vector>

#include "cf_adv32.cuh"
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
    double* qclamp;  // clamp-form source: per box cell, the adjoint where the clamp fired, else 0
};

__device__ __forceinline__ void put_rec(const RecKind& R, int t, int kx, int ky, double val, const double* wx,
                                        const double* wy, int n) {
    R.base[t] = make_int2(kx, ky);
    for (int a = 0; a < n; ++a) {
        R.cx[a * R.nt + t] = val * wx[a];
        R.wy[a * R.nt + t] = wy[a];
    }
}

// The adjoint of an advected value through the inputs that replace it:
// the clamp-form quantity source (q < Q in the box: q becomes Q; the
// adjoint is recorded per box cell for dL/dQ and none flows back) and the
// velocity inflow (|w| < |V| in the box: w becomes V).  val is the advected
// value as the forward compared it.
template <typename TV>
__device__ __forceinline__ double inputs_adjoint_gate(const Phys& p, int ent, int li, int lj, TV val, double fbar,
                                                      double* qclamp) {
    if (!in_box_idx(p, ent, li, lj)) return fbar;
    if (ent == E_CELL) {
        if (p.src_mode != 0) return fbar;
        // FP64 and the unfused FP32 inputs compare in FP64; the fused FP32
        // epilogue compares with Q rounded to FP32
        const bool clamped =
            (sizeof(TV) == 8 || p.force_density) ? (double)val < p.src_q : (float)val < (float)p.src_q;
        qclamp[(lj - p.box[E_CELL][2]) * (p.box[E_CELL][1] - p.box[E_CELL][0]) + (li - p.box[E_CELL][0])] =
            clamped ? fbar : 0.0;
        return clamped ? 0.0 : fbar;
    }
    return fabs((double)val) < fabs(p.src_vel[ent - 1]) ? 0.0 : fbar;
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
    // inputs that replace the advected value where they fire carry no
    // sensitivity to it there: the clamp q = max(q, Q) (the adjoint goes to
    // dL/dQ instead) and the velocity inflow (src/InflowSource.hpp:39-77)
    const double fb = inputs_adjoint_gate(p, ent, li, lj, sf.val, fbar, a.qclamp);
    put_rec(a.F[ent], t, sf.kx, sf.ky, fb, sf.wx, sf.wy, a.order == 1 ? 2 : 4);
    double tbx = fb * sf.gx, tby = fb * sf.gy;
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

// --------------------------------------------------------------------------
// Mixed precision (FP32 bulk): the transpose of the FP32 advection without
// records.  One warp per strip of 28 destination columns x 32 destination
// rows (ghosted index space, from (1, 1)); lane l takes target column
// X0 - 2 + l, and lanes 2 .. 29 own destination column X0 - 2 + l.  While
// every RK position stays within a cell of its entity (checked; the call
// fails otherwise), each tap of a target lies within two columns and two
// rows of it, for every entity kind, stage and sample.  So a lane gathers
// the contributions of one target row (cell, I-face and J-face targets at
// its column) into three 5 x 5 register tiles P[dy][dx] (destination
// fields q, u, v at offsets dx, dy in [-2, 2]); five shuffles per tile row
// then hand each destination lane the contributions of the five target
// columns that reach it, in a fixed order, into a window of five
// destination rows per field.  The warp walks the target rows from Y0 - 2
// to Y0 + 33; after target row t, destination row t - 2 is complete and is
// written.  No atomics, no scatter records: deterministic, and the
// forward's traces are recomputed with the forward's own FP32 arithmetic
// (cf_adv32.cuh), so every stencil is the forward's.
constexpr int AJ_COLS = 28;
constexpr int AJ_ROWS = 32;
constexpr int AJ_WARPS = 4;

struct AdjAdv32 {
    Phys p;
    Grid<float> q;            // forward quantity of the step (ghosts filled)
    Grid<double> u, v;        // forward velocities, pairs (hi parts read)
    Grid<float> aq;           // adjoint of the advected quantity
    Grid<double> au, av;      // adjoint of the advected velocities, pairs (hi parts read)
    Grid<float> oq;           // adjoint of the step's initial fields (ghosted): q in FP32,
    Grid<double> ou, ov;      // u, v as pairs (value, 0)
    float c;                  // dt / dx, as the forward's
    int nsx, nsy;             // strips along x, y
    int* err;
    double* qclamp;           // clamp-form source (inputs_adjoint_gate)
};

__device__ __forceinline__ int aj_at(int dx, int dy) { return (dy + 2) * 5 + (dx + 2); }

// a cubic sample's weights, stencil start o in {-2, -1}
__device__ __forceinline__ void aj_spread_cub(int o, const float* w, float* W) {
#pragma unroll
    for (int k = 0; k < 5; ++k) W[k] = o == -2 ? (k < 4 ? w[k] : 0.f) : (k > 0 ? w[k - 1] : 0.f);
}
__device__ __forceinline__ void aj_outer(float* P, float s, const float* WX, const float* WY) {
    float x[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) x[k] = s * WX[k];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
        for (int k = 0; k < 5; ++k) P[r * 5 + k] = fmaf(WY[r], x[k], P[r * 5 + k]);
}
// A linear sample at a position p = o + d of the target (o in {-1/2, 0,
// 1/2} per axis, |d| < 1) has its stencil cell in [floor(o - 1) + 1 ..
// floor(o + 1)] and its taps in columns [XLO, XLO + XN): o = 0: [-1, 2),
// o = 1/2: [-1, 3), o = -1/2: [-2, 2).  Only that block of the tile is
// touched (the same products as the full tile, without the zero terms).
template <int TWO_O>
struct AjSpan {
    static constexpr int lo = TWO_O < 0 ? -2 : -1;
    static constexpr int n = TWO_O == 0 ? 3 : 4;
};
template <int TWO_OX, int TWO_OY>
__device__ __forceinline__ void aj_lin(float* P, float s, const Lin32& l) {
    constexpr int XL = AjSpan<TWO_OX>::lo, XN = AjSpan<TWO_OX>::n;
    constexpr int YL = AjSpan<TWO_OY>::lo, YN = AjSpan<TWO_OY>::n;
    float x[XN];
#pragma unroll
    for (int k = 0; k < XN; ++k) x[k] = s * ((XL + k == l.ox) ? 1.f - l.tx : ((XL + k == l.ox + 1) ? l.tx : 0.f));
#pragma unroll
    for (int r = 0; r < YN; ++r) {
        const float wy = (YL + r == l.oy) ? 1.f - l.ty : ((YL + r == l.oy + 1) ? l.ty : 0.f);
#pragma unroll
        for (int k = 0; k < XN; ++k) P[aj_at(XL + k, YL + r)] = fmaf(wy, x[k], P[aj_at(XL + k, YL + r)]);
    }
}

// A trace displacement (index units) that reaches a full cell, or is NaN,
// fails the call; it is replaced by 0 so that every tap stays inside the
// arrays (a valid trace keeps its bits).
__device__ __forceinline__ float aj_safe(float d, bool& bad) {
    if (fabsf(d) < 1.f) return d;
    bad = true;
    return 0.f;
}

// One target: the forward trace (advect_value in cf_fields.cu, same
// operations), then its transpose with fbar the adjoint of the advected
// value.  Position derivatives are in index units (the trace moves by
// d = -c a, c = dt / dx).
template <int ORDER, bool GATE, int ENT, typename T>
__device__ __forceinline__ void aj_target(const AdjAdv32& a, const T& U, const T& V, const T& Q, int li, int lj,
                                          float fbar, float* Pq, float* Pu, float* Pv, bool& bad) {
    const float ox_e = ENT == E_FACEI ? 0.f : 0.5f;
    const float oy_e = ENT == E_FACEJ ? 0.f : 0.5f;
    const float uox = ox_e, uoy = oy_e - 0.5f, vox = ox_e - 0.5f, voy = oy_e;
    float v0x, v0y;
    stage0_32(ENT, U, V, li, lj, v0x, v0y);
    const float c = a.c;
    const float h1 = -0.5f * c, h2 = -0.75f * c;
    const float d1x = aj_safe(h1 * v0x, bad), d1y = aj_safe(h1 * v0y, bad);
    const Lin32 s1u = lin32g(U, li, lj, uox + d1x, uoy + d1y);
    const Lin32 s1v = lin32g(V, li, lj, vox + d1x, voy + d1y);
    const bool ralston = (a.p.quirks & 2u) != 0;
    const float d2x = aj_safe(h2 * (ralston ? s1u.val : v0x), bad);
    const float d2y = aj_safe(h2 * (ralston ? s1v.val : v0y), bad);
    const Lin32 s2u = lin32g(U, li, lj, uox + d2x, uoy + d2y);
    const Lin32 s2v = lin32g(V, li, lj, vox + d2x, voy + d2y);
    const float ax = fmaf(4.f / 9.f, s2u.val, fmaf(3.f / 9.f, s1u.val, (2.f / 9.f) * v0x));
    const float ay = fmaf(4.f / 9.f, s2v.val, fmaf(3.f / 9.f, s1v.val, (2.f / 9.f) * v0y));
    const float dx = aj_safe(-c * ax, bad), dy = aj_safe(-c * ay, bad);
    // the advected field's sample at the foot: its value (the forward's
    // bits: the inputs that replace it compare it), derivatives, weights
    float* PF = ENT == E_CELL ? Pq : (ENT == E_FACEI ? Pu : Pv);
    const T& F = ENT == E_CELL ? Q : (ENT == E_FACEI ? U : V);
    float gx, gy, val;
    Lin32 sf;
    float WX[5], WY[5];
    if (ORDER == 1) {
        sf = lin32g(F, li, lj, dx, dy);
        gx = sf.gx;
        gy = sf.gy;
        val = sf.val;
    } else {
        const float flx = floorf(dx), fly = floorf(dy);
        const int ox = (int)flx, oy = (int)fly;
        const float tx = dx - flx, ty = dy - fly;
        float wx[4], wy[4], dwx[4], dwy[4];
        cubic_w32(tx, wx);
        cubic_w32(ty, wy);
        cubic_dw32(tx, dwx);
        cubic_dw32(ty, dwy);
        // the value and the derivatives against differences from the centre
        // tap, as the forward samples (a constant field has zero gradient)
        const float* base = F.at(li + ox - 1, lj + oy - 1);
        const int st = F.stride(), e = F.step();
        const float cc = T::ld(base + st + e);
        // rows 0, 1 and 2, 3 as packed pairs (each lane as the scalar form)
        const float2 c2 = make_float2(cc, cc);
        float2 rs01 = make_float2(0.f, 0.f), rd01 = rs01, rs23 = rs01, rd23 = rs01;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 w = make_float2(wx[k], wx[k]), dw = make_float2(dwx[k], dwx[k]);
            const float2 f01 = f2_sub(make_float2(T::ld(base + k * e), T::ld(base + st + k * e)), c2);
            const float2 f23 = f2_sub(make_float2(T::ld(base + 2 * st + k * e), T::ld(base + 3 * st + k * e)), c2);
            rs01 = f2_fma(w, f01, rs01);
            rd01 = f2_fma(dw, f01, rd01);
            rs23 = f2_fma(w, f23, rs23);
            rd23 = f2_fma(dw, f23, rd23);
        }
        const float rs[4] = {rs01.x, rs01.y, rs23.x, rs23.y}, rd[4] = {rd01.x, rd01.y, rd23.x, rd23.y};
        gx = 0.f;
        gy = 0.f;
        float vs = 0.f;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            if (GATE) vs = fmaf(wy[b], rs[b], vs);
            gx = fmaf(wy[b], rd[b], gx);
            gy = fmaf(dwy[b], rs[b], gy);
        }
        val = cc + vs;
        aj_spread_cub(ox - 1, wx, WX);
        aj_spread_cub(oy - 1, wy, WY);
    }
    if (GATE) fbar = (float)inputs_adjoint_gate(a.p, ENT, li, lj, val, (double)fbar, a.qclamp);
    if (ORDER == 1)
        aj_lin<0, 0>(PF, fbar, sf);
    else
        aj_outer(PF, fbar, WX, WY);
    // reverse of a = 2/9 v0 + 3/9 v1 + 4/9 v2, d = -c a
    const float abx = -c * (fbar * gx), aby = -c * (fbar * gy);
    float v0bx = (2.f / 9.f) * abx, v0by = (2.f / 9.f) * aby;
    float v1bx = (3.f / 9.f) * abx, v1by = (3.f / 9.f) * aby;
    const float v2bx = (4.f / 9.f) * abx, v2by = (4.f / 9.f) * aby;
    // stage 2 at d2 = h2 (v1 or v0)
    // doubled sample offsets of the velocity grids from the entity
    constexpr int UX = ENT == E_FACEI ? 0 : 1, UY = ENT == E_FACEJ ? -1 : 0;
    constexpr int VX = ENT == E_FACEI ? -1 : 0, VY = ENT == E_FACEJ ? 0 : 1;
    aj_lin<UX, UY>(Pu, v2bx, s2u);
    aj_lin<VX, VY>(Pv, v2by, s2v);
    const float d2bx = fmaf(v2bx, s2u.gx, v2by * s2v.gx), d2by = fmaf(v2bx, s2u.gy, v2by * s2v.gy);
    if (ralston) {
        v1bx = fmaf(h2, d2bx, v1bx);
        v1by = fmaf(h2, d2by, v1by);
    } else {
        v0bx = fmaf(h2, d2bx, v0bx);
        v0by = fmaf(h2, d2by, v0by);
    }
    // stage 1 at d1 = h1 v0
    aj_lin<UX, UY>(Pu, v1bx, s1u);
    aj_lin<VX, VY>(Pv, v1by, s1v);
    const float d1bx = fmaf(v1bx, s1u.gx, v1by * s1v.gx), d1by = fmaf(v1bx, s1u.gy, v1by * s1v.gy);
    v0bx = fmaf(h1, d1bx, v0bx);
    v0by = fmaf(h1, d1by, v0by);
    // stage 0 at the entity (the taps and weights of stage0_32)
    if (ENT == E_CELL) {
        const float hx = 0.5f * v0bx, hy = 0.5f * v0by;
        Pu[aj_at(0, 0)] += hx;
        Pu[aj_at(1, 0)] += hx;
        Pv[aj_at(0, 0)] += hy;
        Pv[aj_at(0, 1)] += hy;
    } else if (ENT == E_FACEI) {
        const float qy = 0.25f * v0by;
        Pu[aj_at(0, 0)] += v0bx;
        Pv[aj_at(-1, 0)] += qy;
        Pv[aj_at(0, 0)] += qy;
        Pv[aj_at(-1, 1)] += qy;
        Pv[aj_at(0, 1)] += qy;
    } else {
        const float qx = 0.25f * v0bx;
        Pu[aj_at(0, -1)] += qx;
        Pu[aj_at(1, -1)] += qx;
        Pu[aj_at(0, 0)] += qx;
        Pu[aj_at(1, 0)] += qx;
        Pv[aj_at(0, 0)] += v0by;
    }
}

// destination lane c takes P[dy][dx] of the lane at column c - dx, dx from
// +2 down to -2, into the window row of destination row t + dy
__device__ __forceinline__ void aj_exchange(const float* P, float* A) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
        float s = A[r];
        s += __shfl_up_sync(0xffffffffu, P[r * 5 + 4], 2);
        s += __shfl_up_sync(0xffffffffu, P[r * 5 + 3], 1);
        s += P[r * 5 + 2];
        s += __shfl_down_sync(0xffffffffu, P[r * 5 + 1], 1);
        s += __shfl_down_sync(0xffffffffu, P[r * 5 + 0], 2);
        A[r] = s;
    }
}

// A block's AJ_WARPS warps take horizontally adjacent strips and share one
// window per field (the hi parts of u, v; q) in shared memory: ghosted
// columns [28 s0 - 3, 28 s0 + 117) for strips s0 .. s0 + 3 and rows
// [Y0 - 4, Y0 + 36), every tap of the strips' targets (two entities around
// targets [X0 - 2, X0 + 30) x [Y0 - 2, Y0 + 34)); entries outside an
// array read as zero and are never tapped.
constexpr int AJW_X = AJ_WARPS * AJ_COLS + 8;
constexpr int AJW_Y = AJ_ROWS + 8;
constexpr int AJW_N = AJW_X * AJW_Y;
constexpr size_t AJ_SMEM = 3 * AJW_N * sizeof(float);

struct AjWin {
    const float* s;  // ghosted (x0, y0)
    int x0, y0;
    static constexpr bool kClamp = false;
    __device__ __forceinline__ const float* at(int ix, int iy) const { return s + ((iy - y0) * AJW_X + (ix - x0)); }
    __device__ __forceinline__ static constexpr int stride() { return AJW_X; }
    __device__ __forceinline__ static constexpr int step() { return 1; }
    __device__ __forceinline__ static float ld(const float* p) { return *p; }
};

// GATE: the inflow box is active with a replacing input (clamp-form source
// or an inflow velocity), so targets compare their advected value
template <int ORDER, bool GATE>
__global__ void __launch_bounds__(AJ_WARPS * 32) k_adj_advect32(AdjAdv32 a) {
    extern __shared__ __align__(16) float aw[];  // u, v, q windows
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nbx = (a.nsx + AJ_WARPS - 1) / AJ_WARPS;
    const int s0 = (blockIdx.x % nbx) * AJ_WARPS, sy = blockIdx.x / nbx;
    const int Y0 = 1 + sy * AJ_ROWS;
    const int wx0 = 1 + s0 * AJ_COLS - 4, wy0 = Y0 - 4;
    for (int k = threadIdx.x; k < AJW_N; k += AJ_WARPS * 32) {
        const int r = k / AJW_X, cx = k - r * AJW_X;
        const int gx = wx0 + cx, gy = wy0 + r;
        float uu = 0.f, vv = 0.f, qq = 0.f;
        if (gx >= 0 && gy >= 0) {
            if (gx < a.u.ex && gy < a.u.ey) uu = reinterpret_cast<const float2&>(a.u.at(gx, gy)).x;
            if (gx < a.v.ex && gy < a.v.ey) vv = reinterpret_cast<const float2&>(a.v.at(gx, gy)).x;
            if (gx < a.q.ex && gy < a.q.ey) qq = a.q.at(gx, gy);
        }
        aw[k] = uu;
        aw[AJW_N + k] = vv;
        aw[2 * AJW_N + k] = qq;
    }
    __syncthreads();
    const int sx = s0 + warp;
    if (sx >= a.nsx) return;  // whole warps, after the block's last barrier
    const AjWin U{aw, wx0, wy0}, V{aw + AJW_N, wx0, wy0}, Q{aw + 2 * AJW_N, wx0, wy0};
    const int X0 = 1 + sx * AJ_COLS;
    const int tc = X0 - 2 + lane;
    const bool owner = lane >= 2 && lane < 2 + AJ_COLS;
    const Phys& p = a.p;
    const int gi = tc - CF_HALO;
    const int oxu = p.nx + (p.per_x ? 0 : 1), oyv = p.ny + (p.per_y ? 0 : 1);
    float Aq[5], Au[5], Av[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) Aq[k] = Au[k] = Av[k] = 0.f;
    bool bad = false;
    // the adjoint values of a target row, fetched one row ahead (they stream
    // from DRAM; the taps come from the windows)
    auto fetch = [&](int tr, float& fq, float& fu, float& fv) {
        const int gj = tr - CF_HALO;
        const bool in = gi >= 0 && gj >= 0;
        fq = (in && gi < p.nx && gj < p.ny) ? a.aq.at(tc, tr) : 0.f;
        fu = (in && gi < oxu && gj < p.ny) ? reinterpret_cast<const float2&>(a.au.at(tc, tr)).x : 0.f;
        fv = (in && gi < p.nx && gj < oyv) ? reinterpret_cast<const float2&>(a.av.at(tc, tr)).x : 0.f;
    };
    float fq, fu, fv;
    fetch(Y0 - 2, fq, fu, fv);
#pragma unroll 1
    for (int tr = Y0 - 2; tr < Y0 + AJ_ROWS + 2; ++tr) {
        float nq, nu, nv;
        fetch(tr + 1, nq, nu, nv);
        float Pq[25], Pu[25], Pv[25];
#pragma unroll
        for (int k = 0; k < 25; ++k) Pq[k] = Pu[k] = Pv[k] = 0.f;
        const int gj = tr - CF_HALO;
        if (gi >= 0 && gj >= 0) {
            if (gi < p.nx && gj < p.ny) aj_target<ORDER, GATE, E_CELL>(a, U, V, Q, tc, tr, fq, Pq, Pu, Pv, bad);
            if (gi < oxu && gj < p.ny) aj_target<ORDER, GATE, E_FACEI>(a, U, V, Q, tc, tr, fu, Pq, Pu, Pv, bad);
            if (gi < p.nx && gj < oyv) aj_target<ORDER, GATE, E_FACEJ>(a, U, V, Q, tc, tr, fv, Pq, Pu, Pv, bad);
        }
        fq = nq;
        fu = nu;
        fv = nv;
        aj_exchange(Pq, Aq);
        aj_exchange(Pu, Au);
        aj_exchange(Pv, Av);
        const int r = tr - 2;  // complete
        if (owner && r >= Y0 && r < Y0 + AJ_ROWS) {
            if (tc < a.oq.ex && r < a.oq.ey) a.oq.at(tc, r) = Aq[0];
            if (tc < a.ou.ex && r < a.ou.ey) reinterpret_cast<float2&>(a.ou.at(tc, r)) = make_float2(Au[0], 0.f);
            if (tc < a.ov.ex && r < a.ov.ey) reinterpret_cast<float2&>(a.ov.at(tc, r)) = make_float2(Av[0], 0.f);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            Aq[k] = Aq[k + 1];
            Au[k] = Au[k + 1];
            Av[k] = Av[k + 1];
        }
        Aq[4] = Au[4] = Av[4] = 0.f;
    }
    if (bad) atomicOr(a.err, 1);
}

// host arrays (row pitch nox, FP64) <-> owned entries of an FP32 grid
// (pairs = 0) or of a pair grid (pairs = 1)
__global__ void k_adj_import(Grid<double> d, Grid<float> f, int pairs, const double* src, int nox, int noy) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nox || gj >= noy) return;
    const double w = src[(size_t)gj * nox + gi];
    if (pairs)
        reinterpret_cast<float2&>(d.at(gi + CF_HALO, gj + CF_HALO)) = df_split(w);
    else
        f.at(gi + CF_HALO, gj + CF_HALO) = __double2float_rn(w);
}
__global__ void k_adj_export(Grid<double> d, Grid<float> f, int pairs, double* dst, int nox, int noy) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nox || gj >= noy) return;
    dst[(size_t)gj * nox + gi] = pairs ? df_value(reinterpret_cast<const float2&>(d.at(gi + CF_HALO, gj + CF_HALO)))
                                       : (double)f.at(gi + CF_HALO, gj + CF_HALO);
}

// periodic axes: add the adjoint that landed on ghost copies to the owned entity
template <typename T>
__global__ void k_adj_fold(Grid<T> g, int nox, int noy, int per_x, int per_y) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nox || gj >= noy) return;
    T acc = g.at(gi + CF_HALO, gj + CF_HALO);
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

// wall masks on faces: u at SOLID x-walls, v at SOLID y-walls (thread t
// takes wall row / column t)
__global__ void k_adj_mask(Phys p, Grid<double> u, Grid<double> v) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (!p.per_x && t < p.ny) {
        if (p.bc[0] == 0) u.at(CF_HALO, t + CF_HALO) = 0.0;
        if (p.bc[2] == 0) u.at(p.nx + CF_HALO, t + CF_HALO) = 0.0;
    }
    if (!p.per_y && t < p.nx) {
        if (p.bc[1] == 0) v.at(t + CF_HALO, CF_HALO) = 0.0;
        if (p.bc[3] == 0) v.at(t + CF_HALO, p.ny + CF_HALO) = 0.0;
    }
}
static void launch_adj_mask(cf_ctx* c, Grid<double> u, Grid<double> v) {
    const int n = c->ph.nx > c->ph.ny ? c->ph.nx : c->ph.ny;
    k_adj_mask<<<(n + 255) / 256, 256, 0, c->stream>>>(c->ph, u, v);
    c->launches += 1;
}

// periodic axes, pair arrays: add the high parts that landed on ghost copies
// to the owned entity's (the reverse advection writes pairs (value, 0))
__global__ void k_adj_fold_pairs(Grid<double> g, int nox, int noy, int per_x, int per_y) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nox || gj >= noy) return;
    float2& own = reinterpret_cast<float2&>(g.at(gi + CF_HALO, gj + CF_HALO));
    float acc = own.x;
    for (int ky = -1; ky <= 1; ++ky)
        for (int kx = -1; kx <= 1; ++kx) {
            if (kx == 0 && ky == 0) continue;
            if ((kx && !per_x) || (ky && !per_y)) continue;
            int li = gi + CF_HALO + kx * nox, lj = gj + CF_HALO + ky * noy;
            if (li < 0 || lj < 0 || li >= g.ex || lj >= g.ey) continue;
            acc = acc + reinterpret_cast<const float2&>(g.at(li, lj)).x;
        }
    own = make_float2(acc, 0.f);
}

// dL/d(rate) += dt * (sum of the quantity adjoint over the inflow box's
// cells).  One block: the box's cells (local index ranges the host found
// with the forward's coordinate test) in row-major order, thread t taking
// cells t, t + 256, ...; then a fixed-order block sum, so the result is
// deterministic.
constexpr int kBoxThreads = 256;
template <typename T>
__global__ void __launch_bounds__(kBoxThreads) k_adj_rate(Phys p, Grid<T> aq, double dt, double* rbar) {
    const int i0 = p.box[E_CELL][0], i1 = p.box[E_CELL][1], j0 = p.box[E_CELL][2], j1 = p.box[E_CELL][3];
    const int w = i1 - i0, n = w > 0 && j1 > j0 ? w * (j1 - j0) : 0;
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += kBoxThreads) s = s + (double)aq.at(i0 + k % w, j0 + k / w);
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

// Density-scaled body force (u += dt f rho, rho the mean of the face's two
// cells after the cell inputs; Q5): each owned cell's quantity adjoint gains
// dt f / 2 times the adjoint of its two faces per axis (wall faces are
// masked already; periodic faces wrap as the forward's cell reads do).
// Pair arrays (mixed) contribute their value.
template <typename TQ>
__global__ void k_adj_density(Phys p, Grid<TQ> aq, Grid<double> au, Grid<double> av, double dt, int pairs) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= p.nx || gj >= p.ny) return;
    auto face = [&](const Grid<double>& g, int i, int j) {
        const double w = g.at(i + CF_HALO, j + CF_HALO);
        return pairs ? df_value(reinterpret_cast<const float2&>(w)) : w;
    };
    const int ir = (p.per_x && gi + 1 == p.nx) ? 0 : gi + 1;
    const int jt = (p.per_y && gj + 1 == p.ny) ? 0 : gj + 1;
    const double cx = 0.5 * p.force[0] * dt, cy = 0.5 * p.force[1] * dt;
    double s = 0.0;
    if (cx != 0.0) s = cx * (face(au, gi, gj) + face(au, ir, gj));
    if (cy != 0.0) s = s + cy * (face(av, gi, gj) + face(av, gi, jt));
    TQ& q = aq.at(gi + CF_HALO, gj + CF_HALO);
    q = (TQ)((double)q + s);
}

// dL/dQ of the clamp-form source: the sum of the per-box-cell adjoints the
// reverse advection left where the clamp fired, in a fixed order
__global__ void __launch_bounds__(kBoxThreads) k_adj_boxsum(const double* buf, int n, double* rbar) {
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += kBoxThreads) s = s + buf[k];
    __shared__ double ws[kBoxThreads / 32];
    s = warp_fold(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = ws[0];
        for (int k = 1; k < kBoxThreads / 32; ++k) t = t + ws[k];
        *rbar += t;
    }
}

// host side

template <typename T>
static void* grid_base(const Grid<T>& g) {
    return (void*)(g.o - CF_COL0);
}
template <typename T>
static size_t grid_bytes(const Grid<T>& g) {
    return (size_t)g.pitch * g.ey * sizeof(T);
}

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
    // mixed contexts: the adjoint of q in FP32 (aq32; ag[1], ag[2] hold the
    // velocity adjoints as pairs and bg[1], bg[2] the reverse advection's
    // pair outputs, swapped with them after each step) and the reverse
    // advection's FP32 output for q (oq32)
    bool mixed = false;
    bool smem_set = false;  // the reverse advection's shared-memory limit raised
    cudaEvent_t ev_adv[2] = {nullptr, nullptr};  // profiling: around the reverse advection
    Grid<float> aq32{}, oq32{};
    RecKind F[3], Su[3][3], Sv[3][3];
    int* d_err = nullptr;
    double* d_rbar = nullptr;  // dL/d(rate), accumulated on the device
    double* xa = nullptr;      // the adjoint pressure between reverse steps (the warm start)
    double* qclamp = nullptr;  // clamp-form source: per-box-cell adjoints (inputs_adjoint_gate)
    size_t qclamp_n = 0;
    // the forward pass left the last segment's states in seg: the backward's
    // first segment needs no recomputation (cleared once seg is reused)
    bool last_seg_valid = false;
    std::vector<void*> allocs;
};

}  // namespace cf

using namespace cf;

namespace {

bool is_mixed(const cf_ctx* c) { return c->precision == CF_PREC_MIXED; }

// a checkpoint holds the state as the context stores it: q (FP64, or FP32 in
// a mixed context) and u, v (FP64, or pairs), ghosted, back to back
size_t state_bytes(cf_ctx* c) {
    const size_t qb = is_mixed(c) ? grid_bytes(c->q32[0]) : grid_bytes(c->q64[0]);
    return qb + grid_bytes(c->u[0]) + grid_bytes(c->v[0]);
}

int dalloc(cf_ctx* c, AdjState* A, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(c, CF_ERR_NOMEM, "adjoint: cudaMalloc of %zu bytes failed", bytes);
    A->allocs.push_back(*p);
    return CF_OK;
}

// the current state's three arrays as (base, bytes)
void state_parts(cf_ctx* c, void** base, size_t* bytes) {
    const int k = c->cur;
    if (is_mixed(c)) {
        base[0] = grid_base(c->q32[k]);
        bytes[0] = grid_bytes(c->q32[k]);
    } else {
        base[0] = grid_base(c->q64[k]);
        bytes[0] = grid_bytes(c->q64[k]);
    }
    base[1] = grid_base(c->u[k]);
    bytes[1] = grid_bytes(c->u[k]);
    base[2] = grid_base(c->v[k]);
    bytes[2] = grid_bytes(c->v[k]);
}

int save_state(cf_ctx* c, double* dst) {
    char* d = (char*)dst;
    void* base[3];
    size_t bytes[3];
    state_parts(c, base, bytes);
    for (int k = 0; k < 3; ++k) {
        cudaError_t e = cudaMemcpyAsync(d, base[k], bytes[k], cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return cuda_check(c, e, "checkpoint save");
        d += bytes[k];
    }
    return CF_OK;
}

int load_state(cf_ctx* c, const double* src) {
    const char* s = (const char*)src;
    void* base[3];
    size_t bytes[3];
    state_parts(c, base, bytes);
    for (int k = 0; k < 3; ++k) {
        cudaError_t e = cudaMemcpyAsync(base[k], s, bytes[k], cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return cuda_check(c, e, "checkpoint load");
        s += bytes[k];
    }
    return CF_OK;
}

AdjState* adj(cf_ctx* c) { return static_cast<AdjState*>(c->adjoint); }

int check_supported(cf_ctx* c) {
    // a recomputed segment must repeat the forward exactly; a warm start
    // would depend on a pressure the checkpoints do not hold
    if (c->warm) return fail(c, CF_ERR_UNSUPPORTED, "the adjoint needs cold-started projections (warm start is on)");
    const Phys& p = c->ph;
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
    if (!rc) rc = dalloc(c, A, (void**)&A->d_rbar, sizeof(double));
    if (!rc) rc = dalloc(c, A, (void**)&A->xa, sizeof(double) * (size_t)c->vpitch * c->ph.ny);
    return rc;
}

// a zeroed ghosted grid laid out as the context's grids (cf_api.cu alloc_grid)
template <typename T>
int adj_grid(cf_ctx* c, AdjState* A, Grid<T>& g, int ex, int ey) {
    const int pitch = (int)(((size_t)CF_COL0 + ex + 31) / 32 * 32);
    void* base = nullptr;
    const size_t bytes = (size_t)pitch * ey * sizeof(T);
    int rc = dalloc(c, A, &base, bytes);
    if (rc) return rc;
    cudaMemsetAsync(base, 0, bytes, c->stream);
    g.o = (T*)base + CF_COL0;
    g.pitch = pitch;
    g.ex = ex;
    g.ey = ey;
    return CF_OK;
}

// mixed contexts: adjoint grids only (the reverse advection keeps no records)
int setup_mixed(cf_ctx* c, AdjState* A) {
    if (A->aq32.o) return CF_OK;
    const Grid<double>& gu = c->u[0];
    const Grid<double>& gv = c->v[0];
    const Grid<float>& gq = c->q32[0];
    int rc = adj_grid(c, A, A->aq32, gq.ex, gq.ey);
    if (!rc) rc = adj_grid(c, A, A->oq32, gq.ex, gq.ey);
    if (!rc) rc = adj_grid(c, A, A->ag[1], gu.ex, gu.ey);
    if (!rc) rc = adj_grid(c, A, A->ag[2], gv.ex, gv.ey);
    if (!rc) rc = adj_grid(c, A, A->bg[1], gu.ex, gu.ey);
    if (!rc) rc = adj_grid(c, A, A->bg[2], gv.ex, gv.ey);
    if (!rc) rc = dalloc(c, A, (void**)&A->d_err, sizeof(int));
    if (!rc) rc = dalloc(c, A, (void**)&A->d_rbar, sizeof(double));
    if (!rc) rc = dalloc(c, A, (void**)&A->xa, sizeof(double) * (size_t)c->vpitch * c->ph.ny);
    return rc;
}

// A saved state (save_state's layout) as grids of the context's shapes: the
// reverse step reads the forward state of its step in place, with its ghosts
// filled there (the saved copy's ghosts are those of the step before).
struct StateView {
    Grid<double> q64, u, v;
    Grid<float> q32;
};
StateView state_view(cf_ctx* c, double* src) {
    StateView s;
    char* b = (char*)src;
    if (is_mixed(c)) {
        s.q32 = c->q32[0];
        s.q32.o = (float*)b + CF_COL0;
        b += grid_bytes(c->q32[0]);
    } else {
        s.q64 = c->q64[0];
        s.q64.o = (double*)b + CF_COL0;
        b += grid_bytes(c->q64[0]);
    }
    s.u = c->u[0];
    s.u.o = (double*)b + CF_COL0;
    b += grid_bytes(c->u[0]);
    s.v = c->v[0];
    s.v.o = (double*)b + CF_COL0;
    return s;
}
int fill_view_ghosts(cf_ctx* c, const StateView& s) {
    const int k = c->cur;
    const Grid<double> q64 = c->q64[k], u = c->u[k], v = c->v[k];
    const Grid<float> q32 = c->q32[k];
    if (is_mixed(c))
        c->q32[k] = s.q32;
    else
        c->q64[k] = s.q64;
    c->u[k] = s.u;
    c->v[k] = s.v;
    const cudaError_t e = launch_fill_ghosts(c);
    c->q64[k] = q64;
    c->q32[k] = q32;
    c->u[k] = u;
    c->v[k] = v;
    return cuda_check(c, e, "fill ghosts");
}

// Cells of the inflow box when the clamp-form source is on (0 otherwise).
size_t clamp_cells(const cf_ctx* c) {
    const Phys& p = c->ph;
    const int w = p.box[E_CELL][1] - p.box[E_CELL][0], h = p.box[E_CELL][3] - p.box[E_CELL][2];
    return (p.src_mode == 0 && w > 0 && h > 0) ? (size_t)w * h : 0;
}

// The inputs' transpose before the advection's: the density-scaled force
// couples the velocity adjoints into the quantity's, then the rate-form
// source adds to dL/dQ (the clamp form's share comes from the reverse
// advection, which knows where the clamp fired).
template <typename TQ>
void inputs_transpose(cf_ctx* c, AdjState* A, Grid<TQ> aq) {
    const Phys& p = c->ph;
    if (p.force_density && (p.force[0] != 0.0 || p.force[1] != 0.0)) {
        const dim3 blk(32, 8), g((p.nx + 31) / 32, (p.ny + 7) / 8);
        k_adj_density<<<g, blk, 0, c->stream>>>(p, aq, A->ag[1], A->ag[2], A->dt, A->mixed ? 1 : 0);
        c->launches += 1;
    }
    const bool src_active = p.bbox[2] > p.bbox[0] && p.bbox[3] > p.bbox[1];
    if (src_active && p.src_mode == 1) {
        k_adj_rate<<<1, kBoxThreads, 0, c->stream>>>(p, aq, A->dt, A->d_rbar);
        c->launches += 1;
    }
}

// after the advection's transpose: the clamp-form source's dL/dQ
void clamp_sum(cf_ctx* c, AdjState* A) {
    const size_t n = clamp_cells(c);
    if (!n) return;
    k_adj_boxsum<<<1, kBoxThreads, 0, c->stream>>>(A->qclamp, (int)n, A->d_rbar);
    c->launches += 1;
}

// The transposed projection on the adjoint face arrays (pairs in a mixed
// context), starting from the previous reverse step's adjoint pressure.
int adjoint_projection(cf_ctx* c, AdjState* A, const SolveOpts& so, bool params_ready) {
    const Phys& p = c->ph;
    int rc;
    // P^T: mask, then the projection pipeline without the final mask
    launch_adj_mask(c, A->ag[1], A->ag[2]);
    // The solve starts from the previous reverse step's adjoint pressure
    // (zero for the first), kept in A->xa between steps because the forward
    // recomputation uses the solver's solution vector.  The resident graphs
    // of the adjoint's projections (their own cache slots) are built and run
    // with A->xa as the solution vector; the host-polled form, whose batch
    // graphs the forward's projections share, copies it in and out.  A
    // warm-started mixed projection leaves its solution as FP64.
    const bool resident = !c->prof && !c->direct && resident_projection();
    double* const x_fwd = c->x.a;
    const int p_df = c->p_df;
    c->p_df = 0;
    const size_t xbytes = sizeof(double) * (size_t)c->vpitch * p.ny;
    if (resident)
        c->x.a = A->xa;
    else if ((rc = cuda_check(c, cudaMemcpyAsync(c->x.a, A->xa, xbytes, cudaMemcpyDeviceToDevice, c->stream),
                              "adjoint x")))
        return rc;
    SolveResult res{};
    bool deferred = false;
    rc = project_adjoint_async(c, A->dt, so, &res, &deferred, params_ready, A->ag[1], A->ag[2]);
    if (resident) {
        c->x.a = x_fwd;
        c->p_df = p_df;
    }
    if (rc) return rc;
    if (!deferred && res.status != ST_CONVERGED && res.status != ST_MAXIT)
        return fail(c, CF_ERR_NUMERIC, "adjoint projection failed (status %d)", res.status);
    if (!deferred && c->prof) {
        c->pd.adj_projects += 1;
        c->pd.adj_iters += res.iterations;
    }
    if (!resident &&
        (rc = cuda_check(c, cudaMemcpyAsync(A->xa, c->x.a, xbytes, cudaMemcpyDeviceToDevice, c->stream), "adjoint x")))
        return rc;
    // I^T: wall masks of the inputs
    launch_adj_mask(c, A->ag[1], A->ag[2]);
    return CF_OK;
}

// One reverse step of a mixed context: the transposed projection (mixed
// MG/Jacobi PCG on the pair arrays), the inputs' transpose, then the FP32
// reverse advection at the forward state fwd of this step, the periodic
// fold, and the velocity adjoints back to pairs.
int adjoint_step_mixed(cf_ctx* c, AdjState* A, const SolveOpts& so, bool params_ready, double* fwd) {
    const Phys& p = c->ph;
    dim3 blk(32, 8);
    int rc = adjoint_projection(c, A, so, params_ready);
    if (rc) return rc;
    inputs_transpose(c, A, A->aq32);
    const StateView sv = state_view(c, fwd);
    if ((rc = fill_view_ghosts(c, sv))) return rc;
    AdjAdv32 a;
    a.p = p;
    a.q = sv.q32;
    a.u = sv.u;
    a.v = sv.v;
    a.aq = A->aq32;
    a.au = A->ag[1];
    a.av = A->ag[2];
    a.oq = A->oq32;
    a.ou = A->bg[1];
    a.ov = A->bg[2];
    a.c = (float)(A->dt / p.dx);
    // destinations reach two entities past the owned targets: ghosted
    // [1, 3 + n(+1) + 2) on each axis
    const int wx = p.nx + (p.per_x ? 0 : 1) + 4, wy = p.ny + (p.per_y ? 0 : 1) + 4;
    a.nsx = (wx + AJ_COLS - 1) / AJ_COLS;
    a.nsy = (wy + AJ_ROWS - 1) / AJ_ROWS;
    a.err = A->d_err;
    a.qclamp = A->qclamp;
    const int blocks = (a.nsx + AJ_WARPS - 1) / AJ_WARPS * a.nsy;
    if (!A->smem_set) {
        for (auto fn : {k_adj_advect32<1, false>, k_adj_advect32<3, false>, k_adj_advect32<1, true>,
                        k_adj_advect32<3, true>})
            if ((rc = cuda_check(c, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AJ_SMEM),
                                 "adjoint smem")))
                return rc;
        A->smem_set = true;
    }
    const bool box = p.bbox[2] > p.bbox[0] && p.bbox[3] > p.bbox[1];
    const bool gate = box && (p.src_mode == 0 || p.src_vel[0] != 0.0 || p.src_vel[1] != 0.0);
    if (c->prof && !A->ev_adv[0]) {
        for (auto& e : A->ev_adv)
            if ((rc = cuda_check(c, cudaEventCreate(&e), "event create"))) return rc;
    }
    if (c->prof) cudaEventRecord(A->ev_adv[0], c->stream);
    auto kern = A->order == 1 ? (gate ? k_adj_advect32<1, true> : k_adj_advect32<1, false>)
                              : (gate ? k_adj_advect32<3, true> : k_adj_advect32<3, false>);
    kern<<<blocks, AJ_WARPS * 32, AJ_SMEM, c->stream>>>(a);
    c->launches += 1;
    clamp_sum(c, A);
    if (c->prof) {
        cudaEventRecord(A->ev_adv[1], c->stream);
        float ms = 0.f;
        if ((rc = cuda_check(c, cudaEventSynchronize(A->ev_adv[1]), "adjoint timing"))) return rc;
        if (cudaEventElapsedTime(&ms, A->ev_adv[0], A->ev_adv[1]) == cudaSuccess) {
            c->pd.adj_advect_ms += ms;
            c->pd.adj_advect_calls += 1;
        }
    }
    for (int f = 0; f < 3; ++f) {
        const int nox = p.nx + ((f == 1 && !p.per_x) ? 1 : 0);
        const int noy = p.ny + ((f == 2 && !p.per_y) ? 1 : 0);
        const dim3 g((nox + 31) / 32, (noy + 7) / 8);
        if (p.per_x || p.per_y) {
            if (f == 0)
                k_adj_fold<<<g, blk, 0, c->stream>>>(A->oq32, nox, noy, p.per_x, p.per_y);
            else
                k_adj_fold_pairs<<<g, blk, 0, c->stream>>>(A->bg[f], nox, noy, p.per_x, p.per_y);
            c->launches += 1;
        }
    }
    std::swap(A->aq32, A->oq32);
    std::swap(A->ag[1], A->bg[1]);
    std::swap(A->ag[2], A->bg[2]);
    return cuda_check(c, cudaGetLastError(), "adjoint advection");
}

// One reverse step, enqueued without a synchronisation: the transposed
// projection (deferred through its resident graph when that serves it;
// non-convergence and failures are tallied on the device), the inputs'
// transpose with dL/d(rate) accumulated on the device, and the advection's
// transpose (a trace that moved too far sets the device error flag) at the
// forward state fwd of this step (as save_state stored it, read in place).
int adjoint_step(cf_ctx* c, AdjState* A, const SolveOpts& so, bool params_ready, double* fwd) {
    if (A->mixed) return adjoint_step_mixed(c, A, so, params_ready, fwd);
    const Phys& p = c->ph;
    dim3 blk(32, 8);
    int rc = adjoint_projection(c, A, so, params_ready);
    if (rc) return rc;
    // dL/dQ from the rate source
    inputs_transpose(c, A, A->ag[0]);
    // A^T at the forward state of this step
    const StateView sv = state_view(c, fwd);
    if ((rc = fill_view_ghosts(c, sv))) return rc;
    for (int e = 0; e < 3; ++e) A->F[e].n = A->order == 1 ? 2 : 4;
    AdjRec ar;
    ar.p = p;
    ar.q = sv.q64;
    ar.u = sv.u;
    ar.v = sv.v;
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
    ar.qclamp = A->qclamp;
    k_adj_records<<<dim3((p.nx + 1 + 31) / 32, (p.ny + 1 + 7) / 8, 3), blk, 0, c->stream>>>(ar);
    clamp_sum(c, A);
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
    c->launches += 4 + (p.per_x || p.per_y ? 3 : 0);
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

// mixed contexts: owned region of an adjoint array (0: q in FP32, 1, 2: u, v
// as pairs) <-> contiguous FP64 host array, through the FP64 staging buffer
int adj_io_mixed(cf_ctx* c, AdjState* A, int k, double* host, bool to_host) {
    int ox = c->ph.nx, oy = c->ph.ny;
    if (k == 1 && !c->ph.per_x) ox += 1;
    if (k == 2 && !c->ph.per_y) oy += 1;
    const size_t bytes = sizeof(double) * (size_t)ox * oy;
    const Grid<double> d = k == 0 ? Grid<double>{} : A->ag[k];
    const dim3 blk(32, 8), g((ox + 31) / 32, (oy + 7) / 8);
    if (to_host) {
        k_adj_export<<<g, blk, 0, c->stream>>>(d, A->aq32, k != 0, c->staging, ox, oy);
        int rc = cuda_check(c, cudaGetLastError(), "adjoint export");
        if (!rc)
            rc = cuda_check(c, cudaMemcpyAsync(host, c->staging, bytes, cudaMemcpyDeviceToHost, c->stream),
                            "adjoint copy");
        return rc;
    }
    int rc = cuda_check(c, cudaMemcpyAsync(c->staging, host, bytes, cudaMemcpyHostToDevice, c->stream), "adjoint copy");
    if (rc) return rc;
    k_adj_import<<<g, blk, 0, c->stream>>>(d, A->aq32, k != 0, c->staging, ox, oy);
    return cuda_check(c, cudaGetLastError(), "adjoint import");
}

}  // namespace

extern "C" {

int cf_forward_checkpointed(cf_ctx* ctx, int nsteps, int ckpt_every, double dt, int value_order,
                            const cf_solver_opts* opts, cf_solve_stats* last) {
    if (!ctx) return CF_ERR_INVALID;
    if (nsteps <= 0 || ckpt_every <= 0 || !(dt > 0.0) || (value_order != 1 && value_order != 3))
        return fail(ctx, CF_ERR_INVALID, "bad forward_checkpointed arguments");
    if (ctx->warm)
        return fail(ctx, CF_ERR_UNSUPPORTED, "the adjoint needs cold-started projections (warm start is on)");
    cudaSetDevice(ctx->device);
    if (!ctx->adjoint) ctx->adjoint = new AdjState();
    AdjState* A = adj(ctx);
    A->mixed = is_mixed(ctx);
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
    if (!rc) rc = A->mixed ? setup_mixed(ctx, A) : setup_records(ctx, A);
    if (!rc && clamp_cells(ctx) > A->qclamp_n) {
        rc = dalloc(ctx, A, (void**)&A->qclamp, sizeof(double) * clamp_cells(ctx));
        A->qclamp_n = clamp_cells(ctx);
    }
    if (rc) return rc;
    SolveOpts fo{};
    if ((rc = parse_solver_opts(ctx, &A->opts, &fo))) return rc;
    SolveOpts so{};
    so.tol = A->opts.tol;
    so.abs_tol = 0.0;  // the adjoint right-hand side has its own scale
    so.max_iter = A->opts.max_iter;
    // mixed: the forward's reliable-update threshold and outer limit
    so.inner_tol = A->mixed ? fo.inner_tol : 0.1;
    so.max_outer = A->mixed ? fo.max_outer : 200;
    so.precon_none = (!strcmp(A->precon.c_str(), "None") || !strcmp(A->precon.c_str(), "none")) ? 1 : 0;
    so.precon_mg = (A->precon == "PFMG" || A->precon == "SMG" || A->precon == "MG") ? 1 : 0;
    // default relative tolerance of the transposed solves: near the FP64
    // floor; mixed, 1e-7 (the FP32 bulk bounds the gradient's accuracy near
    // 1e-6 relative, and the forward's absolute ||div u|| target is a
    // relative residual of about 4e-7 on the spectral workloads)
    if (!(so.tol > 0.0)) so.tol = A->mixed ? 1e-7 : 1e-12;
    // lambda_T
    const double* seeds[3] = {dL_dq_T, dL_du_T, dL_dv_T};
    const int fields[3] = {CF_FIELD_QUANTITY, CF_FIELD_U, CF_FIELD_V};
    if (A->mixed) {
        cudaMemsetAsync(grid_base(A->aq32), 0, grid_bytes(A->aq32), ctx->stream);
        for (int k = 1; k < 3; ++k) {
            cudaMemsetAsync(grid_base(A->ag[k]), 0, grid_bytes(A->ag[k]), ctx->stream);
            cudaMemsetAsync(grid_base(A->bg[k]), 0, grid_bytes(A->bg[k]), ctx->stream);
        }
        for (int k = 0; k < 3 && !rc; ++k)
            if (seeds[k]) rc = adj_io_mixed(ctx, A, k, const_cast<double*>(seeds[k]), false);
    } else {
        for (int k = 0; k < 3; ++k) cudaMemsetAsync(grid_base(A->ag[k]), 0, grid_bytes(A->ag[k]), ctx->stream);
        for (int k = 0; k < 3 && !rc; ++k)
            if (seeds[k]) rc = adj_io(ctx, A->ag[k], fields[k], const_cast<double*>(seeds[k]), false);
    }
    if (rc) return rc;
    // the forward recomputation, the checkpoint copies and the reverse steps
    // are all enqueued; one synchronisation at the end reads the tally of
    // the pressure solves, the trace check and dL/d(rate)
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
            rc = adjoint_step(ctx, A, so, adj_params, A->seg[k - k0]);
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
    double* outs[3] = {dL_dq0, dL_du0, dL_dv0};
    for (int k = 0; k < 3 && !rc; ++k)
        if (outs[k])
            rc = A->mixed ? adj_io_mixed(ctx, A, k, outs[k], true) : adj_io(ctx, A->ag[k], fields[k], outs[k], true);
    if (!rc) rc = load_state(ctx, A->final_state);
    // the solution vector held recomputed and adjoint pressures: leave zero
    if (!rc)
        rc = cuda_check(ctx, cudaMemsetAsync(ctx->x.a, 0, sizeof(double) * (size_t)ctx->vpitch * ctx->ph.ny, ctx->stream),
                        "pressure reset");
    ctx->p_df = 0;
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "backward");
    if (!rc && dL_drate) *dL_drate = rbar;
    return rc;
}

}  // extern "C"

void cf_adjoint_free(cf_ctx* c) {
    AdjState* A = static_cast<AdjState*>(c->adjoint);
    if (!A) return;
    for (void* p : A->allocs) cudaFree(p);
    for (auto e : A->ev_adv)
        if (e) cudaEventDestroy(e);
    delete A;
    c->adjoint = nullptr;
}
