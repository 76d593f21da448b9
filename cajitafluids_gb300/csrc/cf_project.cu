// Pressure projection: VelocityCorrector::correctVelocity
// (src/VelocityCorrector.hpp:182-282) on one GPU.
//
//   divergence + CG init  (_buildRHS, :182-212, cold start :272)
//   Jacobi-PCG            (Cajita ReferenceConjugateGradient, restated;
//                          matrix :116-144 + BoundaryConditions.hpp:57-97,
//                          Jacobi :158-180)
//   gradient subtraction  (_applyPressure, :214-264, quirk Q1 at :260)
//
// The matrix is never stored: the diagonal and 1/diagonal are looked up
// from a 16-entry table indexed by the cell's wall-adjacency bits, and the
// legs are -scale.  Scalars (alpha, beta, norms, status) stay on the device;
// the last block of each reduction kernel finishes the sum in a fixed order
// and advances the solver state, so the host only polls the status between
// CUDA-graph batches of iterations.
//
// FP64 CG per iteration (two kernels, 80 bytes per cell moved):
//   K1  p <- M^-1 r + beta p ; q <- A p ; partial p.q       (R r, p_old; W p_new, q)
//   K2  x += alpha p ; r -= alpha q ; partial r.z, r.r      (R x, p, r, q; W x, r)
// p ping-pongs between two buffers because K1 recomputes the new direction
// on its halo from the old one.
//
// Mixed precision: PCG on FP32 vectors (r, p twice; z for the multigrid
// preconditioner) with FP64 scalars; K2 adds alpha p into x kept as a
// double-float pair (40 bytes per cell per Jacobi-PCG iteration: A p is
// recomputed in K2 instead of stored).  Reliable updates (residual
// replacement, van der Vorst & Ye 2000): whenever the recursive FP32 residual
// has fallen by a factor delta since the last update, r = b - A x is formed
// in double-float from x and the double-float b and replaces the FP32
// residual, and the iteration continues with the same search direction.
// Convergence is judged only on the residual of a reliable update.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cstdlib>
#include <functional>
#include <cstring>

#include "cf_ctx.cuh"

namespace cf {

#define FULLMASK 0xffffffffu

struct Cg64 {
    int nx, ny, per_x, per_y, G, U, pitch;
    Stencil st;
    double *x, *r, *pa, *pb, *qv;
    const double* z;  // MG: z = V-cycle(r), read instead of M^-1 r
    int mg;
    double *part0, *part1;
    SolverState* S;
};

__device__ __forceinline__ int ebits(const Cg64& a, int c, int j) {
    return edge_bits(c, j, a.nx, a.ny, a.per_x, a.per_y);
}

__device__ __forceinline__ bool converged(const SolverState* S, double rr) {
    return rr <= S->tol2 * S->bb || (S->use_abs && rr * S->area <= S->abs2);
}

// new search direction at one cell (0 outside a wall)
__device__ __forceinline__ double pn1(const Cg64& a, const double* pold, int c, int j, bool first, double beta) {
    int cc = wrap_index(c, a.nx, a.per_x), jj = wrap_index(j, a.ny, a.per_y);
    if (cc < 0 || jj < 0) return 0.0;
    size_t k = (size_t)jj * a.pitch + cc;
    double z = a.mg ? __ldg(a.z + k) : a.st.minv[ebits(a, cc, jj)] * __ldg(a.r + k);
    return first ? z : fma(beta, __ldg(pold + k), z);
}

// new search direction at columns c0, c0+1 of row j
__device__ __forceinline__ double2 pn2(const Cg64& a, const double* pold, int c0, int j, bool first, double beta) {
    int jj = wrap_index(j, a.ny, a.per_y);
    if (jj < 0) return make_double2(0.0, 0.0);
    if (c0 + 1 < a.nx) {
        size_t k = (size_t)jj * a.pitch + c0;
        double z0, z1;
        if (a.mg) {
            double2 zv = __ldg(reinterpret_cast<const double2*>(a.z + k));
            z0 = zv.x;
            z1 = zv.y;
        } else {
            double2 rv = __ldg(reinterpret_cast<const double2*>(a.r + k));
            z0 = a.st.minv[ebits(a, c0, jj)] * rv.x;
            z1 = a.st.minv[ebits(a, c0 + 1, jj)] * rv.y;
        }
        if (first) return make_double2(z0, z1);
        double2 po = __ldg(reinterpret_cast<const double2*>(pold + k));
        return make_double2(fma(beta, po.x, z0), fma(beta, po.y, z1));
    }
    return make_double2(pn1(a, pold, c0, jj, first, beta), pn1(a, pold, c0 + 1, jj, first, beta));
}

// K1: direction update + stencil apply + partial p.q
__global__ void __launch_bounds__(CF_RED_THREADS) k_cg_dir_matvec64(Cg64 a) {
    SolverState* S = a.S;
    if (*(volatile int*)&S->status != ST_RUNNING) return;
    const int it = S->iter;
    const bool first = it == 0;
    const double beta = S->beta;
    const double* pold = (it & 1) ? a.pb : a.pa;
    double* pnew = (it & 1) ? a.pa : a.pb;
    const double ms = a.st.ms;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    double acc = 0.0;
    if (unit < a.U) {
        const int g = unit % a.G, band = unit / a.G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS;
        const int j1 = min(j0 + CF_BAND_ROWS, a.ny);
        double2 pm = pn2(a, pold, c0, j0 - 1, first, beta);
        double2 pc = pn2(a, pold, c0, j0, first, beta);
        for (int j = j0; j < j1; ++j) {
            double2 pp = pn2(a, pold, c0, j + 1, first, beta);
            double left = __shfl_up_sync(FULLMASK, pc.y, 1);
            double right = __shfl_down_sync(FULLMASK, pc.x, 1);
            // the two cells just outside the warp's 64 columns, in one branch
            if (lane == 0 || lane == 31) {
                double ext = pn1(a, pold, lane == 0 ? c0 - 1 : c0 + 2, j, first, beta);
                if (lane == 0)
                    left = ext;
                else
                    right = ext;
            }
            if (c0 < a.nx) {
                size_t k = (size_t)j * a.pitch + c0;
                double q0 = a.st.diag[ebits(a, c0, j)] * pc.x;
                q0 = fma(ms, left, q0);
                q0 = fma(ms, pc.y, q0);
                q0 = fma(ms, pm.x, q0);
                q0 = fma(ms, pp.x, q0);
                acc = fma(pc.x, q0, acc);
                if (c0 + 1 < a.nx) {
                    double q1 = a.st.diag[ebits(a, c0 + 1, j)] * pc.y;
                    q1 = fma(ms, pc.x, q1);
                    q1 = fma(ms, right, q1);
                    q1 = fma(ms, pm.y, q1);
                    q1 = fma(ms, pp.y, q1);
                    acc = fma(pc.y, q1, acc);
                    *reinterpret_cast<double2*>(pnew + k) = pc;
                    *reinterpret_cast<double2*>(a.qv + k) = make_double2(q0, q1);
                } else {
                    pnew[k] = pc.x;
                    a.qv[k] = q0;
                }
            }
            pm = pc;
            pc = pp;
        }
    }
    acc = warp_fold(acc);
    if (unit < a.U && lane == 0) a.part0[unit] = acc;
    if (last_block_arrive(&S->ticket[0])) {
        double pq = final_tree(a.part0, a.U);
        if (threadIdx.x == 0) {
            S->ticket[0] = 0;
            if (!(pq > 0.0))
                S->status = isnan(pq) ? ST_NAN : ST_BREAKDOWN;
            else
                S->alpha = S->rho / pq;
        }
    }
}

// K2: solution / residual update + partial r.z and r.r
__global__ void __launch_bounds__(CF_RED_THREADS) k_cg_update64(Cg64 a) {
    SolverState* S = a.S;
    if (*(volatile int*)&S->status != ST_RUNNING) return;
    const int it = S->iter;
    const double* pv = (it & 1) ? a.pa : a.pb;
    const double alpha = S->alpha, malpha = -alpha;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    double arz = 0.0, arr = 0.0;
    if (unit < a.U) {
        const int g = unit % a.G, band = unit / a.G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS;
        const int j1 = min(j0 + CF_BAND_ROWS, a.ny);
        if (c0 + 1 < a.nx) {
            for (int j = j0; j < j1; ++j) {
                size_t k = (size_t)j * a.pitch + c0;
                double2 xv = *reinterpret_cast<const double2*>(a.x + k);
                double2 p2 = __ldg(reinterpret_cast<const double2*>(pv + k));
                double2 rv = *reinterpret_cast<const double2*>(a.r + k);
                double2 qv = __ldg(reinterpret_cast<const double2*>(a.qv + k));
                xv.x = fma(alpha, p2.x, xv.x);
                xv.y = fma(alpha, p2.y, xv.y);
                rv.x = fma(malpha, qv.x, rv.x);
                rv.y = fma(malpha, qv.y, rv.y);
                double z0 = a.st.minv[ebits(a, c0, j)] * rv.x;
                double z1 = a.st.minv[ebits(a, c0 + 1, j)] * rv.y;
                arz = fma(rv.x, z0, arz);
                arr = fma(rv.x, rv.x, arr);
                arz = fma(rv.y, z1, arz);
                arr = fma(rv.y, rv.y, arr);
                *reinterpret_cast<double2*>(a.x + k) = xv;
                *reinterpret_cast<double2*>(a.r + k) = rv;
            }
        } else if (c0 < a.nx) {
            for (int j = j0; j < j1; ++j) {
                size_t k = (size_t)j * a.pitch + c0;
                double xv = fma(alpha, pv[k], a.x[k]);
                double rv = fma(malpha, a.qv[k], a.r[k]);
                double z0 = a.st.minv[ebits(a, c0, j)] * rv;
                arz = fma(rv, z0, arz);
                arr = fma(rv, rv, arr);
                a.x[k] = xv;
                a.r[k] = rv;
            }
        }
    }
    arz = warp_fold(arz);
    arr = warp_fold(arr);
    if (unit < a.U && lane == 0) {
        a.part0[unit] = arz;
        a.part1[unit] = arr;
    }
    if (last_block_arrive(&S->ticket[1])) {
        double rz = final_tree(a.part0, a.U);
        double rr = final_tree(a.part1, a.U);
        if (threadIdx.x == 0) {
            S->ticket[1] = 0;
            if (!a.mg) {
                S->beta = rz / S->rho;
                S->rho = rz;
            }
            S->rr = rr;
            S->iter = it + 1;
            if (isnan(rr))
                S->status = ST_NAN;
            else if (converged(S, rr))
                S->status = ST_CONVERGED;
            else if (it + 1 >= S->max_iter)
                S->status = ST_MAXIT;
        }
    }
}

// MG-PCG: rho_new = r.z after the V-cycle, beta = rho_new / rho (init = 1:
// rho only).  Runs only while the solve is live.
__global__ void __launch_bounds__(CF_RED_THREADS) k_mg_rz64(Cg64 a, int init) {
    SolverState* S = a.S;
    if (*(volatile int*)&S->status != ST_RUNNING) return;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    double arz = 0.0;
    if (unit < a.U) {
        const int g = unit % a.G, band = unit / a.G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS;
        const int j1 = min(j0 + CF_BAND_ROWS, a.ny);
        if (c0 + 1 < a.nx) {
            for (int j = j0; j < j1; ++j) {
                size_t k = (size_t)j * a.pitch + c0;
                double2 rv = __ldg(reinterpret_cast<const double2*>(a.r + k));
                double2 zv = __ldg(reinterpret_cast<const double2*>(a.z + k));
                arz = fma(rv.x, zv.x, arz);
                arz = fma(rv.y, zv.y, arz);
            }
        } else if (c0 < a.nx) {
            for (int j = j0; j < j1; ++j) {
                size_t k = (size_t)j * a.pitch + c0;
                arz = fma(a.r[k], a.z[k], arz);
            }
        }
    }
    arz = warp_fold(arz);
    if (unit < a.U && lane == 0) a.part0[unit] = arz;
    if (last_block_arrive(&S->ticket[7])) {
        double rz = final_tree(a.part0, a.U);
        if (threadIdx.x == 0) {
            S->ticket[7] = 0;
            if (!init) S->beta = rz / S->rho;
            S->rho = rz;
        }
    }
}

// Warm start (FP64): r = b - A x from the previous solution, with A x in the
// matvec's order (diag x_C, then the W, E, S, N legs), canonical r.z and r.r,
// and the solver state as the cold init sets it (||b||^2 from k_div_init64).
__global__ void __launch_bounds__(CF_RED_THREADS) k_warm_resid64(Cg64 a) {
    SolverState* S = a.S;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    const double ms = a.st.ms;
    double arz = 0.0, arr = 0.0;
    if (unit < a.U) {
        const int g = unit % a.G, band = unit / a.G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS;
        const int j1 = min(j0 + CF_BAND_ROWS, a.ny);
        auto xv = [&](int c, int j) -> double {
            int cc = wrap_index(c, a.nx, a.per_x), jj = wrap_index(j, a.ny, a.per_y);
            if (cc < 0 || jj < 0) return 0.0;
            return a.x[(size_t)jj * a.pitch + cc];
        };
        for (int j = j0; j < j1; ++j)
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const int c = c0 + s;
                if (c >= a.nx) continue;
                const int eb = ebits(a, c, j);
                double ax = a.st.diag[eb] * xv(c, j);
                ax = fma(ms, xv(c - 1, j), ax);
                ax = fma(ms, xv(c + 1, j), ax);
                ax = fma(ms, xv(c, j - 1), ax);
                ax = fma(ms, xv(c, j + 1), ax);
                const size_t k = (size_t)j * a.pitch + c;
                const double r = a.r[k] - ax;
                a.r[k] = r;
                const double z = a.st.minv[eb] * r;
                arz = fma(r, z, arz);
                arr = fma(r, r, arr);
            }
    }
    arz = warp_fold(arz);
    arr = warp_fold(arr);
    if (unit < a.U && lane == 0) {
        a.part0[unit] = arz;
        a.part1[unit] = arr;
    }
    if (last_block_arrive(&S->ticket[3])) {
        double rz = final_tree(a.part0, a.U);
        double rr = final_tree(a.part1, a.U);
        if (threadIdx.x == 0) {
            S->ticket[3] = 0;
            S->rr = rr;
            S->rho = rz;
            S->beta = 0.0;
            S->iter = 0;
            if (S->bb == 0.0 || converged(S, rr))
                S->status = ST_CONVERGED;
            else if (S->max_iter <= 0)
                S->status = ST_MAXIT;
            else if (isnan(rr))
                S->status = ST_NAN;
            else
                S->status = ST_RUNNING;
        }
    }
}

// --------------------------------------------------------------------------
// Divergence: b = -(1/dx) (u(i+1) - u(i) + v(j+1) - v(j))  (:204-210)
struct DivArgs {
    int nx, ny, per_x, per_y, G, U, pitch, pitch32;
    Grid<double> u, v;
    double mscale;  // -(1/dx)
    Stencil st;
    double *x, *r, *b;
    float* r32;
    double *part0, *part1;
    double* out;
    SolverState* S;
    int warm;  // keep x from the previous solve (warm start) instead of x = 0
    int mixed;        // k_div_norms: squares and magnitudes in FP32
    float mscale32;   // -(1/dx) in FP32
    float2 mscale2;   // -(1/dx) as a double-float pair
    // k_div_init_mixed (when set): the faces k_apply_pairs_norms cannot read
    // once the gradient has started, saved as pairs: u on each unit's west
    // column (ubnd[g * ny + j] = u(64 g, j)) and v on each unit's south row
    // (vbnd[band * nx + c] = v(c, 16 band))
    float2 *ubnd, *vbnd;
};

__device__ __forceinline__ double div_b(const DivArgs& a, int gi, int gj) {
    int ie = gi + 1, jn = gj + 1;
    if (a.per_x && ie == a.nx) ie = 0;
    if (a.per_y && jn == a.ny) jn = 0;
    double u0 = a.u.at(gi + CF_HALO, gj + CF_HALO), u1 = a.u.at(ie + CF_HALO, gj + CF_HALO);
    double v0 = a.v.at(gi + CF_HALO, gj + CF_HALO), v1 = a.v.at(gi + CF_HALO, jn + CF_HALO);
    double t = u1 - u0;
    t = t + v1;
    t = t - v0;
    return a.mscale * t;
}

// FP32 solver vectors carry a ghost ring (cf_cg32.cu); r's periodic ghost
// copies are written by whoever writes r.
__device__ __forceinline__ void put_r32(float* o, int pitch, int nx, int ny, int per_x, int per_y, int i, int j,
                                        float val) {
    const ptrdiff_t row = (ptrdiff_t)j * pitch;
    o[row + i] = val;
    if (per_x) {
        if (i == 0) o[row + nx] = val;
        if (i == nx - 1) o[row - 1] = val;
    }
    if (per_y) {
        if (j == 0) o[(ptrdiff_t)ny * pitch + i] = val;
        if (j == ny - 1) o[-(ptrdiff_t)pitch + i] = val;
    }
}

// The mixed solution x and right-hand side b are kept as double-float pairs
// (hi + lo, two FP32 numbers, about 48 significant bits; Dekker 1971): the
// reliable update r = b - A x then runs on the FP32 pipe instead of GB300's
// narrow FP64 pipe, with an error (~1e-14 relative to |b| + |A x|) far below
// what the 1e-8 divergence target needs.  nvcc --fmad=false keeps the
// error-free transformations exact.
// (df_add, df_mul, df_split and df_value: cf_internal.cuh)

// FP64 init: b, r = b, x = 0, partial r.z and r.r
__global__ void __launch_bounds__(CF_RED_THREADS) k_div_init64(DivArgs a) {
    SolverState* S = a.S;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    double arz = 0.0, arr = 0.0;
    if (unit < a.U) {
        const int g = unit % a.G, band = unit / a.G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS;
        const int j1 = min(j0 + CF_BAND_ROWS, a.ny);
        for (int j = j0; j < j1; ++j)
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                int c = c0 + s;
                if (c >= a.nx) continue;
                double b = div_b(a, c, j);
                size_t k = (size_t)j * a.pitch + c;
                a.r[k] = b;
                if (!a.warm) a.x[k] = 0.0;
                double z = a.st.minv[edge_bits(c, j, a.nx, a.ny, a.per_x, a.per_y)] * b;
                arz = fma(b, z, arz);
                arr = fma(b, b, arr);
            }
    }
    arz = warp_fold(arz);
    arr = warp_fold(arr);
    if (unit < a.U && lane == 0) {
        a.part0[unit] = arz;
        a.part1[unit] = arr;
    }
    if (last_block_arrive(&S->ticket[2])) {
        double rz = final_tree(a.part0, a.U);
        double rr = final_tree(a.part1, a.U);
        if (threadIdx.x == 0) {
            S->ticket[2] = 0;
            S->bb = rr;
            S->rr = rr;
            S->rho = rz;
            S->beta = 0.0;
            S->iter = 0;
            if (rr == 0.0 || converged(S, rr))
                S->status = ST_CONVERGED;
            else if (S->max_iter <= 0)
                S->status = ST_MAXIT;
            else if (isnan(rr))
                S->status = ST_NAN;
            else
                S->status = ST_RUNNING;
        }
    }
}

// A mixed context's u, v element as its double-float pair
__device__ __forceinline__ float2 pair_at(const Grid<double>& g, int i, int j) {
    return reinterpret_cast<const float2&>(g.at(i, j));
}
__device__ __forceinline__ float2 df_neg(float2 x) { return make_float2(-x.x, -x.y); }

// The divergences of one unit's cells (64 columns x up to 16 rows, lane l
// on columns c0 = 64 g + 2 l and c0 + 1), row by row: each row loads the
// lane's two u pairs and two v pairs of row j + 1 as 16-byte vectors (row j's
// v pairs come from the previous row), the E face of column c0 + 1 from the
// next lane, and reads directly only the one pair a wrap, the domain's last
// column or the warp's last lane needs; every load of row j + 1 is issued
// before row j's divergences are handed to f.  Calls f(c, j, div) for every
// owned cell, div = ((u_E - u_W) + v_N) - v_S of its face pairs in
// double-float (E across a periodic wrap is column 0, N row 0).
template <typename F>
__device__ __forceinline__ void div_pairs_unit(const DivArgs& a, int g, int band, int lane, F&& f) {
    const int c0 = g * CF_UNIT_COLS + 2 * lane;
    const int j0 = band * CF_BAND_ROWS, j1 = min(j0 + CF_BAND_ROWS, a.ny);
    const bool live = c0 < a.nx, two = c0 + 1 < a.nx;
    // the pair read directly: the E face of column c0 + 1 (the warp's last
    // lane, the domain's last column: a boundary face, or column 0 across a
    // periodic wrap), or of column c0 (its wrap to column 0)
    const bool e2 = live && two && (lane == 31 || c0 + 2 >= a.nx);
    const bool e1 = live && !two && a.per_x;
    const int ie = e2 ? ((a.per_x && c0 + 2 == a.nx) ? 0 : c0 + 2) : 0;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    // the two pairs at columns c0, c0 + 1 of a row of u or v (in the ghosted
    // arrays: a column past the owned range is a ghost or a boundary face,
    // read but unused)
    auto pair2 = [&](const Grid<double>& g2, int jj) {
        return live ? *reinterpret_cast<const float4*>(&g2.at(c0 + CF_HALO, jj + CF_HALO)) : zero4;
    };
    auto north = [&](int j) { return (a.per_y && j + 1 == a.ny) ? 0 : j + 1; };
    auto edge = [&](int j) {
        return (e1 || e2) ? pair_at(a.u, ie + CF_HALO, j + CF_HALO) : make_float2(0.f, 0.f);
    };
    float4 v0 = pair2(a.v, j0);
    float4 un = pair2(a.u, j0), vn = pair2(a.v, north(j0));
    float2 en = edge(j0);
    if (a.vbnd && live) {
        a.vbnd[(size_t)band * a.nx + c0] = make_float2(v0.x, v0.y);
        if (two) a.vbnd[(size_t)band * a.nx + c0 + 1] = make_float2(v0.z, v0.w);
    }
    for (int j = j0; j < j1; ++j) {
        const float4 uu = un, v1 = vn;
        const float2 ex = en;
        if (a.ubnd && lane == 0 && live) a.ubnd[(size_t)g * a.ny + j] = make_float2(uu.x, uu.y);
        if (j + 1 < j1) {
            un = pair2(a.u, j + 1);
            vn = pair2(a.v, north(j + 1));
            en = edge(j + 1);
        }
        // u at column c0 + 2 (the E face of column c0 + 1): the next lane's
        // first pair, or the pair read directly
        float2 ue2 = make_float2(__shfl_down_sync(FULLMASK, uu.x, 1), __shfl_down_sync(FULLMASK, uu.y, 1));
        if (e2) ue2 = ex;
        if (live) {
            // column c0: E face c0 + 1 (or column 0 across a periodic wrap)
            float2 ue1 = make_float2(uu.z, uu.w);
            if (e1) ue1 = ex;
            float2 t = df_add(ue1, df_neg(make_float2(uu.x, uu.y)));
            t = df_add(t, make_float2(v1.x, v1.y));
            t = df_add(t, df_neg(make_float2(v0.x, v0.y)));
            f(c0, j, t);
            if (two) {
                float2 t1 = df_add(ue2, df_neg(make_float2(uu.z, uu.w)));
                t1 = df_add(t1, make_float2(v1.z, v1.w));
                t1 = df_add(t1, df_neg(make_float2(v0.z, v0.w)));
                f(c0 + 1, j, t1);
            }
        }
        v0 = v1;
    }
}

// Mixed init: b (double-float, kept for the outer residual), x = 0, inner
// r = hi part of b; partial b.b (the tolerance base), inner r.z and r.r
// (FP32 per lane, FP64 beyond).
__global__ void __launch_bounds__(CF_RED_THREADS) k_div_init_mixed(DivArgs a) {
    SolverState* S = a.S;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    float abb = 0.f, arz = 0.f;
    if (unit < a.U) {
        // the divergence of the velocity pairs and its scale -1/dx, in
        // double-float on the FP32 pipe
        div_pairs_unit(a, unit % a.G, unit / a.G, lane, [&](int c, int j, float2 t) {
            const size_t k = (size_t)j * a.pitch + c;
            const float2 bs = df_mul(a.mscale2, t);
            reinterpret_cast<float2*>(a.b)[k] = bs;
            // x as a double-float pair: 0, or (warm start) the previous
            // FP64 solution split in place (same 8 bytes per cell)
            reinterpret_cast<float2*>(a.x)[k] = a.warm ? df_split(a.x[k]) : make_float2(0.f, 0.f);
            const float r = bs.x;
            put_r32(a.r32, a.pitch32, a.nx, a.ny, a.per_x, a.per_y, c, j, r);
            float z = a.st.minv32[edge_bits(c, j, a.nx, a.ny, a.per_x, a.per_y)] * r;
            abb = fmaf(r, r, abb);
            arz = fmaf(r, z, arz);
        });
    }
    // inner r.r equals b.b here (the same squares in the same order)
    const double dbb = (double)warp_fold_f(abb);
    const double drz = (double)warp_fold_f(arz);
    if (unit < a.U && lane == 0) {
        a.part0[unit] = dbb;
        a.part1[unit] = drz;
    }
    if (last_block_arrive(&S->ticket[2])) {
        const double bb = final_tree(a.part0, a.U);
        const double rz = final_tree(a.part1, a.U);
        const double rr = bb;
        if (threadIdx.x == 0) {
            S->ticket[2] = 0;
            S->bb = bb;
            S->rr = bb;
            S->rr_out = bb;
            S->rho_in = rz;
            S->rr_in0 = rr;
            S->rr_in = rr;
            S->beta_in = 0.0;
            S->iter = 0;
            S->inner_iter = 0;
            S->outer_iter = 0;
            S->target2 = S->tol2 * bb;
            if (S->use_abs) S->target2 = fmax(S->target2, S->abs2 / S->area);
            S->tau2 = S->inner_tol2;
            S->restart = 1;
            S->refreshed = 1;
            if (bb == 0.0 || converged(S, bb))
                S->status = ST_CONVERGED;
            else if (isnan(bb))
                S->status = ST_NAN;
            else if (S->max_iter <= 0)
                S->status = ST_MAXIT;
            else
                S->status = ST_RUNNING;
            S->inner_status = ST_RUNNING;
        }
    }
}

// Outer refinement (reliable update): r = b - A x in double-float, x as the
// inner iterations left it; inner r = hi part.  The mixed MG-PCG with an
// update after every iteration (x_only) fuses the iteration's x += alpha p
// into it: x is read from one of two buffers and the updated x written to the
// other (SolverState::xsel names the current one), since a unit reads its
// neighbours' boundary rows while they write theirs.
struct Outer {
    int nx, ny, per_x, per_y, G, U, pitch, pitch32;
    float dfac[16];  // diagonal / scale by wall-adjacency bits
    float minv32[16];
    float2 scale;    // dt / (rho dx^2) as hi + lo
    float2* xbuf[2]; // the solution as double-float pairs: two buffers
    const float2* b;
    const float *pa, *pb;  // search directions (fused update: p of iteration it is pa when it is odd)
    float* r32;
    double *part0, *part1;
    SolverState* S;
    int gated;  // inside the MG-PCG graph: run only while the refinement is due
};

// The solution values the residual is taken of: x itself, or (fused, upd)
// x + alpha p, one df_add_f of fl32(alpha p) per cell (the x update of the
// mixed CG's K2).
struct XSrc {
    const float2* x;
    const float* p;
    float alpha;
    bool upd;
};

__device__ __forceinline__ float2 xval(const Outer& a, const XSrc& xs, int c, int j) {
    int cc = wrap_index(c, a.nx, a.per_x), jj = wrap_index(j, a.ny, a.per_y);
    if (cc < 0 || jj < 0) return make_float2(0.f, 0.f);
    const float2 v = xs.x[(size_t)jj * a.pitch + cc];
    return xs.upd ? df_add_f(v, xs.alpha * xs.p[(ptrdiff_t)jj * a.pitch32 + cc]) : v;
}

// x at columns c0, c0 + 1 of row j (wrapped row; 0 beyond a wall or past nx)
__device__ __forceinline__ float4 xrow2(const Outer& a, const XSrc& xs, int c0, int j) {
    int jj = wrap_index(j, a.ny, a.per_y);
    if (jj < 0 || c0 >= a.nx) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float2* row = xs.x + (size_t)jj * a.pitch + c0;
    const float* prow = xs.p + (ptrdiff_t)jj * a.pitch32 + c0;
    if (c0 + 1 < a.nx) {
        float4 v = *reinterpret_cast<const float4*>(row);
        if (xs.upd) {
            const float2 n0 = df_add_f(make_float2(v.x, v.y), xs.alpha * prow[0]);
            const float2 n1 = df_add_f(make_float2(v.z, v.w), xs.alpha * prow[1]);
            v = make_float4(n0.x, n0.y, n1.x, n1.y);
        }
        return v;
    }
    float2 x0 = row[0];
    if (xs.upd) x0 = df_add_f(x0, xs.alpha * prow[0]);
    return make_float4(x0.x, x0.y, 0.f, 0.f);
}

// b at columns c0, c0 + 1 of row j (owned row)
__device__ __forceinline__ float4 brow2(const Outer& a, int c0, int j) {
    if (c0 >= a.nx) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float2* row = a.b + (size_t)j * a.pitch + c0;
    if (c0 + 1 < a.nx) return *reinterpret_cast<const float4*>(row);
    const float2 b0 = row[0];
    return make_float4(b0.x, b0.y, 0.f, 0.f);
}

// a + b for double-float pairs of like magnitude, error ~2^-44 (|a| + |b|)
__device__ __forceinline__ float2 df_add_s(float2 x, float2 y) {
    float2 s = df_two_sum(x.x, y.x);
    s.y = s.y + (x.y + y.y);
    return df_quick(s.x, s.y);
}

// r = b - A x at one cell, A x = scale (dfac x_c - (x_W + x_E + x_S + x_N))
__device__ __forceinline__ float2 df_resid(const Outer& a, int eb, float2 b, float2 c, float2 w, float2 e, float2 s,
                                           float2 n) {
    float2 nb = df_add_s(w, e);
    nb = df_add_s(nb, s);
    nb = df_add_s(nb, n);
    float2 t = df_mul(make_float2(a.dfac[eb], 0.f), c);
    t = df_add_s(t, make_float2(-nb.x, -nb.y));
    float2 ax = df_mul(a.scale, t);
    return df_add_s(b, make_float2(-ax.x, -ax.y));
}

// interior cell: wall-adjacency bits 0, so the diagonal factor is 4 and
// 4 x is exact
__device__ __forceinline__ float2 df_resid_int(const Outer& a, float2 b, float2 c, float2 w, float2 e, float2 s,
                                               float2 n) {
    float2 nb = df_add_s(w, e);
    nb = df_add_s(nb, s);
    nb = df_add_s(nb, n);
    float2 t = df_add_s(make_float2(4.f * c.x, 4.f * c.y), make_float2(-nb.x, -nb.y));
    float2 ax = df_mul(a.scale, t);
    return df_add_s(b, make_float2(-ax.x, -ax.y));
}

// Two double-float values side by side, (h.x, l.x) and (h.y, l.y): a lane's
// two cells, so that each error-free step runs as one packed f32x2
// instruction for both (each half rounded as the scalar form, hence the bits
// of df_resid_int cell by cell).
struct DF2 {
    float2 h, l;
};
__device__ __forceinline__ DF2 df2_two_sum(float2 a, float2 b) {
    const float2 s = f2_add(a, b);
    const float2 bb = f2_sub(s, a);
    return DF2{s, f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb))};
}
__device__ __forceinline__ DF2 df2_quick(float2 a, float2 b) {
    const float2 s = f2_add(a, b);
    return DF2{s, f2_sub(b, f2_sub(s, a))};
}
__device__ __forceinline__ DF2 df2_add_s(DF2 x, DF2 y) {
    DF2 s = df2_two_sum(x.h, y.h);
    s.l = f2_add(s.l, f2_add(x.l, y.l));
    return df2_quick(s.h, s.l);
}
__device__ __forceinline__ DF2 df2_neg(DF2 x) {
    const float2 m = make_float2(-1.f, -1.f);
    return DF2{f2_mul(m, x.h), f2_mul(m, x.l)};
}
// df_resid_int for a lane's two cells: the residuals' high parts
__device__ __forceinline__ float2 df2_resid_int(float2 scale, DF2 b, DF2 c, DF2 w, DF2 e, DF2 s, DF2 n) {
    DF2 nb = df2_add_s(w, e);
    nb = df2_add_s(nb, s);
    nb = df2_add_s(nb, n);
    const float2 four = make_float2(4.f, 4.f);
    const DF2 t = df2_add_s(DF2{f2_mul(four, c.h), f2_mul(four, c.l)}, df2_neg(nb));
    // df_mul(scale, t)
    const float2 sh = make_float2(scale.x, scale.x), sl = make_float2(scale.y, scale.y);
    const float2 p = f2_mul(sh, t.h);
    float2 er = f2_fma(sh, t.h, f2_mul(make_float2(-1.f, -1.f), p));
    er = f2_fma(sh, t.l, er);
    er = f2_fma(sl, t.h, er);
    const DF2 ax = df2_quick(p, er);
    const DF2 r = df2_add_s(b, df2_neg(ax));
    return r.h;
}

// Interior unit (no wall next to any of its cells, whole 64-column group):
// the same arithmetic without the boundary logic.  Along a periodic axis the
// halo rows and columns are fetched from their wrapped positions, so every
// full unit of a periodic domain takes this path.  The rows arrive
// through a per-warp cp.async ring OR_RING - 1 rows ahead (group k: x (and,
// fused, p) of row j0 - 1 + k, and for the unit's own rows b; the outer
// columns' neighbours of lanes 0 and 31); each lane reads back only what it
// copied.  Slot layout (floats): x row [0, 128), b row [128, 256), the edge
// x pairs of lanes 0 / 31 at 256 / 258, p row [264, 328), edge p at 328 / 329.
constexpr int OR_RING = 4;
template <bool FUSED>
struct OrSlot {
    static constexpr int value = FUSED ? 332 : 264;  // 16-byte multiples
};
template <bool FUSED>
__device__ __forceinline__ void outer_unit_interior(const Outer& a, const XSrc& xs, float2* xo, float* ring, int lane,
                                                    int c0, int j0, int j1, float& arz, float& arr) {
    constexpr int SLOT = OrSlot<FUSED>::value;
    const bool upd = FUSED && xs.upd;
    const float m0 = a.minv32[0];
    const bool edge = lane == 0 || lane == 31;
    int ec = lane == 0 ? c0 - 1 : c0 + 2;  // outer neighbour column of lanes 0 and 31 (wrapped)
    ec = ec < 0 ? ec + a.nx : (ec >= a.nx ? ec - a.nx : ec);
    // periodic ghost copies of r: columns 0 and nx - 1, rows 0 and ny - 1
    const bool gx0 = a.per_x && c0 == 0, gx1 = a.per_x && c0 + 2 == a.nx;
    const bool ghosts = __any_sync(FULLMASK, gx0 || gx1) || (a.per_y && (j0 == 0 || j1 == a.ny));
    const int eo = 256 + (lane == 31 ? 2 : 0);
    const int eop = 328 + (lane == 31 ? 1 : 0);
    const int last = j1;                         // groups cover rows j0 - 1 .. j1
    auto issue = [&](int k) {
        const int row = j0 - 1 + k;
        float* sl = ring + (k % OR_RING) * SLOT;
        if (row <= last) {
            const int pr = row < 0 ? row + a.ny : (row >= a.ny ? row - a.ny : row);  // wrapped halo row
            const size_t o = (size_t)pr * a.pitch;
            cpa16(sl + 4 * lane, xs.x + o + c0);
            if (upd) cpa8(sl + 264 + 2 * lane, xs.p + (ptrdiff_t)pr * a.pitch32 + c0);
            if (row >= j0 && row < j1) cpa16(sl + 128 + 4 * lane, a.b + o + c0);
            if (edge) {
                cpa8(sl + eo, xs.x + o + ec);
                if (upd) cpa4(sl + eop, xs.p + (ptrdiff_t)pr * a.pitch32 + ec);
            }
        }
        cpa_commit();
    };
    auto xrow = [&](int k) {
        const float* sl = ring + (k % OR_RING) * SLOT;
        float4 v = *reinterpret_cast<const float4*>(sl + 4 * lane);
        if (upd) {
            const float2 pv = *reinterpret_cast<const float2*>(sl + 264 + 2 * lane);
            const float2 n0 = df_add_f(make_float2(v.x, v.y), xs.alpha * pv.x);
            const float2 n1 = df_add_f(make_float2(v.z, v.w), xs.alpha * pv.y);
            v = make_float4(n0.x, n0.y, n1.x, n1.y);
        }
        return v;
    };
    auto brow = [&](int k) {
        return *reinterpret_cast<const float4*>(ring + (k % OR_RING) * SLOT + 128 + 4 * lane);
    };
    auto erow = [&](int k) {
        if (!edge) return make_float2(0.f, 0.f);
        const float* sl = ring + (k % OR_RING) * SLOT;
        float2 v = *reinterpret_cast<const float2*>(sl + eo);
        if (upd) v = df_add_f(v, xs.alpha * sl[eop]);
        return v;
    };
#pragma unroll
    for (int k = 0; k < OR_RING - 1; ++k) issue(k);
    issue(OR_RING - 1);
    cpa_wait<OR_RING - 1>();
    float4 xm = xrow(0);  // row j0 - 1
    issue(OR_RING);
    cpa_wait<OR_RING - 1>();
    float4 xc = xrow(1), bv = brow(1);  // row j0
    float2 ev = erow(1);
    for (int j = j0; j < j1; ++j) {
        const int k = j - j0 + 2;  // group of row j + 1
        if (upd) *reinterpret_cast<float4*>(xo + (size_t)j * a.pitch + c0) = xc;
        issue(k + OR_RING - 1);
        cpa_wait<OR_RING - 1>();
        const float4 xp = xrow(k), bn = brow(k);
        const float2 en = erow(k);
        float2 left = make_float2(__shfl_up_sync(FULLMASK, xc.z, 1), __shfl_up_sync(FULLMASK, xc.w, 1));
        float2 right = make_float2(__shfl_down_sync(FULLMASK, xc.x, 1), __shfl_down_sync(FULLMASK, xc.y, 1));
        if (lane == 0) left = ev;
        if (lane == 31) right = ev;
        // cell c0: W = left, E = the lane's second cell; cell c0 + 1: W = the
        // first cell, E = right
        const float2 rr2 = df2_resid_int(a.scale, DF2{make_float2(bv.x, bv.z), make_float2(bv.y, bv.w)},
                                         DF2{make_float2(xc.x, xc.z), make_float2(xc.y, xc.w)},
                                         DF2{make_float2(left.x, xc.x), make_float2(left.y, xc.y)},
                                         DF2{make_float2(xc.z, right.x), make_float2(xc.w, right.y)},
                                         DF2{make_float2(xm.x, xm.z), make_float2(xm.y, xm.w)},
                                         DF2{make_float2(xp.x, xp.z), make_float2(xp.y, xp.w)});
        const float2 r0 = make_float2(rr2.x, 0.f), r1 = make_float2(rr2.y, 0.f);
        *reinterpret_cast<float2*>(a.r32 + (ptrdiff_t)j * a.pitch32 + c0) = make_float2(r0.x, r1.x);
        if (ghosts) {  // periodic copies of boundary cells, as put_r32 writes them
            float* row = a.r32 + (ptrdiff_t)j * a.pitch32;
            if (gx0) row[a.nx] = r0.x;
            if (gx1) row[-1] = r1.x;
            if (a.per_y && j == 0) {
                a.r32[(ptrdiff_t)a.ny * a.pitch32 + c0] = r0.x;
                a.r32[(ptrdiff_t)a.ny * a.pitch32 + c0 + 1] = r1.x;
            }
            if (a.per_y && j == a.ny - 1) {
                a.r32[-(ptrdiff_t)a.pitch32 + c0] = r0.x;
                a.r32[-(ptrdiff_t)a.pitch32 + c0 + 1] = r1.x;
            }
        }
        arz = fmaf(r0.x, m0 * r0.x, arz);
        arr = fmaf(r0.x, r0.x, arr);
        arz = fmaf(r1.x, m0 * r1.x, arz);
        arr = fmaf(r1.x, r1.x, arr);
        xm = xc;
        xc = xp;
        bv = bn;
        ev = en;
    }
    cpa_wait<0>();
}

// One warp per unit of 64 columns x 16 rows, lane l on columns 2l, 2l + 1;
// rows slide through registers, W/E neighbours come by shuffle.  FUSED: the
// x update of the iteration first (when the inner step did not break down),
// the updated x written to the other buffer.
template <bool FUSED>
__global__ void __launch_bounds__(CF_RED_THREADS) k_outer_resid(Outer a) {
    SolverState* S = a.S;
    __shared__ int mode_s, sel_s, it_s;
    __shared__ float alpha_s;
    if (threadIdx.x == 0) {
        const int st = *(volatile const int*)&S->status, ist = *(volatile const int*)&S->inner_status;
        int mode;  // 0: nothing to do, 1: residual of x, 2: x update and residual
        if (FUSED)
            mode = st != ST_RUNNING ? 0 : (ist == ST_RUNNING ? 2 : 1);
        else
            mode = (!a.gated || (st == ST_RUNNING && ist != ST_RUNNING)) ? 1 : 0;
        mode_s = mode;
        sel_s = S->xsel;
        it_s = S->inner_iter;
        alpha_s = (float)S->alpha_in;
    }
    __syncthreads();
    const int mode = mode_s;
    if (mode == 0) return;
    const int sel = sel_s, it = it_s;
    const XSrc xs{a.xbuf[sel], (it & 1) ? a.pa : a.pb, alpha_s, FUSED && mode == 2};
    float2* xo = a.xbuf[sel ^ 1];
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    float arz = 0.f, arr = 0.f;
    // Units next to a wall along x (column groups 0 and G - 1) take the
    // general path, several times slower than the interior one: they are
    // numbered first, two per row band, so that they fill blocks of their own
    // and no interior warp waits for one at the end-of-block barrier.
    int g, band;
    if (!a.per_x && a.G > 2) {
        const int nb = 2 * (a.U / a.G);
        if (unit < nb) {
            band = unit >> 1;
            g = (unit & 1) ? a.G - 1 : 0;
        } else {
            band = (unit - nb) / (a.G - 2);
            g = 1 + (unit - nb) % (a.G - 2);
        }
    } else {
        g = unit % a.G;
        band = unit / a.G;
    }
    const int j0u = band * CF_BAND_ROWS, j1u = min(j0u + CF_BAND_ROWS, a.ny);
    // rows j0u - 1 .. j1u and columns g * 64 - 1 .. g * 64 + 64 are read:
    // inside the domain, or wrapped along a periodic axis
    const bool full_x = (g + 1) * CF_UNIT_COLS <= a.nx;
    const bool interior = unit < a.U && full_x &&
                          (a.per_x || (g * CF_UNIT_COLS >= 1 && (g + 1) * CF_UNIT_COLS + 1 <= a.nx)) &&
                          (a.per_y || (j0u >= 1 && j1u + 2 <= a.ny));
    __shared__ __align__(16) float ring[CF_RED_WARPS * OR_RING * OrSlot<FUSED>::value];
    if (interior) {
        outer_unit_interior<FUSED>(a, xs, xo, ring + (threadIdx.x >> 5) * OR_RING * OrSlot<FUSED>::value, lane,
                                   g * CF_UNIT_COLS + 2 * lane, j0u, j1u, arz, arr);
    } else if (unit < a.U) {
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = j0u;
        const int j1 = j1u;
        // rows j - 1, j, j + 1 in registers; row j + 2 and b of row j + 1 are
        // fetched one row ahead, so the loads overlap the arithmetic
        float4 xm = xrow2(a, xs, c0, j0 - 1), xc = xrow2(a, xs, c0, j0), xp = xrow2(a, xs, c0, j0 + 1);
        float4 bnext = brow2(a, c0, j0);
        for (int j = j0; j < j1; ++j) {
            const float4 xpp = xrow2(a, xs, c0, j + 2);
            const float4 bv = bnext;
            if (j + 1 < j1) bnext = brow2(a, c0, j + 1);
            float2 left = make_float2(__shfl_up_sync(FULLMASK, xc.z, 1), __shfl_up_sync(FULLMASK, xc.w, 1));
            float2 right = make_float2(__shfl_down_sync(FULLMASK, xc.x, 1), __shfl_down_sync(FULLMASK, xc.y, 1));
            if (lane == 0) left = xval(a, xs, c0 - 1, j);
            if (lane == 31 || c0 + 2 >= a.nx) right = xval(a, xs, c0 + 2, j);
            float2 mid1 = make_float2(xc.z, xc.w);
            if (c0 + 1 >= a.nx) mid1 = xval(a, xs, c0 + 1, j);  // E neighbour of the last column
            if (c0 < a.nx) {
                if (xs.upd) xo[(size_t)j * a.pitch + c0] = make_float2(xc.x, xc.y);
                const int eb = edge_bits(c0, j, a.nx, a.ny, a.per_x, a.per_y);
                const float2 r = df_resid(a, eb, make_float2(bv.x, bv.y), make_float2(xc.x, xc.y), left, mid1,
                                          make_float2(xm.x, xm.y), make_float2(xp.x, xp.y));
                put_r32(a.r32, a.pitch32, a.nx, a.ny, a.per_x, a.per_y, c0, j, r.x);
                arz = fmaf(r.x, a.minv32[eb] * r.x, arz);
                arr = fmaf(r.x, r.x, arr);
            }
            if (c0 + 1 < a.nx) {
                if (xs.upd) xo[(size_t)j * a.pitch + c0 + 1] = make_float2(xc.z, xc.w);
                const int eb = edge_bits(c0 + 1, j, a.nx, a.ny, a.per_x, a.per_y);
                const float2 r = df_resid(a, eb, make_float2(bv.z, bv.w), make_float2(xc.z, xc.w),
                                          make_float2(xc.x, xc.y), right, make_float2(xm.z, xm.w),
                                          make_float2(xp.z, xp.w));
                put_r32(a.r32, a.pitch32, a.nx, a.ny, a.per_x, a.per_y, c0 + 1, j, r.x);
                arz = fmaf(r.x, a.minv32[eb] * r.x, arz);
                arr = fmaf(r.x, r.x, arr);
            }
            xm = xc;
            xc = xp;
            xp = xpp;
        }
    }
    const double drz = (double)warp_fold_f(arz), drr = (double)warp_fold_f(arr);
    if (unit < a.U && lane == 0) {
        a.part0[unit] = drr;
        a.part1[unit] = drz;
    }
    if (last_block_arrive(&S->ticket[4])) {
        const double rr64 = final_tree(a.part0, a.U);
        const double rz = final_tree(a.part1, a.U);
        const double rr = rr64;
        if (threadIdx.x == 0) {
            S->ticket[4] = 0;
            if (FUSED && mode == 2) {
                // the end of the inner step (as K2 ends it)
                S->rho_prev = S->rho_in;
                S->inner_iter = it + 1;
                S->iter = S->iter + 1;
                S->inner_status = ST_CONVERGED;
                S->xsel = sel ^ 1;
            }
            S->outer_iter += 1;
            S->rr = rr64;
            S->rr_out = rr64;
            if (isnan(rr64))
                S->status = ST_NAN;
            else if (converged(S, rr64))
                S->status = ST_CONVERGED;
            else if (S->iter >= S->max_iter || S->outer_iter >= S->max_outer)
                S->status = ST_MAXIT;
            else {
                // residual replacement: keep the search direction, rescale beta
                // to the replaced residual (restart only after an FP32 breakdown)
                if (S->inner_status == ST_BREAKDOWN) {
                    S->restart = 1;
                    S->beta_in = 0.0;
                } else {
                    S->beta_in = rz / S->rho_prev;
                }
                S->rho_in = rz;
                S->rr_in0 = rr;
                S->rr_in = rr;
                S->refreshed = 1;
                S->inner_status = ST_RUNNING;
            }
        }
    }
}

// mixed: the double-float solution (in the buffer SolverState::xsel names)
// to FP64 in the first buffer, for the gradient
__global__ void k_df_to_f64(double* x, const float2* xb, const SolverState* S, int nx, int ny, int pitch) {
    int gi = blockIdx.x * blockDim.x + threadIdx.x;
    int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nx || gj >= ny) return;
    const float2* src = S->xsel ? xb : reinterpret_cast<const float2*>(x);
    const size_t k = (size_t)gj * pitch + gi;
    const float2 v = src[k];
    x[k] = f2d_exact(v.x) + f2d_exact(v.y);
}

// the same into out (owned cells, row pitch nx), for a download
__global__ void k_df_to_f64_out(const float2* x, const float2* xb, const SolverState* S, int nx, int ny, int pitch,
                                double* out) {
    int gi = blockIdx.x * blockDim.x + threadIdx.x;
    int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nx || gj >= ny) return;
    const float2 v = (S->xsel ? xb : x)[(size_t)gj * pitch + gi];
    out[(size_t)gj * nx + gi] = f2d_exact(v.x) + f2d_exact(v.y);
}

// --------------------------------------------------------------------------
// _applyPressure (:214-264).  z = 0: I-faces, z = 1: J-faces.  Quirk Q1 (the
// J-face wall condition lands on u, :260) zeroes u in row 0 (done in the
// I-face pass, which owns u) and u's ghost row ny (done in the J-face pass).
struct Press {
    Phys p;
    Grid<double> u, v;
    const double* x;
    int pitch;
    double ms;    // -(dt / (density dx))
    int adjoint;  // 1: transpose of the projection (masks applied by the caller, none here)
    // mixed (pairs = 1): u, v hold double-float pairs and the solution is read
    // as pairs from the buffer SolverState::xsel names (x or xb); the update
    // u + ms (p(c) - p(n)) runs in double-float on the FP32 pipe (ms2 = ms as
    // a pair)
    int pairs;
    float2 ms2;
    const float2* xb;
    const SolverState* S;
};

__device__ __forceinline__ double pval(const Press& a, int gi, int gj) {
    int ci = wrap_index(gi, a.p.nx, a.p.per_x), cj = wrap_index(gj, a.p.ny, a.p.per_y);
    if (ci < 0 || cj < 0) return 0.0;
    return a.x[(size_t)cj * a.pitch + ci];
}

__device__ __forceinline__ float2 pval_df(const Press& a, const float2* x, int gi, int gj) {
    int ci = wrap_index(gi, a.p.nx, a.p.per_x), cj = wrap_index(gj, a.p.ny, a.p.per_y);
    if (ci < 0 || cj < 0) return make_float2(0.f, 0.f);
    return x[(size_t)cj * a.pitch + ci];
}

// w + ms (p(c) - p(n)): FP64 as the reference writes it (one rounding per
// operation; ms = -scale), or (pairs) on the pair stored in w's 8 bytes
__device__ __forceinline__ double press_update(const Press& a, const float2* xdf, double w, int ci, int cj, int ni,
                                               int nj) {
    if (a.pairs) {
        const float2 pc = pval_df(a, xdf, ci, cj), pn = pval_df(a, xdf, ni, nj);
        const float2 m = df_mul(a.ms2, df_add_s(pc, make_float2(-pn.x, -pn.y)));
        const float2 r = df_add(reinterpret_cast<const float2&>(w), m);
        return __hiloint2double(__float_as_int(r.y), __float_as_int(r.x));  // the pair's 8 bytes
    }
    const double d = pval(a, ci, cj) - pval(a, ni, nj);
    return __dadd_rn(w, __dmul_rn(a.ms, d));
}

// One face: I face (axis 0) or J face (axis 1) of index (gi, gj), with the
// reference's wall rules (src/VelocityCorrector.hpp:245-262).  (A zero
// written to u or v is the pair (0, 0) as well.)
__device__ __forceinline__ void apply_face(const Press& a, const float2* xdf, int axis, int gi, int gj) {
    const Phys& p = a.p;
    const bool fix_q1 = (p.quirks & 1u) != 0;
    if (axis == 0) {
        double& u = a.u.at(gi + CF_HALO, gj + CF_HALO);
        // u -= scale * (p(i) - p(i-1)) (src/VelocityCorrector.hpp:245)
        double w = press_update(a, xdf, u, gi, gj, gi - 1, gj);
        if (!a.adjoint) {
            if (!p.per_x) {
                if (gi <= 0 && p.bc[0] == 0) w = 0.0;
                if (gi > p.nx - 1 && p.bc[2] == 0) w = 0.0;
            }
            if (!fix_q1 && !p.per_y && gj == 0 && gi < p.nx && p.bc[1] == 0) w = 0.0;
        }
        u = w;
    } else {
        double& v = a.v.at(gi + CF_HALO, gj + CF_HALO);
        double w = press_update(a, xdf, v, gi, gj, gi, gj - 1);  // :256
        if (!p.per_y && !a.adjoint) {
            if (fix_q1) {
                if (gj <= 0 && p.bc[1] == 0) w = 0.0;
                if (gj > p.ny - 1 && p.bc[3] == 0) w = 0.0;
            } else if (gj > p.ny - 1 && p.bc[3] == 0) {
                a.u.at(gi + CF_HALO, gj + CF_HALO) = 0.0;  // u ghost row ny
            }
        }
        v = w;
    }
}

__device__ __forceinline__ const float2* press_pairs(const Press& a) {
    return a.pairs ? (a.S->xsel ? a.xb : reinterpret_cast<const float2*>(a.x)) : nullptr;
}

// One thread per (I-face, J-face) of index (gi, gj), both axes in the same
// block so that a tile's pressure is read from memory once.  The FP64
// gradient, and every face of the mixed one under cf_test_apply_general.
__global__ void k_apply_pressure(Press a) {
    const Phys& p = a.p;
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    const float2* xdf = press_pairs(a);
#pragma unroll 1
    for (int axis = 0; axis < 2; ++axis) {
        const int ox = p.nx + ((axis == 0 && !p.per_x) ? 1 : 0);
        const int oy = p.ny + ((axis == 1 && !p.per_y) ? 1 : 0);
        if (gi >= ox || gj >= oy) continue;
        apply_face(a, xdf, axis, gi, gj);
    }
}

// The mixed gradient on the faces of the owned cells (I faces 0 .. nx - 1, J
// faces 0 .. ny - 1), one warp per 64-column x 16-row unit as the divergence
// kernels: lane l updates the I and J faces of columns c0 = 64 g + 2 l and
// c0 + 1 row by row, each row's solution, u and v pairs as 16-byte vectors
// (the next row's loaded before this row's stores); p(c0 - 1) comes from the
// previous lane (lane 0 reads it: its wrap, or 0 beyond a wall) and p(j - 1)
// from the previous row.  The same operations in the same order as
// press_update and apply_face, so the same bits as k_apply_pressure; the faces
// past the last cell of a walled axis are k_apply_edges'.
__global__ void __launch_bounds__(CF_RED_THREADS) k_apply_pairs(Press a, int G, int U) {
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    if (unit >= U) return;  // warp-uniform; no block barrier below
    const Phys& p = a.p;
    const int g = unit % G, band = unit / G;
    const int c0 = g * CF_UNIT_COLS + 2 * lane;
    const int j0 = band * CF_BAND_ROWS, j1 = min(j0 + CF_BAND_ROWS, p.ny);
    const float2* xdf = press_pairs(a);
    const bool live = c0 < p.nx, two = c0 + 1 < p.nx;
    const bool fix_q1 = (p.quirks & 1u) != 0;
    const bool walls = !a.adjoint;
    // I face 0 of a walled x axis; the I faces of row 0 (unfixed Q1 quirk)
    // and the J faces of row 0 (fixed) of a walled y axis
    const bool zero_w = walls && !p.per_x && p.bc[0] == 0 && c0 == 0;
    const bool zero_u0 = walls && !fix_q1 && !p.per_y && p.bc[1] == 0;
    const bool zero_v0 = walls && fix_q1 && !p.per_y && p.bc[1] == 0;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    auto xrow = [&](int j) { return live ? *reinterpret_cast<const float4*>(&xdf[(size_t)j * a.pitch + c0]) : zero4; };
    auto frow = [&](const Grid<double>& f, int j) {
        return live ? *reinterpret_cast<const float4*>(&f.at(c0 + CF_HALO, j + CF_HALO)) : zero4;
    };
    auto west = [&](int j) { return (lane == 0 && live) ? pval_df(a, xdf, c0 - 1, j) : make_float2(0.f, 0.f); };
    auto upd = [&](float x0, float x1, float pc0, float pc1, float pn0, float pn1) {
        const float2 m = df_mul(a.ms2, df_add_s(make_float2(pc0, pc1), make_float2(-pn0, -pn1)));
        return df_add(make_float2(x0, x1), m);
    };
    // p(j0 - 1): the row below, its wrap, or 0 beyond a wall
    float4 xs = j0 > 0 ? xrow(j0 - 1) : (p.per_y ? xrow(p.ny - 1) : zero4);
    float4 xn = xrow(j0), un = frow(a.u, j0), vn = frow(a.v, j0);
    float2 wn = west(j0);
    for (int j = j0; j < j1; ++j) {
        const float4 xc = xn, uu = un, vv = vn;
        float2 xw = make_float2(__shfl_up_sync(FULLMASK, xc.z, 1), __shfl_up_sync(FULLMASK, xc.w, 1));
        if (lane == 0) xw = wn;
        if (j + 1 < j1) {
            xn = xrow(j + 1);
            un = frow(a.u, j + 1);
            vn = frow(a.v, j + 1);
            wn = west(j + 1);
        }
        if (!live) continue;
        float2 u0 = upd(uu.x, uu.y, xc.x, xc.y, xw.x, xw.y);
        float2 u1 = upd(uu.z, uu.w, xc.z, xc.w, xc.x, xc.y);
        float2 v0 = upd(vv.x, vv.y, xc.x, xc.y, xs.x, xs.y);
        float2 v1 = upd(vv.z, vv.w, xc.z, xc.w, xs.z, xs.w);
        if (zero_w) u0 = make_float2(0.f, 0.f);
        if (j == 0 && zero_u0) u0 = u1 = make_float2(0.f, 0.f);
        if (j == 0 && zero_v0) v0 = v1 = make_float2(0.f, 0.f);
        float2* pu = reinterpret_cast<float2*>(&a.u.at(c0 + CF_HALO, j + CF_HALO));
        float2* pv = reinterpret_cast<float2*>(&a.v.at(c0 + CF_HALO, j + CF_HALO));
        if (two) {
            *reinterpret_cast<float4*>(pu) = make_float4(u0.x, u0.y, u1.x, u1.y);
            *reinterpret_cast<float4*>(pv) = make_float4(v0.x, v0.y, v1.x, v1.y);
        } else {
            pu[0] = u0;
            pv[0] = v0;
        }
        xs = xc;
    }
}

// The faces past the last cell of a walled axis (I face nx of rows 0 ..
// ny - 1, J face ny of columns 0 .. nx - 1): thread t takes one of each.
__global__ void k_apply_edges(Press a) {
    const Phys& p = a.p;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const float2* xdf = press_pairs(a);
    if (!p.per_x && t < p.ny) apply_face(a, xdf, 0, p.nx, t);
    if (!p.per_y && t < p.nx) apply_face(a, xdf, 1, t, p.ny);
}

// The mixed gradient of k_apply_pairs fused with the divergence norms of its
// result (k_div_norms' mixed form), for a grid periodic along both axes (no
// wall rule, no face past the last cell).  A lane's divergences need two faces
// that other warps update in place: the I face east of the warp (the next
// unit's west column, or column 0 across the wrap) and the J faces above the
// unit (the next band's south row, or row 0).  Their values before the
// gradient were saved by k_div_init_mixed (d.ubnd, d.vbnd); the lane updates
// them itself with the owner's operands, so it holds the owner's bits.  The
// J faces of row j + 1 are updated one row ahead and carried, and each cell's
// divergence, square and magnitude are taken in k_div_norms' operation order,
// lane order and folds: the same stored faces and the same norms.
__global__ void __launch_bounds__(CF_RED_THREADS, 4) k_apply_pairs_norms(Press a, DivArgs d) {
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    float fss = 0.f, fmx = 0.f;
    if (unit < d.U) {  // warp-uniform
        const int nx = a.p.nx, ny = a.p.ny;
        const int g = unit % d.G, band = unit / d.G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS, j1 = min(j0 + CF_BAND_ROWS, ny);
        const int jn = j1 == ny ? 0 : j1;  // the row above the unit
        const float2* xdf = press_pairs(a);
        const bool live = c0 < nx, two = c0 + 1 < nx;
        // the lane whose east face is another warp's: the warp's last lane
        // (column ie = c0 + 2) or the domain's last column (ie = 0)
        const bool e2 = live && two && (lane == 31 || c0 + 2 >= nx);
        const bool e1 = live && !two;
        const int ie = (e2 && c0 + 2 < nx) ? c0 + 2 : 0;
        const float2* ub = d.ubnd + (size_t)(ie / CF_UNIT_COLS) * ny;
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        auto xrow = [&](int j) {
            return live ? *reinterpret_cast<const float4*>(&xdf[(size_t)j * a.pitch + c0]) : zero4;
        };
        auto frow = [&](const Grid<double>& f, int j) {
            return live ? *reinterpret_cast<const float4*>(&f.at(c0 + CF_HALO, j + CF_HALO)) : zero4;
        };
        auto west = [&](int j) { return (lane == 0 && live) ? pval_df(a, xdf, c0 - 1, j) : make_float2(0.f, 0.f); };
        // the saved east face (before the gradient) and p at its column
        auto halo = [&](int j) {
            if (!(e1 || e2)) return zero4;
            const float2 uo = ub[j], xo = xdf[(size_t)j * a.pitch + ie];
            return make_float4(uo.x, uo.y, xo.x, xo.y);
        };
        auto upd = [&](float x0, float x1, float pc0, float pc1, float pn0, float pn1) {
            const float2 m = df_mul(a.ms2, df_add_s(make_float2(pc0, pc1), make_float2(-pn0, -pn1)));
            return df_add(make_float2(x0, x1), m);
        };
        // the J faces of row j0 (p of the row below: its wrap)
        const float4 xs = xrow(j0 > 0 ? j0 - 1 : ny - 1);
        float4 xc = xrow(j0), uu = frow(a.u, j0);
        const float4 vv = frow(a.v, j0);
        float2 wc = west(j0);
        float4 hc = halo(j0);
        float2 vs0 = upd(vv.x, vv.y, xc.x, xc.y, xs.x, xs.y);
        float2 vs1 = upd(vv.z, vv.w, xc.z, xc.w, xs.z, xs.w);
        for (int j = j0; j < j1; ++j) {
            float4 xn, un = zero4, vn, hn = zero4;
            float2 wn = make_float2(0.f, 0.f);
            if (j + 1 < j1) {
                xn = xrow(j + 1);
                un = frow(a.u, j + 1);
                vn = frow(a.v, j + 1);
                wn = west(j + 1);
                hn = halo(j + 1);
            } else {
                // the row above the unit: p, and the J faces as saved
                xn = xrow(jn);
                const float2* vb = d.vbnd + (size_t)(jn / CF_BAND_ROWS) * nx + c0;
                const float2 b0 = live ? vb[0] : make_float2(0.f, 0.f);
                const float2 b1 = two ? vb[1] : make_float2(0.f, 0.f);
                vn = make_float4(b0.x, b0.y, b1.x, b1.y);
            }
            float2 xw = make_float2(__shfl_up_sync(FULLMASK, xc.z, 1), __shfl_up_sync(FULLMASK, xc.w, 1));
            if (lane == 0) xw = wc;
            const float2 u0 = upd(uu.x, uu.y, xc.x, xc.y, xw.x, xw.y);
            const float2 u1 = upd(uu.z, uu.w, xc.z, xc.w, xc.x, xc.y);
            // the J faces of row j + 1
            const float2 vn0 = upd(vn.x, vn.y, xn.x, xn.y, xc.x, xc.y);
            const float2 vn1 = upd(vn.z, vn.w, xn.z, xn.w, xc.z, xc.w);
            // the east faces: the next lane's first I face, or the saved one
            // updated here (p west of it: the lane's last column)
            float2 ue2 = make_float2(__shfl_down_sync(FULLMASK, u0.x, 1), __shfl_down_sync(FULLMASK, u0.y, 1));
            float2 uh = make_float2(0.f, 0.f);
            if (e1 || e2) uh = upd(hc.x, hc.y, hc.z, hc.w, e2 ? xc.z : xc.x, e2 ? xc.w : xc.y);
            if (e2) ue2 = uh;
            if (live) {
                float2* pu = reinterpret_cast<float2*>(&a.u.at(c0 + CF_HALO, j + CF_HALO));
                float2* pv = reinterpret_cast<float2*>(&a.v.at(c0 + CF_HALO, j + CF_HALO));
                if (two) {
                    *reinterpret_cast<float4*>(pu) = make_float4(u0.x, u0.y, u1.x, u1.y);
                    *reinterpret_cast<float4*>(pv) = make_float4(vs0.x, vs0.y, vs1.x, vs1.y);
                } else {
                    pu[0] = u0;
                    pv[0] = vs0;
                }
                const float2 ue1 = two ? u1 : uh;
                float2 t = df_add(ue1, df_neg(u0));
                t = df_add(t, vn0);
                t = df_add(t, df_neg(vs0));
                float bf = t.x * d.mscale32;
                fss = fmaf(bf, bf, fss);
                fmx = fmaxf(fmx, fabsf(bf));
                if (two) {
                    float2 t1 = df_add(ue2, df_neg(u1));
                    t1 = df_add(t1, vn1);
                    t1 = df_add(t1, df_neg(vs1));
                    bf = t1.x * d.mscale32;
                    fss = fmaf(bf, bf, fss);
                    fmx = fmaxf(fmx, fabsf(bf));
                }
            }
            xc = xn;
            uu = un;
            wc = wn;
            hc = hn;
            vs0 = vn0;
            vs1 = vn1;
        }
    }
    double ass = warp_fold((double)fss);
    double amx = warp_max((double)fmx);
    if (unit < d.U && lane == 0) {
        d.part0[unit] = ass;
        d.part1[unit] = amx;
    }
    if (last_block_arrive(&d.S->ticket[3])) {
        const double ss = final_tree(d.part0, d.U);
        const double mx = final_max(d.part1, d.U);
        if (threadIdx.x == 0) {
            d.S->ticket[3] = 0;
            d.out[0] = ss;
            d.out[1] = mx;
        }
    }
}

// ||div u||: canonical sum of b^2 and max |b|
__global__ void __launch_bounds__(CF_RED_THREADS) k_div_norms(DivArgs a) {
    SolverState* S = a.S;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    double ass = 0.0, amx = 0.0;
    float fss = 0.f, fmx = 0.f;
    if (unit < a.U && a.mixed) {
        // the divergence of the pairs, then its square and magnitude in FP32
        div_pairs_unit(a, unit % a.G, unit / a.G, lane, [&](int, int, float2 t) {
            const float bf = t.x * a.mscale32;
            fss = fmaf(bf, bf, fss);
            fmx = fmaxf(fmx, fabsf(bf));
        });
    } else if (unit < a.U) {
        const int g = unit % a.G, band = unit / a.G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS;
        const int j1 = min(j0 + CF_BAND_ROWS, a.ny);
        for (int j = j0; j < j1; ++j)
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                int c = c0 + s;
                if (c >= a.nx) continue;
                double b = div_b(a, c, j);
                ass = fma(b, b, ass);
                amx = fmax(amx, fabs(b));
            }
    }
    if (a.mixed) {
        ass = (double)fss;
        amx = (double)fmx;
    }
    ass = warp_fold(ass);
    amx = warp_max(amx);
    if (unit < a.U && lane == 0) {
        a.part0[unit] = ass;
        a.part1[unit] = amx;
    }
    if (last_block_arrive(&S->ticket[3])) {
        double ss = final_tree(a.part0, a.U);
        double mx = final_max(a.part1, a.U);
        if (threadIdx.x == 0) {
            S->ticket[3] = 0;
            a.out[0] = ss;
            a.out[1] = mx;
        }
    }
}

// --------------------------------------------------------------------------
// host side
static DivArgs div_args(cf_ctx* c, const Stencil& st) {
    DivArgs a{};
    a.nx = c->ph.nx;
    a.ny = c->ph.ny;
    a.per_x = c->ph.per_x;
    a.per_y = c->ph.per_y;
    a.G = c->G;
    a.U = c->n_units;
    a.pitch = c->vpitch;
    a.pitch32 = c->p32;
    a.u = c->u[c->cur];
    a.v = c->v[c->cur];
    a.mscale = -(1.0 / c->ph.dx);
    a.mixed = c->precision == CF_PREC_MIXED;
    a.mscale32 = (float)a.mscale;
    a.mscale2 = make_float2(a.mscale32, (float)(a.mscale - (double)a.mscale32));
    a.st = st;
    a.x = c->x.a;
    a.r = c->r.a;
    a.b = c->b.a;
    a.r32 = c->r32.a;
    a.part0 = c->partials;
    a.part1 = c->partials + c->n_units;
    a.out = c->d_out;
    a.S = c->S;
    return a;
}

// the gradient subtraction's arguments (mixed: on pairs, from the
// double-float solution)
static Press press_args(cf_ctx* c, double dt, Grid<double> gu, Grid<double> gv, int adjoint) {
    Press pa{};
    pa.p = c->ph;
    pa.u = gu;
    pa.v = gv;
    pa.x = c->x.a;
    pa.pitch = c->vpitch;
    pa.ms = -(dt / (c->density * c->ph.dx));
    pa.adjoint = adjoint;
    pa.pairs = c->precision == CF_PREC_MIXED ? 1 : 0;
    const float hi = (float)pa.ms;
    pa.ms2 = make_float2(hi, (float)(pa.ms - (double)hi));
    pa.xb = reinterpret_cast<const float2*>(c->xb.a);
    pa.S = c->S;
    return pa;
}

static Cg64 cg64_args(cf_ctx* c, const Stencil& st) {
    Cg64 a{};
    a.nx = c->ph.nx;
    a.ny = c->ph.ny;
    a.per_x = c->ph.per_x;
    a.per_y = c->ph.per_y;
    a.G = c->G;
    a.U = c->n_units;
    a.pitch = c->vpitch;
    a.st = st;
    a.x = c->x.a;
    a.r = c->r.a;
    a.pa = c->pa.a;
    a.pb = c->pb.a;
    a.qv = c->qv.a;
    a.part0 = c->partials;
    a.part1 = c->partials + c->n_units;
    a.S = c->S;
    return a;
}

static int red_blocks(const cf_ctx* c) { return (c->n_units + CF_RED_WARPS - 1) / CF_RED_WARPS; }

// The mixed projection of a grid periodic along both axes takes its
// divergence norms inside the gradient (k_apply_pairs_norms), from faces
// that k_div_init_mixed saves (the adjoint's projections take no norms).
static bool fused_norms(const cf_ctx* c, bool mixed, int adjoint) {
    return mixed && !adjoint && c->ph.per_x && c->ph.per_y && !c->test_general_apply;
}
static void save_bounds(const cf_ctx* c, DivArgs* da) {
    da->ubnd = reinterpret_cast<float2*>(c->bnd);
    da->vbnd = da->ubnd + (size_t)c->G * c->ph.ny;
}

// The pressure gradient: with norms (fused_norms), k_apply_pairs_norms; the
// mixed one as k_apply_pairs over the owned faces plus k_apply_edges on a
// walled axis; the FP64 one (and the mixed one under cf_test_apply_general)
// as k_apply_pressure.  Returns the launches made.
static int launch_apply(cf_ctx* c, const Press& pa, const DivArgs* norms = nullptr) {
    if (norms) {
        k_apply_pairs_norms<<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(pa, *norms);
        return 1;
    }
    if (pa.pairs && !c->test_general_apply) {
        k_apply_pairs<<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(pa, c->G, c->n_units);
        if (c->ph.per_x && c->ph.per_y) return 1;
        const int n = std::max(c->ph.nx, c->ph.ny);
        k_apply_edges<<<(n + 255) / 256, 256, 0, c->stream>>>(pa);
        return 2;
    }
    dim3 blk(32, 8), grd((c->ph.nx + 1 + 31) / 32, (c->ph.ny + 1 + 7) / 8);
    k_apply_pressure<<<grd, blk, 0, c->stream>>>(pa);
    return 1;
}

static Outer outer_args(cf_ctx* c, const Stencil& st, int gated) {
    Outer oa{};
    oa.nx = c->ph.nx;
    oa.ny = c->ph.ny;
    oa.per_x = c->ph.per_x;
    oa.per_y = c->ph.per_y;
    oa.G = c->G;
    oa.U = c->n_units;
    oa.pitch = c->vpitch;
    oa.pitch32 = c->p32;
    const double scale = -st.ms;
    for (int b = 0; b < 16; ++b) {
        int d = 4;  // a SOLID side drops the leg and lowers the diagonal (build_stencil)
        if ((b & 1) && c->ph.bc[0] == CF_BC_SOLID) --d;
        if ((b & 2) && c->ph.bc[2] == CF_BC_SOLID) --d;
        if ((b & 4) && c->ph.bc[1] == CF_BC_SOLID) --d;
        if ((b & 8) && c->ph.bc[3] == CF_BC_SOLID) --d;
        oa.dfac[b] = (float)d;
        oa.minv32[b] = st.minv32[b];
    }
    const float hi = (float)scale;
    oa.scale = make_float2(hi, (float)(scale - (double)hi));
    oa.xbuf[0] = reinterpret_cast<float2*>(c->x.a);
    oa.xbuf[1] = reinterpret_cast<float2*>(c->xb.a);
    oa.b = reinterpret_cast<const float2*>(c->b.a);
    oa.pa = c->pa32.a;
    oa.pb = c->pb32.a;
    oa.r32 = c->r32.a;
    oa.part0 = c->partials;
    oa.part1 = c->partials + c->n_units;
    oa.S = c->S;
    oa.gated = gated;
    return oa;
}

// warm start: the initial residual from the previous solution (after the
// divergence kernel), FP64 or double-float; returns kernels launched
static int launch_warm_init(cf_ctx* c, const Stencil& st, bool mixed) {
    if (mixed) {
        Outer oa = outer_args(c, st, 0);
        k_outer_resid<false><<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(oa);
    } else {
        Cg64 a = cg64_args(c, st);
        k_warm_resid64<<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(a);
    }
    return 1;
}

// the outer refinement; gated = 1 inside the MG-PCG graph
static void launch_outer(cf_ctx* c, const Stencil& st, int gated) {
    Outer oa = outer_args(c, st, gated);
    k_outer_resid<false><<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(oa);
}

// one mixed MG-PCG inner iteration before its V-cycle: K1, then the x update
// and the reliable update (fused when every iteration ends with one,
// c->x_only; else K2 and the gated update); returns kernels launched
static int launch_mixed_mg_step(cf_ctx* c, const Stencil& st) {
    cg32_launch_pair_mg(c, st);
    if (c->x_only) {
        Outer oa = outer_args(c, st, 1);
        k_outer_resid<true><<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(oa);
        return 2;
    }
    launch_outer(c, st, 1);
    return 3;
}

static const int kBatch = CF_CG_BATCH;  // CG iterations per graph launch
static const int kBatchMG = 4;          // MG-PCG iterations per graph launch

// kBatch Jacobi-PCG iterations (the body of the batch graph)
static void batch_cg(cf_ctx* c, const Stencil& st, bool mixed) {
    if (mixed) {
        for (int i = 0; i < kBatch; ++i) cg32_launch_iteration(c, st);
    } else {
        const int nb = red_blocks(c);
        Cg64 a = cg64_args(c, st);
        for (int i = 0; i < kBatch; ++i) {
            k_cg_dir_matvec64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a);
            k_cg_update64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a);
        }
    }
}

// kBatchMG MG-PCG iterations: K1 (z-mode), K2, V-cycle, r.z (mixed: the
// gated reliable update too); returns the kernels of one iteration
static int batch_mg(cf_ctx* c, const Stencil& st) {
    const bool mixed = c->precision == CF_PREC_MIXED;
    const int nb = red_blocks(c);
    const double scale = -st.ms;
    Cg64 a = cg64_args(c, st);
    a.mg = 1;
    a.z = mixed ? nullptr : mg_z64(c);
    int per = 0;
    for (int i = 0; i < kBatchMG; ++i) {
        if (mixed) {
            per = launch_mixed_mg_step(c, st);
            per += cg32_mg_precondition(c, scale);
        } else {
            k_cg_dir_matvec64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a);
            k_cg_update64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a);
            per = 3 + mg_vcycle(c, scale);
            k_mg_rz64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a, 0);
        }
    }
    return per;
}

// V-cycle and r.z after the residual was (re)formed; returns kernels launched
static int batch_mg_pre(cf_ctx* c, const Stencil& st) {
    const bool mixed = c->precision == CF_PREC_MIXED;
    const double scale = -st.ms;
    if (mixed) return cg32_mg_precondition(c, scale);
    Cg64 a = cg64_args(c, st);
    a.mg = 1;
    a.z = mg_z64(c);
    const int pre = 1 + mg_vcycle(c, scale);
    k_mg_rz64<<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(a, 1);
    return pre;
}

// One batch of the host-polled projection: the captured graph, or, with
// graphs off (cf_set_graphs), the same kernels issued one by one.
template <typename F>
static int launch_batch(cf_ctx* c, cudaGraphExec_t ge, F&& issue) {
    if (c->direct) {
        issue();
        return cuda_check(c, cudaGetLastError(), "kernel launch");
    }
    return cuda_check(c, cudaGraphLaunch(ge, c->stream), "graph launch");
}

// Build (or reuse) the graph of kBatch iterations for the current stencil.
static int ensure_graph(cf_ctx* c, const Stencil& st, bool mixed) {
    cudaGraphExec_t& ge = mixed ? c->g32 : c->g64;
    Stencil& key = mixed ? c->g32_st : c->g64_st;
    if (ge && std::memcmp(&key, &st, sizeof(Stencil)) == 0) return CF_OK;
    if (ge) {
        cudaGraphExecDestroy(ge);
        ge = nullptr;
    }
    cudaGraph_t g;
    int rc = cuda_check(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture begin");
    if (rc) return rc;
    batch_cg(c, st, mixed);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if ((rc = cuda_check(c, e, "capture end"))) return rc;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if ((rc = cuda_check(c, e, "graph instantiate"))) return rc;
    key = st;
    return CF_OK;
}

// Capture the launches of fn into a graph.
template <typename F>
static int capture(cf_ctx* c, cudaGraphExec_t* ge, F&& fn) {
    if (*ge) {
        cudaGraphExecDestroy(*ge);
        *ge = nullptr;
    }
    cudaGraph_t g;
    int rc = cuda_check(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture begin");
    if (rc) return rc;
    fn();
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if ((rc = cuda_check(c, e, "capture end"))) return rc;
    e = cudaGraphInstantiate(ge, g, 0);
    cudaGraphDestroy(g);
    return cuda_check(c, e, "graph instantiate");
}

// MG-PCG graphs for the current stencil: gmg = kBatchMG iterations of
// K1 (z-mode), K2, V-cycle, r.z; gmg_pre = V-cycle and r.z after the
// residual was formed (cold start, and after each reliable update).
static int ensure_graph_mg(cf_ctx* c, const Stencil& st) {
    if (c->gmg && c->gmg_pre && c->gmg_xonly == c->x_only && std::memcmp(&c->gmg_st, &st, sizeof(Stencil)) == 0)
        return CF_OK;
    int per = 0, pre = 0;
    int rc = capture(c, &c->gmg, [&] { per = batch_mg(c, st); });
    if (!rc) rc = capture(c, &c->gmg_pre, [&] { pre = batch_mg_pre(c, st); });
    if (rc) return rc;
    c->gmg_st = st;
    c->gmg_xonly = c->x_only;
    c->gmg_per_iter = per;
    c->gmg_pre_launches = pre;
    return CF_OK;
}

// accumulate the device time of a CG batch in which every iteration ran
static void batch_profile(cf_ctx* c, int iters, int batch = kBatch) {
    if (!c->prof || iters != batch) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]) == cudaSuccess) {
        c->pd.solve_ms += ms;
        c->pd.solve_iters += iters;
        c->pd.solve_batches += 1;
    }
}

static int read_state(cf_ctx* c) {
    cudaMemcpyAsync(c->hS, c->S, sizeof(SolverState), cudaMemcpyDeviceToHost, c->stream);
    return cuda_check(c, cudaStreamSynchronize(c->stream), "solver state read");
}

// --------------------------------------------------------------------------
// Device-resident projection: one CUDA graph per stencil, state setup and
// current buffer, so that a projection costs one launch and one host
// synchronisation:
//   head : divergence + CG init, [MG: V-cycle and r.z]
//   WHILE (status == RUNNING): kResidentBatch iterations, then k_loop_cond,
//          which ends the loop, and stops it after trip_limit trips
//   tail : [mixed: double-float x to FP64], gradient subtraction, ||div u||,
//          copies of the solver state and the norms to pinned host memory
static const int kResidentBatch = 16;    // Jacobi-PCG iterations per trip
static const int kResidentBatchMG = 1;   // MG-PCG iterations per trip

// after each resident projection: count the solves that did not converge
// (a solve still RUNNING stopped at the trip limit) and keep the worst status
// (tally[2]: loop trips + 1 summed over the projections, for launch counts)
__global__ void k_step_tally(const SolverState* S, int* tally) {
    int st = S->status == ST_RUNNING ? ST_MAXIT : S->status;
    if (st != ST_CONVERGED) {
        tally[0] += 1;
        if (st > tally[1]) tally[1] = st;
    }
    tally[2] += S->trips + 1;
}

__global__ void k_loop_cond(SolverState* S, cudaGraphConditionalHandle h) {
    int run = *(volatile int*)&S->status == ST_RUNNING;
    if (run) {
        S->trips += 1;
        if (S->trips > S->trip_limit) {
            S->status = ST_MAXIT;
            run = 0;
        }
    }
    cudaGraphSetConditional(h, run ? 1u : 0u);
}

// kernels of one iteration (per trip: batch of them); returns launches
static int launch_iterations(cf_ctx* c, const Stencil& st, bool mixed, bool mg, int n) {
    const int nb = red_blocks(c);
    const double scale = -st.ms;
    int k = 0;
    Cg64 a = cg64_args(c, st);
    if (mg && !mixed) {
        a.mg = 1;
        a.z = mg_z64(c);
    }
    for (int i = 0; i < n; ++i) {
        if (mixed) {
            // MG: a reliable update follows almost every iteration, so the
            // gated outer kernels sit in every iteration; Jacobi: once a trip
            if (mg) {
                k += launch_mixed_mg_step(c, st);
                k += cg32_mg_precondition(c, scale);
            } else {
                cg32_launch_iteration(c, st);
                k += 2;
                if (i == n - 1) {
                    launch_outer(c, st, 1);
                    k += 1;
                }
            }
        } else {
            k_cg_dir_matvec64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a);
            k_cg_update64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a);
            k += 2;
            if (mg) {
                k += 1 + mg_vcycle(c, scale);
                k_mg_rz64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a, 0);
            }
        }
    }
    return k;
}

static int capture_graph(cf_ctx* c, cudaGraph_t* g, const std::function<void()>& fn) {
    int rc = cuda_check(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture begin");
    if (rc) return rc;
    fn();
    return cuda_check(c, cudaStreamEndCapture(c->stream, g), "capture end");
}

// slot: the cache entry (0, 1: the two state buffers; 2, 3: the adjoint's
// two pairs of adjoint face arrays); adjoint = 1 builds the transpose of the
// projection on gu, gv (no wall mask after the gradient subtraction, no
// warm start, no event for cf_step_host).
// pre (optional): launches captured into a first child graph the rest
// depends on (a whole step: ghost fill, advection, inputs, the parameters
// copy), returning its kernel count; out: where the executable graph goes
// (null: the projection cache slot).
static int build_resident(cf_ctx* c, const Stencil& st, double dt, bool mixed, bool mg, int slot, Grid<double> gu,
                          Grid<double> gv, int adjoint, const std::function<int()>* pre = nullptr,
                          cudaGraphExec_t* out = nullptr) {
    if (!out) out = &c->rgx[slot];
    if (!c->ev_press) {
        int rc0 = cuda_check(c, cudaEventCreateWithFlags(&c->ev_press, cudaEventDisableTiming), "event create");
        if (rc0) return rc0;
    }
    const int nb = red_blocks(c);
    const double scale = -st.ms;
    const int warm = adjoint ? c->adj_warm : c->warm;
    cudaGraph_t g = nullptr, head = nullptr, tail = nullptr, preg = nullptr;
    int nhead = 0, ntrip = 0, ntail = 0, npre = 0;
    int rc = cuda_check(c, cudaGraphCreate(&g, 0), "graph create");
    if (!rc && pre) rc = capture_graph(c, &preg, [&] { npre = (*pre)(); });
    if (!rc)
        rc = capture_graph(c, &head, [&] {
            DivArgs da = div_args(c, st);
            da.u = gu;
            da.v = gv;
            da.warm = warm;
            if (fused_norms(c, mixed, adjoint)) save_bounds(c, &da);
            if (mixed)
                k_div_init_mixed<<<nb, CF_RED_THREADS, 0, c->stream>>>(da);
            else
                k_div_init64<<<nb, CF_RED_THREADS, 0, c->stream>>>(da);
            nhead = 1;
            if (warm) nhead += launch_warm_init(c, st, mixed);
            if (mg) {
                if (mixed) {
                    nhead += cg32_mg_precondition(c, scale);
                } else {
                    Cg64 a = cg64_args(c, st);
                    a.mg = 1;
                    a.z = mg_z64(c);
                    nhead += 1 + mg_vcycle(c, scale);
                    k_mg_rz64<<<nb, CF_RED_THREADS, 0, c->stream>>>(a, 1);
                }
            }
        });
    cudaGraphNode_t np = nullptr, nh = nullptr, nc = nullptr, nt = nullptr;
    if (!rc && preg) rc = cuda_check(c, cudaGraphAddChildGraphNode(&np, g, nullptr, 0, preg), "graph step");
    if (!rc) rc = cuda_check(c, cudaGraphAddChildGraphNode(&nh, g, np ? &np : nullptr, np ? 1 : 0, head), "graph head");
    cudaGraphConditionalHandle h = 0;
    if (!rc) rc = cuda_check(c, cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault), "handle");
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if (!rc) rc = cuda_check(c, cudaGraphAddNode(&nc, g, &nh, nullptr, 1, &cp), "graph loop");
    if (!rc) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        rc = cuda_check(c, cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0,
                                                         cudaStreamCaptureModeThreadLocal),
                        "capture body");
        if (!rc) {
            ntrip = launch_iterations(c, st, mixed, mg, mg ? kResidentBatchMG : kResidentBatch);
            k_loop_cond<<<1, 1, 0, c->stream>>>(c->S, h);
            ntrip += 1;
            rc = cuda_check(c, cudaStreamEndCapture(c->stream, &body), "capture body end");
        }
    }
    if (!rc)
        rc = capture_graph(c, &tail, [&] {
            dim3 blk(32, 8);
            // mixed: the gradient reads the double-float solution; a warm
            // start then has it converted to the FP64 pressure it starts from
            Press pa = press_args(c, dt, gu, gv, adjoint);
            DivArgs dn = div_args(c, st);
            dn.u = gu;
            dn.v = gv;
            const bool fuse_n = fused_norms(c, mixed, adjoint);
            if (fuse_n) save_bounds(c, &dn);
            ntail += launch_apply(c, pa, fuse_n ? &dn : nullptr) - 1;
            // u, v are final here: a caller may copy them out beside the norms
            if (!adjoint) cudaEventRecordWithFlags(c->ev_press, c->stream, cudaEventRecordExternal);
            if (mixed && warm) {
                dim3 grdc((c->ph.nx + 31) / 32, (c->ph.ny + 7) / 8);
                k_df_to_f64<<<grdc, blk, 0, c->stream>>>(c->x.a, reinterpret_cast<const float2*>(c->xb.a), c->S,
                                                         c->ph.nx, c->ph.ny, c->vpitch);
                ntail += 1;
            }
            // (the adjoint's projections report no divergence norms)
            if (!adjoint && !fuse_n) {
                k_div_norms<<<nb, CF_RED_THREADS, 0, c->stream>>>(dn);
                ntail += 1;
            }
            k_step_tally<<<1, 1, 0, c->stream>>>(c->S, c->d_tally);
            ntail += 2;
            cudaMemcpyAsync(c->hS, c->S, sizeof(SolverState), cudaMemcpyDeviceToHost, c->stream);
            cudaMemcpyAsync(c->h_out, c->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        });
    if (!rc) rc = cuda_check(c, cudaGraphAddChildGraphNode(&nt, g, &nc, 1, tail), "graph tail");
    if (*out) {
        cudaGraphExecDestroy(*out);
        *out = nullptr;
    }
    if (!rc) rc = cuda_check(c, cudaGraphInstantiate(out, g, 0), "graph instantiate");
    if (preg) cudaGraphDestroy(preg);
    if (head) cudaGraphDestroy(head);
    if (tail) cudaGraphDestroy(tail);
    if (g) cudaGraphDestroy(g);
    if (rc) return rc;
    // launch counts for project_collect (a step graph's ghost fill, advection
    // and inputs count with its head)
    const int k = pre ? 4 + slot : slot;
    c->rg_head[k] = npre + nhead;
    c->rg_trip[k] = ntrip;
    c->rg_tail[k] = ntail;
    return CF_OK;
}

static bool resident_enabled() {
    static int on = -1;
    if (on < 0) {
        const char* e = getenv("CF_RESIDENT");
        on = e ? (atoi(e) != 0) : 1;
    }
    return on != 0;
}

bool resident_projection() { return resident_enabled(); }

// A warm start reads the previous solution as an FP64 pressure: convert it in
// place when the last mixed projection left it as double-float pairs (before
// the solver state is replaced: the conversion reads SolverState::xsel).
static void settle_pressure(cf_ctx* c) {
    if (!c->p_df) return;
    dim3 blk(32, 8), grd((c->ph.nx + 31) / 32, (c->ph.ny + 7) / 8);
    k_df_to_f64<<<grd, blk, 0, c->stream>>>(c->x.a, reinterpret_cast<const float2*>(c->xb.a), c->S, c->ph.nx, c->ph.ny,
                                            c->vpitch);
    c->launches += 1;
    c->p_df = 0;
}

// the projection of gu, gv (the current buffers, or with adjoint = 1 the
// adjoint's face arrays) through a resident graph; with defer, returns after
// the launch (project_collect reads the results)
static int project_resident(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res, const Stencil& st,
                            bool mixed, bool mg, bool defer, bool params_ready, Grid<double> gu, Grid<double> gv,
                            int adjoint) {
    int slot = c->cur;
    if (adjoint) {
        // the adjoint's arrays alternate between two buffers: one slot each
        slot = c->rg_u[2] == gu.o ? 2 : (c->rg_u[3] == gu.o ? 3 : (c->rg_u[2] ? 3 : 2));
        if (c->rg_u[slot] != gu.o && c->rg_u[2] && c->rg_u[3]) slot = 2;
    }
    c->x_only = (mixed && mg && o.inner_tol >= 0.5) ? 1 : 0;
    const int flags = (mixed ? 1 : 0) | (mg ? 2 : 0) | ((adjoint ? c->adj_warm : c->warm) ? 4 : 0) | (c->x_only ? 8 : 0) |
                      (adjoint ? 16 : 0) | (c->test_general_apply ? 32 : 0);
    int rc = CF_OK;
    if (!c->rgx[slot] || c->rg_flags[slot] != flags || c->rg_u[slot] != gu.o ||
        std::memcmp(&c->rg_st[slot], &st, sizeof(Stencil)) != 0 ||
        std::memcmp(&c->rg_ph[slot], &c->ph, sizeof(Phys)) != 0) {
        rc = build_resident(c, st, dt, mixed, mg, slot, gu, gv, adjoint);
        if (rc) return rc;
        c->rg_flags[slot] = flags;
        c->rg_st[slot] = st;
        c->rg_ph[slot] = c->ph;
        c->rg_u[slot] = gu.o;
    }
    // The parameters go in from their own pinned buffer: the tail copies the
    // final state back into hS, and a caller that enqueues several steps
    // without synchronising (params_ready: the same parameters, written once)
    // must not have a later step read an earlier step's final state.  The
    // adjoint's projections have a buffer of their own, so that forward and
    // adjoint projections can be enqueued in turn.
    if (flags & 4) settle_pressure(c);
    SolverState* h = adjoint ? c->hPa : c->hP;
    if (!params_ready) {
        memset(h, 0, sizeof(SolverState));
        h->tol2 = o.tol * o.tol;
        h->abs2 = o.abs_tol * o.abs_tol;
        h->use_abs = o.abs_tol > 0.0 ? 1 : 0;
        h->area = c->ph.dx * c->ph.dx;
        h->max_iter = o.max_iter;
        h->max_outer = o.max_outer;
        h->inner_tol2 = o.inner_tol * o.inner_tol;
        h->status = ST_RUNNING;
        const int batch = mg ? kResidentBatchMG : kResidentBatch;
        h->trip_limit = (o.max_iter + (mixed ? o.max_outer : 0)) / batch + 4;
        h->test_stall = c->test_stall;
    }
    cudaMemcpyAsync(c->S, h, sizeof(SolverState), cudaMemcpyHostToDevice, c->stream);
    if ((rc = cuda_check(c, cudaGraphLaunch(c->rgx[slot], c->stream), "graph launch"))) return rc;
    c->p_df = (mixed && !(flags & 4)) ? 1 : 0;
    c->rg_pending = slot;
    if (defer) return CF_OK;
    if ((rc = cuda_check(c, cudaStreamSynchronize(c->stream), "projection"))) return rc;
    project_collect(c, res);
    return CF_OK;
}

int step_resident(cf_ctx* c, double dt, int order, int fuse, const SolveOpts& o, bool params_ready) {
    const bool mixed = c->precision == CF_PREC_MIXED;
    const bool mg = o.precon_mg != 0;
    Stencil st{};
    build_stencil(c, dt, o.precon_none, &st);
    int rc = mg ? mg_setup(c) : CF_OK;
    if (rc) return rc;
    const int s = c->cur, n = 1 - s;
    c->x_only = (mixed && mg && o.inner_tol >= 0.5) ? 1 : 0;
    const int flags =
        (mixed ? 1 : 0) | (mg ? 2 : 0) | (c->warm ? 4 : 0) | (c->x_only ? 8 : 0) | (c->test_unstaged ? 16 : 0) |
        (c->test_general_apply ? 32 : 0);
    if (!c->sgx[s] || c->sg_dt[s] != dt || c->sg_order[s] != order || c->sg_fuse[s] != fuse ||
        c->sg_flags[s] != flags || std::memcmp(&c->sg_st[s], &st, sizeof(Stencil)) != 0 ||
        std::memcmp(&c->sg_ph[s], &c->ph, sizeof(Phys)) != 0) {
        // the step's own launches, on buffer s, then the parameters copy
        const std::function<int()> pre = [&]() {
            const long long l0 = c->launches;
            cudaError_t e = launch_fill_ghosts(c);
            if (e == cudaSuccess) e = launch_advect(c, dt, order, fuse, 0, 3, true, false);
            if (e == cudaSuccess && !fuse) {
                c->cur = n;
                e = launch_add_inputs(c, dt);
                c->cur = s;
            }
            cudaMemcpyAsync(c->S, c->hP, sizeof(SolverState), cudaMemcpyHostToDevice, c->stream);
            const int k = (int)(c->launches - l0);
            c->launches = l0;  // counted per launch of the graph instead
            return k;
        };
        rc = build_resident(c, st, dt, mixed, mg, n, c->u[n], c->v[n], 0, &pre, &c->sgx[s]);
        if (rc) return rc;
        c->sg_dt[s] = dt;
        c->sg_order[s] = order;
        c->sg_fuse[s] = fuse;
        c->sg_flags[s] = flags;
        c->sg_st[s] = st;
        c->sg_ph[s] = c->ph;
    }
    // a warm start reads the previous solution as FP64 (before the graph's
    // parameters copy replaces the solver state the conversion reads)
    if (flags & 4) settle_pressure(c);
    SolverState* h = c->hP;
    if (!params_ready) {
        memset(h, 0, sizeof(SolverState));
        h->tol2 = o.tol * o.tol;
        h->abs2 = o.abs_tol * o.abs_tol;
        h->use_abs = o.abs_tol > 0.0 ? 1 : 0;
        h->area = c->ph.dx * c->ph.dx;
        h->max_iter = o.max_iter;
        h->max_outer = o.max_outer;
        h->inner_tol2 = o.inner_tol * o.inner_tol;
        h->status = ST_RUNNING;
        const int batch = mg ? kResidentBatchMG : kResidentBatch;
        h->trip_limit = (o.max_iter + (mixed ? o.max_outer : 0)) / batch + 4;
        h->test_stall = c->test_stall;
    }
    if ((rc = cuda_check(c, cudaGraphLaunch(c->sgx[s], c->stream), "step graph launch"))) return rc;
    c->cur = n;
    c->p_df = (mixed && !(flags & 4)) ? 1 : 0;
    c->rg_pending = 4 + n;
    return CF_OK;
}

void project_collect(cf_ctx* c, SolveResult* res, int nproj, long long trips) {
    const int cur = c->rg_pending;
    const SolverState* hs = c->hS;
    if (nproj <= 0)
        c->launches += c->rg_head[cur] + (long long)c->rg_trip[cur] * (hs->trips + 1) + c->rg_tail[cur];
    else  // nproj projections with trips loop trips (+1 each) in all
        c->launches += (long long)nproj * (c->rg_head[cur] + c->rg_tail[cur]) + (long long)c->rg_trip[cur] * trips;
    res->iterations = hs->iter;
    res->outer = hs->outer_iter;
    res->status = hs->status == ST_RUNNING ? ST_MAXIT : hs->status;
    res->bb = hs->bb;
    res->rr = hs->rr;
    res->div_l2 = sqrt(c->h_out[0]) * c->ph.dx;
    res->div_linf = c->h_out[1];
}

int project_async(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res, bool* deferred, bool params_ready) {
    const bool mixed = c->precision == CF_PREC_MIXED;
    const bool mg = o.precon_mg != 0;
    *deferred = false;
    if (c->prof || c->direct || !resident_enabled()) return project(c, dt, o, res);
    Stencil st{};
    build_stencil(c, dt, o.precon_none, &st);
    int rc = mg ? mg_setup(c) : CF_OK;
    if (rc) return rc;
    *deferred = true;
    return project_resident(c, dt, o, res, st, mixed, mg, true, params_ready, c->u[c->cur], c->v[c->cur], 0);
}

int project_adjoint_async(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res, bool* deferred,
                          bool params_ready, Grid<double> gu, Grid<double> gv) {
    *deferred = false;
    if (c->prof || c->direct || !resident_enabled()) return project_grids(c, dt, o, res, gu, gv, 1);
    Stencil st{};
    build_stencil(c, dt, o.precon_none, &st);
    const bool mg = o.precon_mg != 0;
    int rc = mg ? mg_setup(c) : CF_OK;
    if (rc) return rc;
    *deferred = true;
    return project_resident(c, dt, o, res, st, c->precision == CF_PREC_MIXED, mg, true, params_ready, gu, gv, 1);
}

cudaError_t pressure_to_f64(cf_ctx* c, double* out) {
    dim3 blk(32, 8), grd((c->ph.nx + 31) / 32, (c->ph.ny + 7) / 8);
    k_df_to_f64_out<<<grd, blk, 0, c->stream>>>(reinterpret_cast<const float2*>(c->x.a),
                                                reinterpret_cast<const float2*>(c->xb.a), c->S, c->ph.nx, c->ph.ny,
                                                c->vpitch, out);
    c->launches += 1;
    return cudaGetLastError();
}

// the norms the last k_div_norms or k_apply_pairs_norms left in d_out
static int read_norms(cf_ctx* c, double* l2, double* linf) {
    cudaMemcpyAsync(c->h_out, c->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    int rc = cuda_check(c, cudaStreamSynchronize(c->stream), "div norms");
    if (rc) return rc;
    *l2 = sqrt(c->h_out[0]) * c->ph.dx;
    *linf = c->h_out[1];
    return CF_OK;
}

int div_norms(cf_ctx* c, double* l2, double* linf) {
    Stencil st{};
    DivArgs a = div_args(c, st);
    k_div_norms<<<red_blocks(c), CF_RED_THREADS, 0, c->stream>>>(a);
    c->launches += 1;
    return read_norms(c, l2, linf);
}

int project(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res) {
    return project_grids(c, dt, o, res, c->u[c->cur], c->v[c->cur], 0);
}

// The projection on the face arrays u, v.  adjoint = 1 applies the transpose
// of the projection: the caller has applied the wall masks, and no mask is
// applied after the gradient subtraction (see cf_adjoint.cu).
int project_grids(cf_ctx* c, double dt, const SolveOpts& o, SolveResult* res, Grid<double> gu, Grid<double> gv,
                  int adjoint) {
    Stencil st{};
    build_stencil(c, dt, o.precon_none, &st);
    const bool mixed = c->precision == CF_PREC_MIXED;
    const bool mg = o.precon_mg != 0;
    int rc = mg ? mg_setup(c) : CF_OK;
    if (rc) return rc;
    c->x_only = (mixed && mg && o.inner_tol >= 0.5) ? 1 : 0;
    // the resident graph serves plain projections; the adjoint's projection
    // (other arrays) and profiled runs (events between batches) take the
    // host-polled batches below
    if (!c->prof && !c->direct && resident_enabled())
        return project_resident(c, dt, o, res, st, mixed, mg, false, false, gu, gv, adjoint);
    rc = mg ? ensure_graph_mg(c, st) : ensure_graph(c, st, mixed);
    if (rc) return rc;

    if (adjoint ? c->adj_warm : c->warm) settle_pressure(c);
    // solver parameters
    SolverState* h = c->hS;
    memset(h, 0, sizeof(SolverState));
    h->tol2 = o.tol * o.tol;
    h->abs2 = o.abs_tol * o.abs_tol;
    h->use_abs = o.abs_tol > 0.0 ? 1 : 0;
    h->area = c->ph.dx * c->ph.dx;
    h->max_iter = o.max_iter;
    h->max_outer = o.max_outer;
    h->inner_tol2 = o.inner_tol * o.inner_tol;
    h->status = ST_RUNNING;
    h->test_stall = c->test_stall;
    cudaMemcpyAsync(c->S, h, sizeof(SolverState), cudaMemcpyHostToDevice, c->stream);
    int nb = red_blocks(c);
    DivArgs da = div_args(c, st);
    da.u = gu;
    da.v = gv;
    const bool warm = adjoint ? c->adj_warm != 0 : c->warm != 0;
    da.warm = warm;
    if (c->prof) cudaEventRecord(c->ev[4], c->stream);
    if (!mixed) {
        k_div_init64<<<nb, CF_RED_THREADS, 0, c->stream>>>(da);
        c->launches += 1;
        if (warm) c->launches += launch_warm_init(c, st, false);
        const int batch = mg ? kBatchMG : kBatch;
        cudaGraphExec_t ge = mg ? c->gmg : c->g64;
        const int per_batch = mg ? c->gmg_per_iter * kBatchMG : 2 * kBatch;
        if (mg) {
            if ((rc = launch_batch(c, c->gmg_pre, [&] { batch_mg_pre(c, st); }))) return rc;
            c->launches += c->gmg_pre_launches;
        }
        int max_launch = o.max_iter / batch + 3;
        int prev_iter = 0;
        for (int l = 0;; ++l) {
            if ((rc = read_state(c))) return rc;
            if (l > 0) batch_profile(c, c->hS->iter - prev_iter, batch);
            prev_iter = c->hS->iter;
            if (c->hS->status != ST_RUNNING) break;
            if (l >= max_launch) return fail(c, CF_ERR_NUMERIC, "solver did not stop after %d batches", l);
            if (c->prof) cudaEventRecord(c->ev[0], c->stream);
            if (mg)
                rc = launch_batch(c, ge, [&] { batch_mg(c, st); });
            else
                rc = launch_batch(c, ge, [&] { batch_cg(c, st, false); });
            if (rc) return rc;
            if (c->prof) cudaEventRecord(c->ev[1], c->stream);
            c->launches += per_batch;
        }
    } else {
        DivArgs di = da;
        if (fused_norms(c, mixed, adjoint)) save_bounds(c, &di);
        k_div_init_mixed<<<nb, CF_RED_THREADS, 0, c->stream>>>(di);
        c->launches += 1;
        if (warm) c->launches += launch_warm_init(c, st, true);
        if (mg) {
            // MG-PCG: the reliable updates run inside the graph (gated
            // kernels), so the host only polls the status between batches
            if ((rc = launch_batch(c, c->gmg_pre, [&] { batch_mg_pre(c, st); }))) return rc;
            c->launches += c->gmg_pre_launches;
            int max_launch = (o.max_iter + o.max_outer) / kBatchMG + 3;
            int prev_iter = 0;
            for (int l = 0;; ++l) {
                if ((rc = read_state(c))) return rc;
                if (l > 0) batch_profile(c, c->hS->iter - prev_iter, kBatchMG);
                prev_iter = c->hS->iter;
                if (c->hS->status != ST_RUNNING) break;
                if (l >= max_launch) return fail(c, CF_ERR_NUMERIC, "mixed MG solver did not stop");
                if (c->prof) cudaEventRecord(c->ev[0], c->stream);
                if ((rc = launch_batch(c, c->gmg, [&] { batch_mg(c, st); }))) return rc;
                if (c->prof) cudaEventRecord(c->ev[1], c->stream);
                c->launches += c->gmg_per_iter * kBatchMG;
            }
        } else {
            if ((rc = read_state(c))) return rc;
            int max_launch = o.max_iter / kBatch + 3 * (o.max_outer + 1);
            int launches = 0;
            while (c->hS->status == ST_RUNNING) {
                while (c->hS->status == ST_RUNNING && c->hS->inner_status == ST_RUNNING) {
                    if (++launches > max_launch) return fail(c, CF_ERR_NUMERIC, "mixed solver did not stop");
                    int prev_iter = c->hS->iter;
                    if (c->prof) cudaEventRecord(c->ev[0], c->stream);
                    if ((rc = launch_batch(c, c->g32, [&] { batch_cg(c, st, true); }))) return rc;
                    if (c->prof) cudaEventRecord(c->ev[1], c->stream);
                    c->launches += 2 * kBatch;
                    if ((rc = read_state(c))) return rc;
                    batch_profile(c, c->hS->iter - prev_iter);
                }
                if (c->hS->status != ST_RUNNING) break;
                launch_outer(c, st, 0);
                c->launches += 1;
                if ((rc = read_state(c))) return rc;
                if (++launches > max_launch) return fail(c, CF_ERR_NUMERIC, "mixed solver did not stop");
            }
        }
    }
    const SolverState* hs = c->hS;
    res->iterations = hs->iter;
    res->outer = hs->outer_iter;
    res->status = hs->status == ST_RUNNING ? ST_MAXIT : hs->status;
    res->bb = hs->bb;
    res->rr = hs->rr;

    // gradient subtraction (mixed: from the double-float solution; the FP64
    // pressure is made afterwards for a warm start, or when it is downloaded)
    Press pa = press_args(c, dt, gu, gv, adjoint);
    const bool fuse_n = fused_norms(c, mixed, adjoint);
    DivArgs dn = da;
    if (fuse_n) save_bounds(c, &dn);
    c->launches += launch_apply(c, pa, fuse_n ? &dn : nullptr);
    c->p_df = mixed ? 1 : 0;
    if (mixed && warm) settle_pressure(c);
    if ((rc = cuda_check(c, cudaGetLastError(), "apply pressure"))) return rc;
    if (c->prof) cudaEventRecord(c->ev[5], c->stream);
    if (adjoint) return cuda_check(c, cudaStreamSynchronize(c->stream), "adjoint projection");
    rc = fuse_n ? read_norms(c, &res->div_l2, &res->div_linf) : div_norms(c, &res->div_l2, &res->div_linf);
    if (!rc && c->prof) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]) == cudaSuccess) {
            c->pd.project_ms += ms;
            c->pd.projects += 1;
        }
    }
    return rc;
}

}  // namespace cf
