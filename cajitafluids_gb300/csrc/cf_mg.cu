// Geometric multigrid V-cycle preconditioner (the stand-in for the HYPRE
// PFMG/SMG preconditioners the reference selects by name,
// src/VelocityCorrector.hpp:324-338; PFMG is the CLI default,
// examples/advection.cpp:186-189).
//
// Cell-centred levels halve both axes while both are even and at least 16;
// level l uses the fine 5-point stencil with scale / 4^l and the same wall
// rules (16-entry diagonal tables by wall-adjacency bits).  Per level:
//   x = 0; MG_NU x (red, black) Gauss-Seidel half sweeps; r = b - A x;
//   b_coarse = R r (transpose of the bilinear prolongation, / 4);
//   recurse; x += P x_coarse (cell-centred bilinear: 3/4, 1/4 per axis,
//   SOLID walls reflect, FREE walls read zero, periodic axes wrap);
//   MG_NU x (black, red) half sweeps.
// The coarsest level runs MG_NC (red, black) and MG_NC (black, red) sweeps,
// in one CTA from shared memory when it fits.  The cycle is symmetric, as
// CG needs.  FP64 arithmetic follows the oracle operation by operation
// (explicit fma, fixed order), so the FP64 MG-PCG stays bit-reproducible.
#include <cuda_runtime.h>
#include <math.h>

#include <cstdlib>
#include <vector>

#include "cf_ctx.cuh"

namespace cf {

constexpr int MG_NU = 2;
constexpr int MG_NC = 8;

template <typename T>
struct MgLev {
    T *x, *b, *r;
    int nx, ny, pitch;
    T scale, ms;
    T diag[16], invd[16];
};

struct MgBc {
    int per_x, per_y;
    int bc[4];
};

__device__ __forceinline__ int mg_bits(const MgBc& p, int nx, int ny, int gi, int gj) {
    int b = 0;
    if (!p.per_x) b |= (gi == 0 ? 1 : 0) | (gi == nx - 1 ? 2 : 0);
    if (!p.per_y) b |= (gj == 0 ? 4 : 0) | (gj == ny - 1 ? 8 : 0);
    return b;
}

template <typename T>
__device__ __forceinline__ T mg_at(const MgBc& p, const T* a, int pitch, int nx, int ny, int gi, int gj) {
    if (gi < 0 || gi >= nx) {
        if (!p.per_x) return T(0);
        gi = gi < 0 ? gi + nx : gi - nx;
    }
    if (gj < 0 || gj >= ny) {
        if (!p.per_y) return T(0);
        gj = gj < 0 ? gj + ny : gj - ny;
    }
    return a[(size_t)gj * pitch + gi];
}

__device__ __forceinline__ double mg_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float mg_fma(float a, float b, float c) { return fmaf(a, b, c); }

// Kernels read the solver status once per block (a per-thread read of the one
// status word serialises every warp of the grid on one L2 slice).
__device__ __forceinline__ bool block_live(const SolverState* S, int inner) {
    __shared__ int live;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        int ok = *(volatile const int*)&S->status == ST_RUNNING;
        if (inner) ok = ok && *(volatile const int*)&S->inner_status == ST_RUNNING;
        live = ok;
    }
    __syncthreads();
    return live != 0;
}

// Blocks are 32 x 8 threads; each thread covers MG_ROWS rows.
constexpr int MG_BX = 32, MG_BY = 8, MG_ROWS = 4;

// Red (color 0) or black (color 1) Gauss-Seidel half sweep; thread k of row
// gj owns the cell pair (2k, 2k+1) and updates its cell of that colour.
// first = 1 is the level's first half sweep from x = 0: the neighbour sum is
// zero and the cell of the other colour is written as 0 (no separate clear).
template <typename T>
__global__ void __launch_bounds__(MG_BX* MG_BY) k_mg_smooth(MgLev<T> L, MgBc p, int color, int first,
                                                             SolverState* S, int inner) {
    if (!block_live(S, inner)) return;
    const int pair = blockIdx.x * MG_BX + threadIdx.x;
#pragma unroll
    for (int rr = 0; rr < MG_ROWS; ++rr) {
        const int gj = (blockIdx.y * MG_ROWS + rr) * MG_BY + threadIdx.y;
        const int par = (gj + color) & 1;
        const int gi = 2 * pair + par;
        if (gj >= L.ny) break;
        const size_t row = (size_t)gj * L.pitch;
        if (gi < L.nx) {
            T s;
            if (first) {
                s = T(0);
            } else {
                s = mg_at(p, L.x, L.pitch, L.nx, L.ny, gi - 1, gj) + mg_at(p, L.x, L.pitch, L.nx, L.ny, gi + 1, gj);
                s = s + mg_at(p, L.x, L.pitch, L.nx, L.ny, gi, gj - 1);
                s = s + mg_at(p, L.x, L.pitch, L.nx, L.ny, gi, gj + 1);
            }
            T t = mg_fma(L.scale, s, L.b[row + gi]);
            L.x[row + gi] = t * L.invd[mg_bits(p, L.nx, L.ny, gi, gj)];
        }
        const int go = 2 * pair + (1 - par);
        if (first && go < L.nx) L.x[row + go] = T(0);
    }
}

template <typename T>
__global__ void __launch_bounds__(MG_BX* MG_BY) k_mg_residual(MgLev<T> L, MgBc p, SolverState* S, int inner) {
    if (!block_live(S, inner)) return;
    const int gi = blockIdx.x * MG_BX + threadIdx.x;
    if (gi >= L.nx) return;
#pragma unroll
    for (int rr = 0; rr < MG_ROWS; ++rr) {
        const int gj = (blockIdx.y * MG_ROWS + rr) * MG_BY + threadIdx.y;
        if (gj >= L.ny) break;
        const size_t k = (size_t)gj * L.pitch + gi;
        T ax = L.diag[mg_bits(p, L.nx, L.ny, gi, gj)] * L.x[k];
        ax = mg_fma(L.ms, mg_at(p, L.x, L.pitch, L.nx, L.ny, gi - 1, gj), ax);
        ax = mg_fma(L.ms, mg_at(p, L.x, L.pitch, L.nx, L.ny, gi + 1, gj), ax);
        ax = mg_fma(L.ms, mg_at(p, L.x, L.pitch, L.nx, L.ny, gi, gj - 1), ax);
        ax = mg_fma(L.ms, mg_at(p, L.x, L.pitch, L.nx, L.ny, gi, gj + 1), ax);
        L.r[k] = L.b[k] - ax;
    }
}

// Prolongation weight, in quarters, of coarse index I for fine index f along
// one axis: 3 from the parent (4 when the other neighbour lies beyond a SOLID
// wall, which reflects) and 1 from the neighbour on f's side (wrapped along a
// periodic axis, absent beyond a wall).  Quarters are exact in FP32 and FP64.
__device__ __forceinline__ int mg_pwq(int f, int I, int nc, int per, int bclo, int bchi) {
    int parent = f >> 1, nb = parent + ((f & 1) ? 1 : -1);
    bool nb_in = nb >= 0 && nb < nc;
    if (!nb_in && per) {
        nb = nb < 0 ? nb + nc : nb - nc;
        nb_in = true;
    }
    int wp = (!nb_in && (nb < 0 ? bclo : bchi) == 0) ? 4 : 3;
    return (parent == I ? wp : 0) + ((nb_in && nb == I) ? 1 : 0);
}

// b_coarse = R r = P^T r / 4 over the 4 x 4 fine cells each coarse cell touches
template <typename T>
__global__ void __launch_bounds__(MG_BX* MG_BY) k_mg_restrict(MgLev<T> F, MgLev<T> C, MgBc p, SolverState* S,
                                                               int inner) {
    if (!block_live(S, inner)) return;
    const int I = blockIdx.x * MG_BX + threadIdx.x;
    if (I >= C.nx) return;
    // the x weights do not depend on the row
    T wxs[4];
    int fxs[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int fx = 2 * I - 1 + q;
        if (fx < 0 || fx >= F.nx) {
            if (!p.per_x) {
                fxs[q] = -1;
                wxs[q] = T(0);
                continue;
            }
            fx = fx < 0 ? fx + F.nx : fx - F.nx;
        }
        fxs[q] = fx;
        wxs[q] = (T)mg_pwq(fx, I, C.nx, p.per_x, p.bc[0], p.bc[2]) * T(0.25);
    }
#pragma unroll
    for (int rr = 0; rr < MG_ROWS; ++rr) {
        const int J = (blockIdx.y * MG_ROWS + rr) * MG_BY + threadIdx.y;
        if (J >= C.ny) break;
        T acc = T(0);
        for (int fy0 = 2 * J - 1; fy0 <= 2 * J + 2; ++fy0) {
            int fy = fy0;
            if (fy < 0 || fy >= F.ny) {
                if (!p.per_y) continue;
                fy = fy < 0 ? fy + F.ny : fy - F.ny;
            }
            const T wy = (T)mg_pwq(fy, J, C.ny, p.per_y, p.bc[1], p.bc[3]) * T(0.25);
            const T* fr = F.r + (size_t)fy * F.pitch;
            T rs = T(0);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (fxs[q] >= 0) rs = mg_fma(wxs[q], fr[fxs[q]], rs);
            acc = mg_fma(wy, rs, acc);
        }
        C.b[(size_t)J * C.pitch + I] = T(0.25) * acc;
    }
}

// coarse neighbour and weights along one axis for fine index f: parent I with
// 3/4 (1 when the neighbour lies beyond a SOLID wall), neighbour N with 1/4
// (N = -1 beyond a wall)
template <typename T>
__device__ __forceinline__ void mg_axis(int f, int nc, int per, int bclo, int bchi, int& I, int& N, T& wI, T& wN) {
    int parent = f >> 1, nb = parent + ((f & 1) ? 1 : -1);
    I = parent;
    wI = T(0.75);
    wN = T(0.25);
    if (nb < 0 || nb >= nc) {
        if (per) {
            nb = nb < 0 ? nb + nc : nb - nc;
        } else {
            if ((nb < 0 ? bclo : bchi) == 0) wI = T(1);
            nb = -1;
            wN = T(0);
        }
    }
    N = nb;
}

template <typename T>
__global__ void __launch_bounds__(MG_BX* MG_BY) k_mg_prolong(MgLev<T> C, MgLev<T> F, MgBc p, SolverState* S,
                                                              int inner) {
    if (!block_live(S, inner)) return;
    const int fx = blockIdx.x * MG_BX + threadIdx.x;
    if (fx >= F.nx) return;
    int I, NI;
    T wxI, wxN;
    mg_axis<T>(fx, C.nx, p.per_x, p.bc[0], p.bc[2], I, NI, wxI, wxN);
#pragma unroll
    for (int rr = 0; rr < MG_ROWS; ++rr) {
        const int fy = (blockIdx.y * MG_ROWS + rr) * MG_BY + threadIdx.y;
        if (fy >= F.ny) break;
        int J, NJ;
        T wyJ, wyN;
        mg_axis<T>(fy, C.ny, p.per_y, p.bc[1], p.bc[3], J, NJ, wyJ, wyN);
        T row0 = wxI * C.x[(size_t)J * C.pitch + I];
        if (NI >= 0) row0 = mg_fma(wxN, C.x[(size_t)J * C.pitch + NI], row0);
        T v = wyJ * row0;
        if (NJ >= 0) {
            T row1 = wxI * C.x[(size_t)NJ * C.pitch + I];
            if (NI >= 0) row1 = mg_fma(wxN, C.x[(size_t)NJ * C.pitch + NI], row1);
            v = mg_fma(wyN, row1, v);
        }
        const size_t k = (size_t)fy * F.pitch + fx;
        F.x[k] = F.x[k] + v;
    }
}

// ---------------------------------------------------------------------------
// Fused level kernels (temporal blocking in shared memory).  A CTA owns a
// tile of TW x TH fine cells (both even) and recomputes a shrinking halo, so that the
// MG_NU = 2 sweep pairs of a level need one pass over memory:
//   k_mg_pre : x = 4 half sweeps from x = 0 (red, black, red, black),
//              r = b - A x (in shared memory), b_coarse = R r
//                                              (R b; W x, b_coarse)
//   k_mg_post: x += P x_coarse, then 4 half sweeps (black, red, black, red)
//                                              (R x, b, x_coarse; W x)
// Every cell value is computed from the same inputs with the same operations
// as by the level-by-level kernels above, so the results are identical.
// k_mg_pre leaves its x in the level's r array (free in this form) and
// k_mg_post reads it from there and writes x: a CTA of k_mg_post reads its
// halo from other tiles, which must not be written by the same launch.
constexpr int FT_THREADS = 256;
// Resident blocks per SM the level kernels are compiled for: the FP32
// 32x16 tiles fit 4 (64 registers, measured faster: 21.5 vs 24.5 us at 1024^2
// post), the register strips and FP64 tiles keep 3 (the strips spill at 64).
template <typename T, int TW>
struct FtBlocks {
    static constexpr int value = (sizeof(T) == 4 && TW == 32) ? 4 : 3;
};

// index along an axis after the periodic wrap; -1 beyond a wall
__device__ __forceinline__ int mg_dom(int g, int n, int per) {
    if (g >= 0 && g < n) return g;
    if (!per) return -1;
    return g < 0 ? g + n : g - n;
}

// one half sweep of colour c over the tile grown by h cells; arrays have halo H
template <typename T, int TW, int TH, int H>
__device__ __forceinline__ void ft_half(const MgLev<T>& L, const MgBc& p, T* xs, const T* bs, int i0, int j0, int c,
                                        int h, bool first) {
    constexpr int W = TW + 2 * H;
    const int ncol = TW + 2 * h, nrow = TH + 2 * h, hw = ncol / 2;
    const int gi0 = i0 - h;
    for (int k = threadIdx.x; k < hw * nrow; k += FT_THREADS) {
        const int rj = k / hw, pk = k % hw;
        const int gj = j0 - h + rj;
        const int gi = gi0 + ((c + gj + gi0) & 1) + 2 * pk;
        const int wi = mg_dom(gi, L.nx, p.per_x), wj = mg_dom(gj, L.ny, p.per_y);
        if (wi < 0 || wj < 0) continue;  // beyond a wall: stays 0
        const int li = gi - (i0 - H), lj = gj - (j0 - H);
        const int q = lj * W + li;
        T s;
        if (first) {
            s = T(0);
        } else {
            s = xs[q - 1] + xs[q + 1];
            s = s + xs[q - W];
            s = s + xs[q + W];
        }
        T t = mg_fma(L.scale, s, bs[q]);
        xs[q] = t * L.invd[mg_bits(p, L.nx, L.ny, wi, wj)];
    }
    __syncthreads();
}

// load x from xsrc (0 when null) and b over the tile with halo H (wrapped; 0
// beyond walls)
template <typename T, int TW, int TH, int H>
__device__ __forceinline__ void ft_load(const MgLev<T>& L, const MgBc& p, T* xs, T* bs, int i0, int j0,
                                        const T* xsrc) {
    constexpr int W = TW + 2 * H, HT = TH + 2 * H;
    for (int q = threadIdx.x; q < W * HT; q += FT_THREADS) {
        const int li = q % W, lj = q / W;
        const int wi = mg_dom(i0 - H + li, L.nx, p.per_x), wj = mg_dom(j0 - H + lj, L.ny, p.per_y);
        T xv = T(0), bv = T(0);
        if (wi >= 0 && wj >= 0) {
            const size_t k = (size_t)wj * L.pitch + wi;
            bv = L.b[k];
            if (xsrc) xv = xsrc[k];
        }
        xs[q] = xv;
        bs[q] = bv;
    }
    __syncthreads();
}

// A tile is interior when no wall is within its array (tile + halo H) and
// the tile is whole: along a non-periodic axis the array lies in [1, n-1),
// along a periodic one the halo wraps (n >= H, one period at most).  Every
// wall-adjacency bit is then 0 and every transfer weight the interior one,
// and those tiles take the index-light paths below, reading their halo
// through mg_wrap.
template <int TW, int TH, int H>
__device__ __forceinline__ bool ft_interior(int nx, int ny, int i0, int j0, const MgBc& p) {
    const bool ix = p.per_x ? (i0 + TW <= nx && nx >= H) : (i0 - H >= 1 && i0 + TW + H <= nx - 1);
    const bool iy = p.per_y ? (j0 + TH <= ny && ny >= H) : (j0 - H >= 1 && j0 + TH + H <= ny - 1);
    return ix && iy;
}

// an index within one period of [0, n): wrapped (interior tiles only)
__device__ __forceinline__ int mg_wrap(int g, int n) { return g < 0 ? g + n : (g >= n ? g - n : g); }

template <typename T, int TW, int TH, int H>
__device__ __forceinline__ void ft_load_int(const MgLev<T>& L, T* xs, T* bs, int i0, int j0, const T* xsrc) {
    constexpr int W = TW + 2 * H, HT = TH + 2 * H;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int lj = warp; lj < HT; lj += FT_THREADS / 32) {
        const size_t row = (size_t)mg_wrap(j0 - H + lj, L.ny) * L.pitch;
        for (int li = lane; li < W; li += 32) {
            const size_t k = row + mg_wrap(i0 - H + li, L.nx);
            bs[lj * W + li] = L.b[k];
            xs[lj * W + li] = xsrc ? xsrc[k] : T(0);
        }
    }
    __syncthreads();
}

// interior half sweep: warp w takes rows w, w + 8, ... (all of one parity, so
// a lane's cells of the colour sit in one column per row parity); lane l
// takes the cells 2l (+ 64) of the row's colour
template <typename T, int TW, int TH, int H>
__device__ __forceinline__ void ft_half_int(const MgLev<T>& L, T* xs, const T* bs, int i0, int j0, int c, int h,
                                            bool first) {
    constexpr int W = TW + 2 * H, RS = FT_THREADS / 32;
    const int nrow = TH + 2 * h, hw = TW / 2 + h;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const T scale = L.scale, id0 = L.invd[0];
    const int off = (c + (j0 - h + warp) + i0 - h) & 1;  // rows step by RS (even): fixed parity
    for (int pk = lane; pk < hw; pk += 32) {
        int q = (warp + H - h) * W + (H - h) + off + 2 * pk;
        for (int rj = warp; rj < nrow; rj += RS, q += RS * W) {
            T s;
            if (first) {
                s = T(0);
            } else {
                s = xs[q - 1] + xs[q + 1];
                s = s + xs[q - W];
                s = s + xs[q + W];
            }
            T t = mg_fma(scale, s, bs[q]);
            xs[q] = t * id0;
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// FP32 register strips for the interior of the large levels.
//
// A warp walks one strip of 128 columns (lane l holds columns 4l .. 4l + 3 as
// a float4) row by row and runs all four half sweeps as a wavefront: at row
// step t, sweep k works on row t - k + 1, which already has every neighbour
// value it needs (RB Gauss-Seidel cells of one colour depend only on cells of
// the other), so each cell value equals that of the tile kernels and of the
// level-by-level kernels.  Rows live in registers; W/E neighbours across
// lanes come by shuffle; the rows read from global memory arrive through a
// per-warp cp.async ring a few rows ahead.  The edge columns and rows of a
// strip are recomputed by the neighbouring strips (halo 6 | 116 | 6 for the
// pre-smoothing, which ends with the restriction; 4 | 120 | 4 for the
// post-smoothing).  Strips cover only cells whose whole read region is inside
// [1, n-1) on both axes (no wrap, no wall, uniform stencil); the frame around
// them is done by the tile path in the same launch.
constexpr int SP_COLS = 128;
constexpr int SP_PRE_OUT = 116, SP_POST_OUT = 120;
constexpr int SP_RING = 3;  // rows per warp in flight (one being read, two ahead); divides 6
constexpr unsigned SP_FULL = 0xffffffffu;

// Launch geometry shared by both paths: blocks [0, nframe) are tiles of the
// frame (all tiles outside [txa, txb) x [tya, tyb)), the rest hold 8 strips
// each (ns x nr strips, rh rows, the first writing from column x0, row y0).
struct StripMap {
    int nframe, ntx, txa, txb, tya, tyb;
    int ns, nr, rh, x0, y0;
};

// Epilogue of the finest FP32 post-smoothing (mixed MG-PCG): rho = r.z over
// the level (r = the level's b, z = its x), the CG scalars updated as by
// k_mg_rz32, and the periodic ghost copies of z written with the edge cells.
// Partials: one per frame tile (slot = block) and one per strip (slot =
// nframe + strip); the last block to finish folds them in a fixed order.
struct RzEpi {
    int on;
    double* part;
};

__device__ __forceinline__ void rz_finish(const RzEpi& E, SolverState* S, int nparts) {
    if (last_block_arrive(&S->ticket[7])) {
        const double rz = final_tree(E.part, nparts);
        if (threadIdx.x == 0) {
            S->ticket[7] = 0;
            const double den = S->refreshed ? S->rho_prev : S->rho_in;
            S->refreshed = 0;
            S->beta_in = den != 0.0 ? rz / den : 0.0;
            S->rho_in = rz;
            if (isnan(rz))
                S->status = ST_NAN;
            else if (!(rz > 0.0))
                S->inner_status = ST_BREAKDOWN;  // FP32 noise floor: refine and restart
        }
    }
}

// sum over the block's threads in a fixed order (FT_THREADS = CF_RED_THREADS)
__device__ __forceinline__ double block_total(double v) {
    __shared__ double ws[FT_THREADS / 32];
    v = warp_fold(v);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = ws[0];
#pragma unroll
    for (int k = 1; k < FT_THREADS / 32; ++k) t = t + ws[k];
    __syncthreads();
    return t;
}

// cell (i, j) lies in the region written by the strips
__device__ __forceinline__ bool in_strips(const StripMap& m, int i, int j) {
    return m.ns > 0 && i >= m.x0 && i < m.x0 + SP_POST_OUT * m.ns && j >= m.y0 && j < m.y0 + m.rh * m.nr;
}

// a frame tile's share of r.z, then the fold by the last block
__device__ __forceinline__ void post_epilogue(const RzEpi& E, SolverState* S, int nparts, double v) {
    const double t = block_total(v);
    if (threadIdx.x == 0) E.part[blockIdx.x] = t;
    rz_finish(E, S, nparts);
}

__host__ __device__ __forceinline__ void frame_tile(const StripMap& m, int f, int& tx, int& ty) {
    const int top = m.tya * m.ntx;
    if (f < top) {
        ty = f / m.ntx;
        tx = f - ty * m.ntx;
        return;
    }
    f -= top;
    const int nty_mid = m.tyb - m.tya, per = m.txa + (m.ntx - m.txb);
    if (f < nty_mid * per) {
        ty = m.tya + f / per;
        const int k = f % per;
        tx = k < m.txa ? k : m.txb + (k - m.txa);
        return;
    }
    f -= nty_mid * per;
    ty = m.tyb + f / m.ntx;
    tx = f % m.ntx;
}

// half sweep of one colour on row j (X), rows j - 1 (Xm) and j + 1 (Xp), b
// (B); the strip's first column is a multiple of 4, so the colour's cells sit
// at k = 0, 2 when sel = (j + colour) & 1 is 0 and at k = 1, 3 otherwise
__device__ __forceinline__ void sp_half(float4& X, const float4& Xm, const float4& Xp, const float4& B, int sel,
                                        float scale, float id0) {
    if (sel == 0) {
        const float w = __shfl_up_sync(SP_FULL, X.w, 1);
        float s = w + X.y;
        s = s + Xm.x;
        s = s + Xp.x;
        X.x = fmaf(scale, s, B.x) * id0;
        s = X.y + X.w;
        s = s + Xm.z;
        s = s + Xp.z;
        X.z = fmaf(scale, s, B.z) * id0;
    } else {
        const float e = __shfl_down_sync(SP_FULL, X.x, 1);
        float s = X.x + X.z;
        s = s + Xm.y;
        s = s + Xp.y;
        X.y = fmaf(scale, s, B.y) * id0;
        s = X.z + e;
        s = s + Xm.w;
        s = s + Xp.w;
        X.w = fmaf(scale, s, B.w) * id0;
    }
}

// first half sweep from x = 0 (neighbour sum 0); the other colour stays 0
__device__ __forceinline__ float4 sp_first(const float4& B, int sel, float scale, float id0) {
    float4 X = make_float4(0.f, 0.f, 0.f, 0.f);
    if (sel == 0) {
        X.x = fmaf(scale, 0.f, B.x) * id0;
        X.z = fmaf(scale, 0.f, B.z) * id0;
    } else {
        X.y = fmaf(scale, 0.f, B.y) * id0;
        X.w = fmaf(scale, 0.f, B.w) * id0;
    }
    return X;
}

__device__ __forceinline__ float sp_ax(float d0, float ms, float c, float w, float e, float sth, float nth) {
    float ax = d0 * c;
    ax = fmaf(ms, w, ax);
    ax = fmaf(ms, e, ax);
    ax = fmaf(ms, sth, ax);
    return fmaf(ms, nth, ax);
}

// The row loops run SP_U steps per trip, fully unrolled, so that a row's
// registers sit in slot (row - first row) mod SP_U at compile-time indices
// and the sliding window costs no moves.  Strip heights keep the step counts
// multiples of SP_U: pre-smoothing walks rh + 10 rows (rh = 2 mod 6),
// post-smoothing rh + 8 (rh = 4 mod 6).
constexpr int SP_U = 6;

// Pre-smoothing strip: x = 0, (red, black) x 2, x to the r array, r = b - A x,
// b_coarse = R r.  Output columns [o, o + 116), rows [y0, y0 + rh); coarse
// cells [o/2, o/2 + 58) x [y0/2, y0/2 + rh/2).  y0 even.  ring: SP_RING x 32
// float4 (rows of b).
__device__ __forceinline__ void strip_pre(const MgLev<float>& F, const MgLev<float>& C, float4* ring, int o, int y0,
                                          int rh) {
    const int lane = threadIdx.x & 31;
    const int s = o - 6;
    const float* bcol = F.b + s + 4 * lane;
    const int ya = y0 - 5, yb = y0 + rh + 5;  // rows of b read; ya is odd
#pragma unroll
    for (int k = 0; k < SP_RING - 1; ++k) {
        cpa16(&ring[k * 32 + lane], bcol + (size_t)(ya + k) * F.pitch);
        cpa_commit();
    }
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 X[SP_U], B[SP_U];
#pragma unroll
    for (int k = 0; k < SP_U; ++k) {
        X[k] = z4;
        B[k] = z4;
    }
    // restriction sums of the coarse row under way (A: two or three fine rows
    // added) and of the next one (N), over the lane's two coarse columns; fine
    // rows are added in increasing order, weights 1/4, 3/4, 3/4, 1/4
    float2 A = make_float2(0.f, 0.f), N = A;
    const float scale = F.scale, id0 = F.invd[0], d0 = F.diag[0], ms = F.ms;
    const bool out_lo = lane >= 1 && lane <= 30;
    for (int tb = ya; tb < yb; tb += SP_U) {
#pragma unroll
        for (int u = 0; u < SP_U; ++u) {
            const int t = tb + u;
            const int pt = (u + 1) & 1;  // parity of t (tb is odd)
            const int s0 = u, s1 = (u + 5) % 6, s2 = (u + 4) % 6, s3 = (u + 3) % 6, s4 = (u + 2) % 6,
                      s5 = (u + 1) % 6;  // slots of rows t .. t - 5
            const int tn = t + SP_RING - 1;
            if (tn < yb) cpa16(&ring[((u + SP_RING - 1) % SP_RING) * 32 + lane], bcol + (size_t)tn * F.pitch);
            cpa_commit();
            cpa_wait<SP_RING - 1>();
            B[s0] = ring[(u % SP_RING) * 32 + lane];
            X[s0] = sp_first(B[s0], pt, scale, id0);                          // row t, colour 0
            sp_half(X[s1], X[s2], X[s0], B[s1], (pt + 1 + 1) & 1, scale, id0);  // row t - 1, colour 1
            sp_half(X[s2], X[s3], X[s1], B[s2], (pt + 2) & 1, scale, id0);      // row t - 2, colour 0
            sp_half(X[s3], X[s4], X[s2], B[s3], (pt + 3 + 1) & 1, scale, id0);  // row t - 3, colour 1: final
            const int jx = t - 3;
            if (jx >= y0 && jx < y0 + rh && out_lo) {
                float* xr = F.r + (size_t)jx * F.pitch + s + 4 * lane;
                if (lane == 1)
                    *reinterpret_cast<float2*>(xr + 2) = make_float2(X[s3].z, X[s3].w);
                else if (lane == 30)
                    *reinterpret_cast<float2*>(xr) = make_float2(X[s3].x, X[s3].y);
                else
                    *reinterpret_cast<float4*>(xr) = X[s3];
            }
            // residual of row t - 4 and the restriction's row sums
            const float4& Xc = X[s4];
            const float w = __shfl_up_sync(SP_FULL, Xc.w, 1), e = __shfl_down_sync(SP_FULL, Xc.x, 1);
            float4 R;
            R.x = B[s4].x - sp_ax(d0, ms, Xc.x, w, Xc.y, X[s5].x, X[s3].x);
            R.y = B[s4].y - sp_ax(d0, ms, Xc.y, Xc.x, Xc.z, X[s5].y, X[s3].y);
            R.z = B[s4].z - sp_ax(d0, ms, Xc.z, Xc.y, Xc.w, X[s5].z, X[s3].z);
            R.w = B[s4].w - sp_ax(d0, ms, Xc.w, Xc.z, e, X[s5].w, X[s3].w);
            const float rl = __shfl_up_sync(SP_FULL, R.w, 1), rr = __shfl_down_sync(SP_FULL, R.x, 1);
            float2 rs;  // row sums of row t - 4 under the lane's coarse columns
            rs.x = fmaf(0.25f, rl, 0.f);
            rs.x = fmaf(0.75f, R.x, rs.x);
            rs.x = fmaf(0.75f, R.y, rs.x);
            rs.x = fmaf(0.25f, R.z, rs.x);
            rs.y = fmaf(0.25f, R.y, 0.f);
            rs.y = fmaf(0.75f, R.z, rs.y);
            rs.y = fmaf(0.75f, R.w, rs.y);
            rs.y = fmaf(0.25f, rr, rs.y);
            const int jr = t - 4;
            if (pt) {
                // odd fine row 2J + 1: third term of coarse row J, first of J + 1
                A.x = fmaf(0.75f, rs.x, A.x);
                A.y = fmaf(0.75f, rs.y, A.y);
                N.x = fmaf(0.25f, rs.x, 0.f);
                N.y = fmaf(0.25f, rs.y, 0.f);
            } else {
                // even fine row 2J + 2: last term of coarse row J, second of J + 1
                A.x = fmaf(0.25f, rs.x, A.x);
                A.y = fmaf(0.25f, rs.y, A.y);
                if (jr >= y0 + 2 && jr < y0 + rh + 2 && out_lo) {
                    float* cb = C.b + (size_t)((jr - 2) >> 1) * C.pitch + (s >> 1) + 2 * lane;
                    if (lane == 1)
                        cb[1] = 0.25f * A.y;
                    else if (lane == 30)
                        cb[0] = 0.25f * A.x;
                    else
                        *reinterpret_cast<float2*>(cb) = make_float2(0.25f * A.x, 0.25f * A.y);
                }
                A.x = fmaf(0.75f, rs.x, N.x);
                A.y = fmaf(0.75f, rs.y, N.y);
            }
        }
    }
    cpa_wait<0>();
}

// horizontal prolongation weights of one coarse row for the lane's 4 fine
// columns (coarse columns I0 - 1 .. I0 + 2, I0 = first column / 2); lanes 0
// and 31 take the outer neighbours from el and er (the strip's edge columns
// need them: their x enters the half sweeps of the columns next to them)
__device__ __forceinline__ float4 sp_hrow(float2 c, float el, float er) {
    float cl = __shfl_up_sync(SP_FULL, c.y, 1), cr = __shfl_down_sync(SP_FULL, c.x, 1);
    const int lane = threadIdx.x & 31;
    if (lane == 0) cl = el;
    if (lane == 31) cr = er;
    float4 h;
    h.x = fmaf(0.25f, cl, 0.75f * c.x);
    h.y = fmaf(0.25f, c.y, 0.75f * c.x);
    h.z = fmaf(0.25f, c.x, 0.75f * c.y);
    h.w = fmaf(0.25f, cr, 0.75f * c.y);
    return h;
}

// Post-smoothing strip: x = x_pre + P x_coarse, (black, red) x 2, x written.
// Output columns [o, o + 120), rows [y0, y0 + rh); y0 even.  ring: SP_RING
// slots of 32 float4 (b), 32 float4 (x_pre), 32 float2 (coarse row) and the
// coarse row's two outer neighbours (padded to 16 bytes).
constexpr int SP_POST_SLOT = 32 * 4 + 32 * 4 + 32 * 2 + 4;  // floats per slot
__device__ __forceinline__ float strip_post(const MgLev<float>& C, const MgLev<float>& F, float4* ring, int o,
                                            int y0, int rh) {
    float rz = 0.f;  // b.x over the cells this lane writes
    const int lane = threadIdx.x & 31;
    const int s = o - 4;
    const size_t col = (size_t)s + 4 * lane, ccol = (size_t)(s >> 1) + 2 * lane;
    // coarse column read by this lane for the edge neighbour: I0 - 1 (lane 0), I0 + 2 (lane 31)
    const size_t ecol = lane == 0 ? ccol - 1 : ccol + 2;
    const bool edge = lane == 0 || lane == 31;
    const int ya = y0 - 4, yb = y0 + rh + 4;  // rows read: [ya, yb), ya even
    float* rg = reinterpret_cast<float*>(ring);
    auto issue = [&](int row, int slot) {
        float* sl = rg + slot * SP_POST_SLOT;
        if (row < yb) {
            cpa16(sl + 4 * lane, F.b + (size_t)row * F.pitch + col);
            cpa16(sl + 128 + 4 * lane, F.r + (size_t)row * F.pitch + col);
            if (row & 1) {
                const float* crow = C.x + (size_t)((row + 1) >> 1) * C.pitch;
                cpa8(sl + 256 + 2 * lane, crow + ccol);
                if (edge) cpa4(sl + 320 + (lane >> 4), crow + ecol);
            }
        }
        cpa_commit();
    };
#pragma unroll
    for (int k = 0; k < SP_RING - 1; ++k) issue(ya + k, k);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    auto hrow_direct = [&](int J) {
        const float* crow = C.x + (size_t)J * C.pitch;
        const float e = edge ? crow[ecol] : 0.f;
        return sp_hrow(*reinterpret_cast<const float2*>(crow + ccol), e, e);
    };
    // horizontal coarse rows by slot (J - ya / 2) mod 3
    float4 H[3];
    H[0] = hrow_direct(ya / 2);
    H[1] = z4;
    H[2] = hrow_direct(ya / 2 - 1);
    float4 X[SP_U], B[SP_U];
#pragma unroll
    for (int k = 0; k < SP_U; ++k) {
        X[k] = z4;
        B[k] = z4;
    }
    const float scale = F.scale, id0 = F.invd[0];
    const bool out = lane >= 1 && lane <= 30;
    // step t forms x of row t + 1, then sweeps rows t .. t - 3
    for (int tb = ya - 1; tb < yb - 1; tb += SP_U) {
#pragma unroll
        for (int u = 0; u < SP_U; ++u) {
            const int t = tb + u, row = t + 1;
            const int pr = u & 1;  // parity of row (ya is even)
            const int s0 = u, s1 = (u + 5) % 6, s2 = (u + 4) % 6, s3 = (u + 3) % 6, s4 = (u + 2) % 6,
                      s5 = (u + 1) % 6;  // slots of rows t + 1 .. t - 4
            issue(row + SP_RING - 1, (u + SP_RING - 1) % SP_RING);
            cpa_wait<SP_RING - 1>();
            const float* sl = rg + (u % SP_RING) * SP_POST_SLOT;
            B[s0] = *reinterpret_cast<const float4*>(sl + 4 * lane);
            const float4 xr = *reinterpret_cast<const float4*>(sl + 128 + 4 * lane);
            const int ch = ((u + 1) >> 1) % 3, cl = (ch + 2) % 3;  // slots of coarse rows hi, hi - 1
            if (pr) {
                const float e = edge ? sl[320 + (lane >> 4)] : 0.f;
                H[ch] = sp_hrow(*reinterpret_cast<const float2*>(sl + 256 + 2 * lane), e, e);
            }
            const float4 H0 = pr ? H[cl] : H[ch], H1 = pr ? H[ch] : H[cl];  // rows J, NJ
            float4& X0 = X[s0];
            X0.x = xr.x + fmaf(0.25f, H1.x, 0.75f * H0.x);
            X0.y = xr.y + fmaf(0.25f, H1.y, 0.75f * H0.y);
            X0.z = xr.z + fmaf(0.25f, H1.z, 0.75f * H0.z);
            X0.w = xr.w + fmaf(0.25f, H1.w, 0.75f * H0.w);
            // row t has parity 1 - pr
            sp_half(X[s1], X[s2], X[s0], B[s1], (pr + 1 + 1) & 1, scale, id0);  // row t, colour 1
            sp_half(X[s2], X[s3], X[s1], B[s2], (pr + 2) & 1, scale, id0);      // row t - 1, colour 0
            sp_half(X[s3], X[s4], X[s2], B[s3], (pr + 3 + 1) & 1, scale, id0);  // row t - 2, colour 1
            sp_half(X[s4], X[s5], X[s3], B[s4], (pr + 4) & 1, scale, id0);      // row t - 3, colour 0: final
            const int jx = t - 3;
            if (jx >= y0 && jx < y0 + rh && out) {
                *reinterpret_cast<float4*>(F.x + (size_t)jx * F.pitch + col) = X[s4];
                rz = fmaf(B[s4].x, X[s4].x, rz);
                rz = fmaf(B[s4].y, X[s4].y, rz);
                rz = fmaf(B[s4].z, X[s4].z, rz);
                rz = fmaf(B[s4].w, X[s4].w, rz);
            }
        }
    }
    cpa_wait<0>();
    return rz;
}

template <typename T, int TW, int TH>
__global__ void __launch_bounds__(FT_THREADS, FtBlocks<T, TW>::value) k_mg_pre(MgLev<T> F, MgLev<T> C, MgBc p,
                                                                        SolverState* S, int inner,
                                                       StripMap m) {
    if (!block_live(S, inner)) return;
    constexpr int H = 5, W = TW + 2 * H, HT = TH + 2 * H;
    constexpr bool STRIPS = sizeof(T) == 4 && TW == 64;
    constexpr size_t TILE_B = 2 * sizeof(T) * W * HT;
    constexpr size_t RING_B = STRIPS ? (FT_THREADS / 32) * SP_RING * 32 * sizeof(float4) : 0;
    __shared__ __align__(16) unsigned char smem[TILE_B > RING_B ? TILE_B : RING_B];
    if constexpr (STRIPS) {
        if ((int)blockIdx.x >= m.nframe) {
            const int warp = threadIdx.x >> 5;
            const int k = ((int)blockIdx.x - m.nframe) * (FT_THREADS / 32) + warp;
            if (k >= m.ns * m.nr) return;
            const int sx = k % m.ns, sy = k / m.ns;
            strip_pre(F, C, reinterpret_cast<float4*>(smem) + warp * SP_RING * 32, m.x0 + SP_PRE_OUT * sx,
                      m.y0 + m.rh * sy, m.rh);
            return;
        }
    }
    T* xs = reinterpret_cast<T*>(smem);
    T* bs = xs + W * HT;  // b, then r in place on the residual ring
    int tx, ty;
    frame_tile(m, blockIdx.x, tx, ty);
    const int i0 = tx * TW, j0 = ty * TH;
    if (ft_interior<TW, TH, H>(F.nx, F.ny, i0, j0, p)) {
        ft_load_int<T, TW, TH, H>(F, xs, bs, i0, j0, nullptr);
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 0, 5, true);
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 1, 4, false);
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 0, 3, false);
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 1, 2, false);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const T d0 = F.diag[0], ms = F.ms;
        for (int rj = warp; rj < TH + 2; rj += FT_THREADS / 32)
            for (int ci = lane; ci < TW + 2; ci += 32) {
                const int q = (rj + H - 1) * W + (ci + H - 1);
                T ax = d0 * xs[q];
                ax = mg_fma(ms, xs[q - 1], ax);
                ax = mg_fma(ms, xs[q + 1], ax);
                ax = mg_fma(ms, xs[q - W], ax);
                ax = mg_fma(ms, xs[q + W], ax);
                bs[q] = bs[q] - ax;
            }
        __syncthreads();
        for (int k = threadIdx.x; k < TW * TH; k += FT_THREADS) {
            const int li = k % TW, lj = k / TW;
            F.r[(size_t)(j0 + lj) * F.pitch + i0 + li] = xs[(lj + H) * W + li + H];
        }
        // restriction with the interior weights 1/4, 3/4, 3/4, 1/4 per axis
        const T w4[4] = {T(0.25), T(0.75), T(0.75), T(0.25)};
        for (int k = threadIdx.x; k < (TW / 2) * (TH / 2); k += FT_THREADS) {
            const int ci = k % (TW / 2), cj = k / (TW / 2);
            const int qr = (2 * cj - 1 + H) * W + (2 * ci - 1 + H);
            T acc = T(0);
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const T* row = bs + qr + a * W;
                T rs = T(0);
#pragma unroll
                for (int b = 0; b < 4; ++b) rs = mg_fma(w4[b], row[b], rs);
                acc = mg_fma(w4[a], rs, acc);
            }
            C.b[(size_t)(j0 / 2 + cj) * C.pitch + i0 / 2 + ci] = T(0.25) * acc;
        }
        return;
    }
    ft_load<T, TW, TH, H>(F, p, xs, bs, i0, j0, nullptr);
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 0, 5, true);
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 1, 4, false);
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 0, 3, false);
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 1, 2, false);
    // residual on the tile grown by 1 (read by the restriction), in place of b
    {
        const int ncol = TW + 2, nrow = TH + 2;
        for (int k = threadIdx.x; k < ncol * nrow; k += FT_THREADS) {
            const int gi = i0 - 1 + k % ncol, gj = j0 - 1 + k / ncol;
            const int wi = mg_dom(gi, F.nx, p.per_x), wj = mg_dom(gj, F.ny, p.per_y);
            if (wi < 0 || wj < 0) continue;
            const int q = (gj - (j0 - H)) * W + (gi - (i0 - H));
            T ax = F.diag[mg_bits(p, F.nx, F.ny, wi, wj)] * xs[q];
            ax = mg_fma(F.ms, xs[q - 1], ax);
            ax = mg_fma(F.ms, xs[q + 1], ax);
            ax = mg_fma(F.ms, xs[q - W], ax);
            ax = mg_fma(F.ms, xs[q + W], ax);
            bs[q] = bs[q] - ax;
        }
    }
    __syncthreads();
    // x on the tile, into the r array (read back by k_mg_post)
    for (int k = threadIdx.x; k < TW * TH; k += FT_THREADS) {
        const int gi = i0 + k % TW, gj = j0 + k / TW;
        if (gi < F.nx && gj < F.ny) F.r[(size_t)gj * F.pitch + gi] = xs[(gj - (j0 - H)) * W + (gi - (i0 - H))];
    }
    // restriction of the coarse cells under the tile
    for (int k = threadIdx.x; k < (TW / 2) * (TH / 2); k += FT_THREADS) {
        const int I = i0 / 2 + k % (TW / 2), J = j0 / 2 + k / (TW / 2);
        if (I >= C.nx || J >= C.ny) continue;
        T acc = T(0);
        for (int fy0 = 2 * J - 1; fy0 <= 2 * J + 2; ++fy0) {
            const int fy = mg_dom(fy0, F.ny, p.per_y);
            if (fy < 0) continue;
            const T wy = (T)mg_pwq(fy, J, C.ny, p.per_y, p.bc[1], p.bc[3]) * T(0.25);
            const int rowq = (fy0 - (j0 - H)) * W - (i0 - H);
            T rs = T(0);
            for (int fx0 = 2 * I - 1; fx0 <= 2 * I + 2; ++fx0) {
                const int fx = mg_dom(fx0, F.nx, p.per_x);
                if (fx < 0) continue;
                const T wx = (T)mg_pwq(fx, I, C.nx, p.per_x, p.bc[0], p.bc[2]) * T(0.25);
                rs = mg_fma(wx, bs[rowq + fx0], rs);
            }
            acc = mg_fma(wy, rs, acc);
        }
        C.b[(size_t)J * C.pitch + I] = T(0.25) * acc;
    }
}

template <typename T, int TW, int TH>
__global__ void __launch_bounds__(FT_THREADS, FtBlocks<T, TW>::value) k_mg_post(MgLev<T> C, MgLev<T> F, MgBc p,
                                                                         SolverState* S, int inner,
                                                           StripMap m, RzEpi E) {
    if (!block_live(S, inner)) return;
    constexpr int H = 4, W = TW + 2 * H, HT = TH + 2 * H;
    // coarse cells read by the prolongation of an interior tile's array
    constexpr int CW = TW / 2 + H + 2, CH = TH / 2 + H + 2;
    constexpr bool STRIPS = sizeof(T) == 4 && TW == 64;
    constexpr size_t TILE_B = sizeof(T) * (2 * W * HT + CW * CH);
    constexpr size_t RING_B = STRIPS ? (FT_THREADS / 32) * SP_RING * SP_POST_SLOT * sizeof(float) : 0;
    __shared__ __align__(16) unsigned char smem[TILE_B > RING_B ? TILE_B : RING_B];
    const int nparts = m.nframe + m.ns * m.nr;
    if constexpr (STRIPS) {
        if ((int)blockIdx.x >= m.nframe) {
            const int warp = threadIdx.x >> 5;
            const int k = ((int)blockIdx.x - m.nframe) * (FT_THREADS / 32) + warp;
            float rz = 0.f;
            if (k < m.ns * m.nr) {
                const int sx = k % m.ns, sy = k / m.ns;
                rz = strip_post(C, F, reinterpret_cast<float4*>(smem) + warp * SP_RING * (SP_POST_SLOT / 4),
                                m.x0 + SP_POST_OUT * sx, m.y0 + m.rh * sy, m.rh);
            }
            if (E.on) {
                const double d = warp_fold((double)rz);
                if (k < m.ns * m.nr && (threadIdx.x & 31) == 0) E.part[m.nframe + k] = d;
                rz_finish(E, S, nparts);
            }
            return;
        }
    }
    T* xs = reinterpret_cast<T*>(smem);
    T* bs = xs + W * HT;
    T* cs = bs + W * HT;
    int tx, ty;
    frame_tile(m, blockIdx.x, tx, ty);
    const int i0 = tx * TW, j0 = ty * TH;
    if (ft_interior<TW, TH, H>(F.nx, F.ny, i0, j0, p)) {
        // coarse block from (i0 - H) / 2 - 1, (j0 - H) / 2 - 1 (wrapped
        // along periodic axes)
        const int ci0 = (i0 - H) / 2 - 1, cj0 = (j0 - H) / 2 - 1;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int cj = warp; cj < CH; cj += FT_THREADS / 32) {
            const size_t crow = (size_t)mg_wrap(cj0 + cj, C.ny) * C.pitch;
            for (int ci = lane; ci < CW; ci += 32) cs[cj * CW + ci] = C.x[crow + mg_wrap(ci0 + ci, C.nx)];
        }
        __syncthreads();
        // b, and x (kept in the r array by k_mg_pre) plus the prolongation,
        // one warp per row
        for (int lj = warp; lj < HT; lj += FT_THREADS / 32) {
            const int fy = j0 - H + lj;
            const int J = (fy >> 1) - cj0, NJ = J + ((fy & 1) ? 1 : -1);
            const T* c0 = cs + J * CW;
            const T* c1 = cs + NJ * CW;
            const size_t frow = (size_t)mg_wrap(fy, F.ny) * F.pitch;
            for (int li = lane; li < W; li += 32) {
                const int fx = i0 - H + li;
                const int I = (fx >> 1) - ci0, NI = I + ((fx & 1) ? 1 : -1);
                T row0 = T(0.75) * c0[I];
                row0 = mg_fma(T(0.25), c0[NI], row0);
                T v = T(0.75) * row0;
                T row1 = T(0.75) * c1[I];
                row1 = mg_fma(T(0.25), c1[NI], row1);
                v = mg_fma(T(0.25), row1, v);
                const size_t k = frow + mg_wrap(fx, F.nx);
                bs[lj * W + li] = F.b[k];
                xs[lj * W + li] = F.r[k] + v;
            }
        }
        __syncthreads();
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 1, 3, false);
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 0, 2, false);
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 1, 1, false);
        ft_half_int<T, TW, TH, H>(F, xs, bs, i0, j0, 0, 0, false);
        T rz = T(0);
        for (int k = threadIdx.x; k < TW * TH; k += FT_THREADS) {
            const int li = k % TW, lj = k / TW, gi = i0 + li, gj = j0 + lj;
            const int q = (lj + H) * W + li + H;
            T* row = F.x + (size_t)gj * F.pitch;
            row[gi] = xs[q];
            if (E.on) {
                if (!in_strips(m, gi, gj)) rz = mg_fma(bs[q], xs[q], rz);
                // ghost copies along periodic axes (the finest level's x has a ghost ring)
                if (p.per_x) {
                    if (gi == 0) row[F.nx] = xs[q];
                    if (gi == F.nx - 1) row[-1] = xs[q];
                }
                if (p.per_y) {
                    if (gj == 0) F.x[(ptrdiff_t)F.ny * F.pitch + gi] = xs[q];
                    if (gj == F.ny - 1) F.x[-(ptrdiff_t)F.pitch + gi] = xs[q];
                }
            }
        }
        if (E.on) post_epilogue(E, S, nparts, (double)rz);
        return;
    }
    ft_load<T, TW, TH, H>(F, p, xs, bs, i0, j0, F.r);
    // x += P x_coarse on every cell of the array inside the domain
    for (int q = threadIdx.x; q < W * HT; q += FT_THREADS) {
        const int fx = mg_dom(i0 - H + q % W, F.nx, p.per_x), fy = mg_dom(j0 - H + q / W, F.ny, p.per_y);
        if (fx < 0 || fy < 0) continue;
        int I, NI, J, NJ;
        T wxI, wxN, wyJ, wyN;
        mg_axis<T>(fx, C.nx, p.per_x, p.bc[0], p.bc[2], I, NI, wxI, wxN);
        mg_axis<T>(fy, C.ny, p.per_y, p.bc[1], p.bc[3], J, NJ, wyJ, wyN);
        T row0 = wxI * C.x[(size_t)J * C.pitch + I];
        if (NI >= 0) row0 = mg_fma(wxN, C.x[(size_t)J * C.pitch + NI], row0);
        T v = wyJ * row0;
        if (NJ >= 0) {
            T row1 = wxI * C.x[(size_t)NJ * C.pitch + I];
            if (NI >= 0) row1 = mg_fma(wxN, C.x[(size_t)NJ * C.pitch + NI], row1);
            v = mg_fma(wyN, row1, v);
        }
        xs[q] = xs[q] + v;
    }
    __syncthreads();
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 1, 3, false);
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 0, 2, false);
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 1, 1, false);
    ft_half<T, TW, TH, H>(F, p, xs, bs, i0, j0, 0, 0, false);
    T rz = T(0);
    for (int k = threadIdx.x; k < TW * TH; k += FT_THREADS) {
        const int gi = i0 + k % TW, gj = j0 + k / TW;
        if (gi < F.nx && gj < F.ny) {
            const int q = (gj - (j0 - H)) * W + (gi - (i0 - H));
            const T v = xs[q];
            T* row = F.x + (size_t)gj * F.pitch;
            row[gi] = v;
            if (E.on) {
                if (!in_strips(m, gi, gj)) rz = mg_fma(bs[q], v, rz);
                // ghost copies along periodic axes (the finest level's x has a ghost ring)
                if (p.per_x) {
                    if (gi == 0) row[F.nx] = v;
                    if (gi == F.nx - 1) row[-1] = v;
                }
                if (p.per_y) {
                    if (gj == 0) F.x[(ptrdiff_t)F.ny * F.pitch + gi] = v;
                    if (gj == F.ny - 1) F.x[-(ptrdiff_t)F.pitch + gi] = v;
                }
            }
        }
    }
    if (E.on) post_epilogue(E, S, nparts, (double)rz);
}

// tile shapes: 64 x 32 (FP64: 64 x 24, both arrays in 48 KB of shared
// memory) on large levels; 32 x 16 on levels with fewer than 1024 large tiles,
// where more, smaller CTAs shorten the latency-bound passes
template <typename T>
struct FtRows {
    static constexpr int value = 32;
};
template <>
struct FtRows<double> {
    static constexpr int value = 24;
};

// ---------------------------------------------------------------------------
// Bottom of the V-cycle in one CTA: every level with at most MgBottomMax
// cells, from the restricted right-hand side of the first of them down to the
// coarsest and back, in shared memory.  The per-cell arithmetic is the same as
// in the grid kernels above (same formulas and order), so the result is the
// same as that of the level-by-level launches; each phase ends at a barrier.
// Levels up to 32^2 go to the one CTA: a 64^2 level's eleven phases there
// (2048 cells per half sweep on one SM) took longer than its two tile
// launches (8 CTAs each), in FP32 as in FP64.
template <typename T>
struct MgBottomMax {
    static constexpr int value = 1024;
};
constexpr int MG_BOTTOM_LEVELS = 6;
constexpr int MG_BOTTOM_THREADS = 1024;

template <typename T>
struct MgBottom {
    MgLev<T> lev[MG_BOTTOM_LEVELS];  // lev[0]: b read from and x written to global memory
    int off[MG_BOTTOM_LEVELS];       // shared-memory offsets (elements) of x, b, r: off, off + n, off + 2n
    int nlev;
};

template <typename T>
__device__ __forceinline__ T gs_cell(const MgBc& p, const T* x, int nx, int ny, int gi, int gj, T bval, T scale,
                                     const T* invd, bool first) {
    T s;
    if (first) {
        s = T(0);
    } else {
        s = mg_at(p, x, nx, nx, ny, gi - 1, gj) + mg_at(p, x, nx, nx, ny, gi + 1, gj);
        s = s + mg_at(p, x, nx, nx, ny, gi, gj - 1);
        s = s + mg_at(p, x, nx, nx, ny, gi, gj + 1);
    }
    T t = mg_fma(scale, s, bval);
    return t * invd[mg_bits(p, nx, ny, gi, gj)];
}

template <typename T>
__global__ void __launch_bounds__(MG_BOTTOM_THREADS) k_mg_bottom(MgBottom<T> P, MgBc p, SolverState* S, int inner) {
    if (!block_live(S, inner)) return;
    extern __shared__ __align__(16) unsigned char mg_smem[];
    T* sm = reinterpret_cast<T*>(mg_smem);
    // 32 x 32 threads: tx walks columns (or column pairs), ty rows
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    auto X = [&](int l) { return sm + P.off[l]; };
    auto B = [&](int l) { return sm + P.off[l] + P.lev[l].nx * P.lev[l].ny; };
    auto R = [&](int l) { return sm + P.off[l] + 2 * P.lev[l].nx * P.lev[l].ny; };
    {
        const MgLev<T>& G = P.lev[0];
        T* b = B(0);
        for (int gj = ty; gj < G.ny; gj += 32)
            for (int gi = tx; gi < G.nx; gi += 32) b[gj * G.nx + gi] = G.b[(size_t)gj * G.pitch + gi];
    }
    __syncthreads();
    auto half = [&](int l, int color, bool first) {
        const MgLev<T>& L = P.lev[l];
        T* x = X(l);
        const T* b = B(l);
        const int pairs = (L.nx + 1) / 2;
        for (int gj = ty; gj < L.ny; gj += 32) {
            const int par = (gj + color) & 1;
            for (int pr = tx; pr < pairs; pr += 32) {
                const int gi = 2 * pr + par, go = 2 * pr + 1 - par;
                if (gi < L.nx)
                    x[gj * L.nx + gi] = gs_cell(p, x, L.nx, L.ny, gi, gj, b[gj * L.nx + gi], L.scale, L.invd, first);
                if (first && go < L.nx) x[gj * L.nx + go] = T(0);
            }
        }
        __syncthreads();
    };
    auto residual = [&](int l) {
        const MgLev<T>& L = P.lev[l];
        const T* x = X(l);
        const T* b = B(l);
        T* r = R(l);
        for (int gj = ty; gj < L.ny; gj += 32)
            for (int gi = tx; gi < L.nx; gi += 32) {
                const int k = gj * L.nx + gi;
                T ax = L.diag[mg_bits(p, L.nx, L.ny, gi, gj)] * x[k];
                ax = mg_fma(L.ms, mg_at(p, x, L.nx, L.nx, L.ny, gi - 1, gj), ax);
                ax = mg_fma(L.ms, mg_at(p, x, L.nx, L.nx, L.ny, gi + 1, gj), ax);
                ax = mg_fma(L.ms, mg_at(p, x, L.nx, L.nx, L.ny, gi, gj - 1), ax);
                ax = mg_fma(L.ms, mg_at(p, x, L.nx, L.nx, L.ny, gi, gj + 1), ax);
                r[k] = b[k] - ax;
            }
        __syncthreads();
    };
    auto restrict_to = [&](int l) {
        const MgLev<T>& F = P.lev[l];
        const MgLev<T>& C = P.lev[l + 1];
        const T* fr = R(l);
        T* cb = B(l + 1);
        for (int J = ty; J < C.ny; J += 32)
            for (int I = tx; I < C.nx; I += 32) {
                T acc = T(0);
                for (int fy0 = 2 * J - 1; fy0 <= 2 * J + 2; ++fy0) {
                    int fy = fy0;
                    if (fy < 0 || fy >= F.ny) {
                        if (!p.per_y) continue;
                        fy = fy < 0 ? fy + F.ny : fy - F.ny;
                    }
                    const T wy = (T)mg_pwq(fy, J, C.ny, p.per_y, p.bc[1], p.bc[3]) * T(0.25);
                    T rs = T(0);
                    for (int fx0 = 2 * I - 1; fx0 <= 2 * I + 2; ++fx0) {
                        int fx = fx0;
                        if (fx < 0 || fx >= F.nx) {
                            if (!p.per_x) continue;
                            fx = fx < 0 ? fx + F.nx : fx - F.nx;
                        }
                        const T wx = (T)mg_pwq(fx, I, C.nx, p.per_x, p.bc[0], p.bc[2]) * T(0.25);
                        rs = mg_fma(wx, fr[fy * F.nx + fx], rs);
                    }
                    acc = mg_fma(wy, rs, acc);
                }
                cb[J * C.nx + I] = T(0.25) * acc;
            }
        __syncthreads();
    };
    auto prolong_from = [&](int l) {  // x_l += P x_{l+1}
        const MgLev<T>& F = P.lev[l];
        const MgLev<T>& C = P.lev[l + 1];
        const T* cx = X(l + 1);
        T* fxs = X(l);
        for (int fy = ty; fy < F.ny; fy += 32)
            for (int fx = tx; fx < F.nx; fx += 32) {
                int I, NI, J, NJ;
                T wxI, wxN, wyJ, wyN;
                mg_axis<T>(fx, C.nx, p.per_x, p.bc[0], p.bc[2], I, NI, wxI, wxN);
                mg_axis<T>(fy, C.ny, p.per_y, p.bc[1], p.bc[3], J, NJ, wyJ, wyN);
                T row0 = wxI * cx[J * C.nx + I];
                if (NI >= 0) row0 = mg_fma(wxN, cx[J * C.nx + NI], row0);
                T v = wyJ * row0;
                if (NJ >= 0) {
                    T row1 = wxI * cx[NJ * C.nx + I];
                    if (NI >= 0) row1 = mg_fma(wxN, cx[NJ * C.nx + NI], row1);
                    v = mg_fma(wyN, row1, v);
                }
                fxs[fy * F.nx + fx] = fxs[fy * F.nx + fx] + v;
            }
        __syncthreads();
    };
    const int nb = P.nlev;
    for (int l = 0; l < nb - 1; ++l) {
        for (int k = 0; k < MG_NU; ++k) {
            half(l, 0, k == 0);
            half(l, 1, false);
        }
        residual(l);
        restrict_to(l);
    }
    for (int k = 0; k < MG_NC; ++k) {
        half(nb - 1, 0, k == 0);
        half(nb - 1, 1, false);
    }
    for (int k = 0; k < MG_NC; ++k) {
        half(nb - 1, 1, false);
        half(nb - 1, 0, false);
    }
    for (int l = nb - 2; l >= 0; --l) {
        prolong_from(l);
        for (int k = 0; k < MG_NU; ++k) {
            half(l, 1, false);
            half(l, 0, false);
        }
    }
    {
        const MgLev<T>& G = P.lev[0];
        const T* x = X(0);
        for (int gj = ty; gj < G.ny; gj += 32)
            for (int gi = tx; gi < G.nx; gi += 32) G.x[(size_t)gj * G.pitch + gi] = x[gj * G.nx + gi];
    }
}

// --------------------------------------------------------------------------
// host side: hierarchy and the V-cycle launch sequence

template <typename T>
static void level_tables(const cf_ctx* c, double scale, MgLev<T>& L) {
    for (int b = 0; b < 16; ++b) {
        double d = 4.0 * scale;
        if ((b & 1) && c->ph.bc[0] == CF_BC_SOLID) d = d - scale;
        if ((b & 2) && c->ph.bc[2] == CF_BC_SOLID) d = d - scale;
        if ((b & 4) && c->ph.bc[1] == CF_BC_SOLID) d = d - scale;
        if ((b & 8) && c->ph.bc[3] == CF_BC_SOLID) d = d - scale;
        L.diag[b] = (T)d;
        L.invd[b] = (T)(1.0 / d);
    }
    L.scale = (T)scale;
    L.ms = (T)(-1.0 * scale);
}

// first level handled by the one-CTA bottom solver (nlev when none is small
// enough) and the bytes of shared memory it needs
template <typename T>
static int bottom_level(const MgLev<T>* lev, int nlev, size_t* smem) {
    int lb = nlev;
    for (int l = 0; l < nlev; ++l)
        if ((long long)lev[l].nx * lev[l].ny <= MgBottomMax<T>::value && nlev - l <= MG_BOTTOM_LEVELS) {
            lb = l;
            break;
        }
    size_t n = 0;
    for (int l = lb; l < nlev; ++l) n += 3 * (size_t)lev[l].nx * lev[l].ny;
    *smem = n * sizeof(T);
    return lb;
}

struct MgHierarchy {
    int nlev = 0;
    int fused = -1;  // 1: all levels fused, 0: none, -1: by level (see vcycle)
    int strip_rows = 32;  // rows per FP32 register strip (0: tiles only)
    int rz_fused = 1;     // mixed: r.z and z's ghosts in the finest post-smoothing kernel
    MgLev<double> d[16];
    MgLev<float> f[16];
    double* z64 = nullptr;
    float* r32s = nullptr;  // level-0 residual scratch (mixed)
    std::vector<void*> allocs;
};

static int mg_alloc(cf_ctx* c, MgHierarchy* H, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(c, CF_ERR_NOMEM, "multigrid: cudaMalloc of %zu bytes failed", bytes);
    H->allocs.push_back(*p);
    return cuda_check(c, cudaMemsetAsync(*p, 0, bytes, c->stream), "multigrid memset");
}

// Halve a level while both axes are even and at least 16, and the halved
// extent stays even along periodic axes (so that no two cells of one colour
// are neighbours through the wrap and every half sweep is order-free).
bool mg_coarsen_ok(int nx, int ny, int per_x, int per_y) {
    if ((nx & 1) || (ny & 1) || nx < 16 || ny < 16) return false;
    if (per_x && ((nx / 2) & 1)) return false;
    if (per_y && ((ny / 2) & 1)) return false;
    return true;
}

// Build the hierarchy once per context (the sizes depend on the grid only).
int mg_setup(cf_ctx* c) {
    if (c->mg) return CF_OK;
    if ((c->ph.per_x && (c->ph.nx & 1)) || (c->ph.per_y && (c->ph.ny & 1)))
        return fail(c, CF_ERR_UNSUPPORTED, "multigrid needs an even cell count along periodic axes");
    const bool mixed = c->precision == CF_PREC_MIXED;
    int rc = mixed ? cg32_mg_setup(c) : CF_OK;
    if (rc) return rc;
    MgHierarchy* H = new MgHierarchy();
    c->mg = H;
    if (const char* e = getenv("CF_MG_FUSED")) H->fused = atoi(e) != 0;
    if (const char* e = getenv("CF_MG_STRIPS")) H->strip_rows = atoi(e);
    if (const char* e = getenv("CF_MG_RZ_FUSED")) H->rz_fused = atoi(e) != 0;
    int nx = c->ph.nx, ny = c->ph.ny;
    for (int l = 0; l < 16 && !rc; ++l) {
        if (l == 0) {
            if (!mixed) {
                rc = mg_alloc(c, H, (void**)&H->z64, sizeof(double) * (size_t)c->vpitch * ny);
                H->d[0] = MgLev<double>{H->z64, c->r.a, c->qv.a, nx, ny, c->vpitch};
            } else {
                rc = mg_alloc(c, H, (void**)&H->r32s, sizeof(float) * (size_t)c->p32 * ny);
                H->f[0] = MgLev<float>{c->z32.a, c->r32.a, H->r32s, nx, ny, c->p32};
            }
        } else {
            const int pitch = (nx + 31) / 32 * 32;
            const size_t bytes = (mixed ? sizeof(float) : sizeof(double)) * (size_t)pitch * ny;
            void *x = nullptr, *b = nullptr, *r = nullptr;
            rc = mg_alloc(c, H, &x, bytes);
            if (!rc) rc = mg_alloc(c, H, &b, bytes);
            if (!rc) rc = mg_alloc(c, H, &r, bytes);
            if (!mixed)
                H->d[l] = MgLev<double>{(double*)x, (double*)b, (double*)r, nx, ny, pitch};
            else
                H->f[l] = MgLev<float>{(float*)x, (float*)b, (float*)r, nx, ny, pitch};
        }
        H->nlev = l + 1;
        if (!mg_coarsen_ok(nx, ny, c->ph.per_x, c->ph.per_y)) break;
        nx /= 2;
        ny /= 2;
    }
    if (!rc) {
        size_t smem = 0;
        if (mixed)
            bottom_level(H->f, H->nlev, &smem);
        else
            bottom_level(H->d, H->nlev, &smem);
        cudaError_t e = mixed ? cudaFuncSetAttribute(k_mg_bottom<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)smem)
                              : cudaFuncSetAttribute(k_mg_bottom<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)smem);
        rc = cuda_check(c, e, "multigrid bottom solver shared memory");
    }
    return rc;
}

void mg_free(cf_ctx* c) {
    MgHierarchy* H = static_cast<MgHierarchy*>(c->mg);
    if (!H) return;
    for (void* p : H->allocs) cudaFree(p);
    delete H;
    c->mg = nullptr;
}

double* mg_z64(cf_ctx* c) { return static_cast<MgHierarchy*>(c->mg)->z64; }

// fused = 1: levels above the bottom solver run the fused pre/post kernels;
// 0: one launch per half sweep, residual, restriction and prolongation (the
// same arithmetic); -1 (default): fused for FP32 levels, which are bound by
// memory traffic, and for FP64 levels of at most 2^20 cells, which are bound
// by launch latency; larger FP64 levels are bound by the FP64 pipe, where the
// fused tiles' halo recomputation costs more than it saves.  CF_MG_FUSED=0/1
// in the environment forces one form.
// Launch geometry of a fused pre (or post) launch: tiles of tw x th over the
// level; with strip_rows > 0 (FP32 64-wide tiles only), register strips of
// that many rows over the interior and tiles only over the frame around them.
static StripMap strip_map(int nx, int ny, int tw, int th, int strip_rows, bool pre) {
    StripMap m{};
    m.ntx = (nx + tw - 1) / tw;
    const int nty = (ny + th - 1) / th;
    m.tya = m.tyb = nty;  // default: every tile in the first band
    m.nframe = m.ntx * nty;
    if (strip_rows <= 0) return m;
    // strip height nearest to strip_rows with rh + 2 hr a multiple of SP_U
    const int hr = pre ? 5 : 4, want = (SP_U - (2 * hr) % SP_U) % SP_U;
    const int dn = strip_rows - (((strip_rows - want) % SP_U) + SP_U) % SP_U, up = dn + SP_U;
    const int rh = dn >= 2 && strip_rows - dn < up - strip_rows ? dn : up;
    const int out = pre ? SP_PRE_OUT : SP_POST_OUT, hc = pre ? 6 : 4;
    const int x0 = 4 + hc, y0 = 6;  // first strip reads from column 4, row y0 - hr >= 1
    const int span = nx - 1 - SP_COLS - 4;  // last strip: 4 + out (ns - 1) + 128 <= nx - 1
    const int ns = span >= 0 ? span / out + 1 : 0;
    const int nr = (ny - 1 - hr - y0) / rh;  // y0 + rh nr + hr <= ny - 1
    if (ns < 1 || nr < 1) return m;
    const int xb = x0 + out * ns, yb = y0 + rh * nr;
    const int txa = (x0 + tw - 1) / tw, txb = xb / tw, tya = (y0 + th - 1) / th, tyb = yb / th;
    if (txa >= txb || tya >= tyb) return m;
    m.txa = txa;
    m.txb = txb;
    m.tya = tya;
    m.tyb = tyb;
    m.nframe = m.ntx * nty - (txb - txa) * (tyb - tya);
    m.ns = ns;
    m.nr = nr;
    m.rh = rh;
    m.x0 = x0;
    m.y0 = y0;
    return m;
}

static int launch_blocks(const StripMap& m) { return m.nframe + (m.ns * m.nr + FT_THREADS / 32 - 1) / (FT_THREADS / 32); }

// The launch geometry above, on the host, for tests: the StripMap fields, the
// strip shape constants and the tile of every frame block (host arithmetic
// only; nothing is launched).
int mg_strip_geometry(int nx, int ny, int tw, int th, int strip_rows, int pre, int* fields, int* frame_xy, int cap) {
    const StripMap m = strip_map(nx, ny, tw, th, strip_rows, pre != 0);
    const int v[CF_STRIP_FIELDS] = {m.nframe, m.ntx, m.txa, m.txb, m.tya, m.tyb, m.ns, m.nr, m.rh, m.x0, m.y0,
                                    pre ? SP_PRE_OUT : SP_POST_OUT, pre ? 6 : 4, pre ? 5 : 4, SP_COLS, SP_U,
                                    FT_THREADS / 32, launch_blocks(m)};
    for (int k = 0; k < CF_STRIP_FIELDS; ++k) fields[k] = v[k];
    if (frame_xy)
        for (int f = 0; f < m.nframe && f < cap; ++f) frame_tile(m, f, frame_xy[2 * f], frame_xy[2 * f + 1]);
    return CF_OK;
}

template <typename T>
static int vcycle(cf_ctx* c, MgLev<T>* lev, int nlev, double scale0, int inner, int fused, int strip_rows,
                  double* epi_part, bool* epi_done) {
    MgBc p{c->ph.per_x, c->ph.per_y, {c->ph.bc[0], c->ph.bc[1], c->ph.bc[2], c->ph.bc[3]}};
    double s = scale0;
    for (int l = 0; l < nlev; ++l) {
        level_tables(c, s, lev[l]);
        s = s * 0.25;
    }
    const dim3 blk(MG_BX, MG_BY);
    const int rows = MG_BY * MG_ROWS;
    auto grid2 = [&](int nx, int ny) { return dim3((nx + MG_BX - 1) / MG_BX, (ny + rows - 1) / rows); };
    int launches = 0;
    auto smooth = [&](int l, int color, int first) {
        const MgLev<T>& L = lev[l];
        k_mg_smooth<T><<<grid2((L.nx + 1) / 2, L.ny), blk, 0, c->stream>>>(L, p, color, first, c->S, inner);
        ++launches;
    };
    size_t smem = 0;
    const int lb = bottom_level(lev, nlev, &smem);
    const int top_end = lb < nlev ? lb : nlev - 1;  // levels smoothed by grid kernels on the way down
    constexpr int TH = FtRows<T>::value;
    auto big = [&](const MgLev<T>& L) { return (long long)((L.nx + 63) / 64) * ((L.ny + TH - 1) / TH) >= 1024; };
    auto fuse_level = [&](int l) {
        if (fused >= 0) return fused != 0;
        return sizeof(T) == 4 || (long long)lev[l].nx * lev[l].ny <= (1ll << 20);
    };
    const int srows = sizeof(T) == 4 ? strip_rows : 0;
    for (int l = 0; l < top_end; ++l) {
        if (fuse_level(l)) {
            if (big(lev[l])) {
                const StripMap m = strip_map(lev[l].nx, lev[l].ny, 64, TH, srows, true);
                k_mg_pre<T, 64, TH><<<launch_blocks(m), FT_THREADS, 0, c->stream>>>(lev[l], lev[l + 1], p, c->S,
                                                                                   inner, m);
            } else {
                const StripMap m = strip_map(lev[l].nx, lev[l].ny, 32, 16, 0, true);
                k_mg_pre<T, 32, 16><<<launch_blocks(m), FT_THREADS, 0, c->stream>>>(lev[l], lev[l + 1], p, c->S,
                                                                                   inner, m);
            }
            ++launches;
            continue;
        }
        for (int k = 0; k < MG_NU; ++k) {
            smooth(l, 0, k == 0);
            smooth(l, 1, 0);
        }
        k_mg_residual<T><<<grid2(lev[l].nx, lev[l].ny), blk, 0, c->stream>>>(lev[l], p, c->S, inner);
        k_mg_restrict<T><<<grid2(lev[l + 1].nx, lev[l + 1].ny), blk, 0, c->stream>>>(lev[l], lev[l + 1], p, c->S,
                                                                                      inner);
        launches += 2;
    }
    if (lb < nlev) {
        MgBottom<T> P{};
        P.nlev = nlev - lb;
        int off = 0;
        for (int l = 0; l < P.nlev; ++l) {
            P.lev[l] = lev[lb + l];
            P.off[l] = off;
            off += 3 * lev[lb + l].nx * lev[lb + l].ny;
        }
        k_mg_bottom<T><<<1, MG_BOTTOM_THREADS, smem, c->stream>>>(P, p, c->S, inner);
        ++launches;
    } else {
        // coarsest level too large for one CTA: sweeps by grid kernels
        for (int k = 0; k < MG_NC; ++k) {
            smooth(nlev - 1, 0, k == 0);
            smooth(nlev - 1, 1, 0);
        }
        for (int k = 0; k < MG_NC; ++k) {
            smooth(nlev - 1, 1, 0);
            smooth(nlev - 1, 0, 0);
        }
    }
    for (int l = top_end - 1; l >= 0; --l) {
        if (fuse_level(l)) {
            RzEpi E{0, epi_part};
            if (l == 0 && epi_part) {
                E.on = 1;
                *epi_done = true;
            }
            if (big(lev[l])) {
                const StripMap m = strip_map(lev[l].nx, lev[l].ny, 64, TH, srows, false);
                k_mg_post<T, 64, TH><<<launch_blocks(m), FT_THREADS, 0, c->stream>>>(lev[l + 1], lev[l], p, c->S,
                                                                                    inner, m, E);
            } else {
                const StripMap m = strip_map(lev[l].nx, lev[l].ny, 32, 16, 0, false);
                k_mg_post<T, 32, 16><<<launch_blocks(m), FT_THREADS, 0, c->stream>>>(lev[l + 1], lev[l], p, c->S,
                                                                                    inner, m, E);
            }
            ++launches;
            continue;
        }
        k_mg_prolong<T><<<grid2(lev[l].nx, lev[l].ny), blk, 0, c->stream>>>(lev[l + 1], lev[l], p, c->S, inner);
        ++launches;
        for (int k = 0; k < MG_NU; ++k) {
            smooth(l, 1, 0);
            smooth(l, 0, 0);
        }
    }
    return launches;
}

// Enqueue z = V-cycle(r) at stencil scale scale0 (FP64: z64 <- r; mixed:
// z32 <- r32) and return the number of kernels launched.  Every kernel
// returns at once when the solve has stopped.
int mg_vcycle(cf_ctx* c, double scale0, bool* rz_done) {
    MgHierarchy* H = static_cast<MgHierarchy*>(c->mg);
    bool done = false;
    int n;
    if (c->precision == CF_PREC_MIXED)
        n = vcycle<float>(c, H->f, H->nlev, scale0, 1, H->fused, H->strip_rows,
                          rz_done && H->rz_fused ? c->partials : nullptr, &done);
    else
        n = vcycle<double>(c, H->d, H->nlev, scale0, 0, H->fused, 0, nullptr, &done);
    if (rz_done) *rz_done = done;
    return n;
}

int mg_levels(const cf_ctx* c) { return c->mg ? static_cast<const MgHierarchy*>(c->mg)->nlev : 0; }

}  // namespace cf
