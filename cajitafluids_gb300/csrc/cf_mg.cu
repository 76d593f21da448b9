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

#include <vector>

#include "cf_ctx.cuh"

namespace cf {

constexpr int MG_NU = 2;
constexpr int MG_NC = 16;
constexpr int MG_COARSE_MAX = 2048;  // cells handled by the one-CTA coarse solver

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

// coarsest level in one CTA: x = 0, MG_NC (red, black) and MG_NC (black, red)
// sweeps in shared memory
template <typename T>
__global__ void __launch_bounds__(256) k_mg_coarse(MgLev<T> L, MgBc p, SolverState* S, int inner) {
    if (!block_live(S, inner)) return;
    __shared__ T xs[MG_COARSE_MAX];
    __shared__ T bs[MG_COARSE_MAX];
    const int n = L.nx * L.ny;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        xs[k] = T(0);
        bs[k] = L.b[(size_t)(k / L.nx) * L.pitch + (k % L.nx)];
    }
    __syncthreads();
    auto at = [&](int gi, int gj) -> T {
        if (gi < 0 || gi >= L.nx) {
            if (!p.per_x) return T(0);
            gi = gi < 0 ? gi + L.nx : gi - L.nx;
        }
        if (gj < 0 || gj >= L.ny) {
            if (!p.per_y) return T(0);
            gj = gj < 0 ? gj + L.ny : gj - L.ny;
        }
        return xs[gj * L.nx + gi];
    };
    auto half = [&](int color) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            int gi = k % L.nx, gj = k / L.nx;
            if (((gi + gj) & 1) != color) continue;
            T s = at(gi - 1, gj) + at(gi + 1, gj);
            s = s + at(gi, gj - 1);
            s = s + at(gi, gj + 1);
            T t = mg_fma(L.scale, s, bs[k]);
            xs[k] = t * L.invd[mg_bits(p, L.nx, L.ny, gi, gj)];
        }
        __syncthreads();
    };
    for (int s = 0; s < MG_NC; ++s) {
        half(0);
        half(1);
    }
    for (int s = 0; s < MG_NC; ++s) {
        half(1);
        half(0);
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) L.x[(size_t)(k / L.nx) * L.pitch + (k % L.nx)] = xs[k];
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

struct MgHierarchy {
    int nlev = 0;
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

template <typename T>
static int vcycle(cf_ctx* c, MgLev<T>* lev, int nlev, double scale0, int inner) {
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
    for (int l = 0; l < nlev - 1; ++l) {
        for (int k = 0; k < MG_NU; ++k) {
            smooth(l, 0, k == 0);
            smooth(l, 1, 0);
        }
        k_mg_residual<T><<<grid2(lev[l].nx, lev[l].ny), blk, 0, c->stream>>>(lev[l], p, c->S, inner);
        k_mg_restrict<T><<<grid2(lev[l + 1].nx, lev[l + 1].ny), blk, 0, c->stream>>>(lev[l], lev[l + 1], p, c->S,
                                                                                      inner);
        launches += 2;
    }
    const MgLev<T>& Lc = lev[nlev - 1];
    if (Lc.nx * Lc.ny <= MG_COARSE_MAX) {
        k_mg_coarse<T><<<1, 256, 0, c->stream>>>(Lc, p, c->S, inner);
        ++launches;
    } else {
        for (int k = 0; k < MG_NC; ++k) {
            smooth(nlev - 1, 0, k == 0);
            smooth(nlev - 1, 1, 0);
        }
        for (int k = 0; k < MG_NC; ++k) {
            smooth(nlev - 1, 1, 0);
            smooth(nlev - 1, 0, 0);
        }
    }
    for (int l = nlev - 2; l >= 0; --l) {
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
int mg_vcycle(cf_ctx* c, double scale0) {
    MgHierarchy* H = static_cast<MgHierarchy*>(c->mg);
    if (c->precision == CF_PREC_MIXED) return vcycle<float>(c, H->f, H->nlev, scale0, 1);
    return vcycle<double>(c, H->d, H->nlev, scale0, 0);
}

int mg_levels(const cf_ctx* c) { return c->mg ? static_cast<const MgHierarchy*>(c->mg)->nlev : 0; }

}  // namespace cf
