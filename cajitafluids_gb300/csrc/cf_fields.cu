// Field kernels: on-device ghost fill, fused RK3 semi-Lagrangian advection
// (FP64 and FP32 arithmetic), inflow / body force / wall inputs, and the
// point-sampling test exports.
//
// FP64 arithmetic follows the reference step by step so the FP64 path is
// reproducible: src/TimeIntegrator.hpp:36-116 (rk3, advect),
// src/Interpolation.hpp:30-54 (spline sample), src/Solver.hpp:181-263
// (_addInputs), src/InflowSource.hpp:33-77, src/BodyForce.hpp:44-60,
// src/BoundaryConditions.hpp:102-129.
#include <cuda_runtime.h>
#include <math.h>

#include "cf_adv32.cuh"
#include "cf_ctx.cuh"

namespace cf {

static __constant__ double ENT_OFF_D[3][2] = {{0.5, 0.5}, {0.0, 0.5}, {0.5, 0.0}};

// --------------------------------------------------------------------------
// Ghost fill: the one-GPU form of Cajita's advection halo gather
// (src/ProblemManager.hpp:173-176, 394-398).  Wall ghosts keep their
// construction zeros; periodic ghosts copy the wrapped owned entity.
// One thread per ghost cell: thread t walks the frame around the owned
// block [H, H + nox) x [H, H + noy): the H rows above it, then per owned row
// its left and right ghosts, then the rows below it.
__device__ __forceinline__ int ghost_count(int ex, int ey, int nox, int noy) {
    return CF_HALO * ex + noy * (ex - nox) + (ey - CF_HALO - noy) * ex;
}

template <typename T>
__global__ void k_fill_ghosts(Grid<T> g, int nox, int noy, int per_x, int per_y) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ghost_count(g.ex, g.ey, nox, noy)) return;
    int i, j;
    const int top = CF_HALO * g.ex, midw = g.ex - nox, mid = noy * midw;
    if (t < top) {
        j = t / g.ex;
        i = t - j * g.ex;
    } else if (t < top + mid) {
        t -= top;
        j = CF_HALO + t / midw;
        const int k = t % midw;
        i = k < CF_HALO ? k : nox + k;
    } else {
        t -= top + mid;
        j = CF_HALO + noy + t / g.ex;
        i = t % g.ex;
    }
    int gi = i - CF_HALO, gj = j - CF_HALO;
    bool in_x = gi >= 0 && gi < nox, in_y = gj >= 0 && gj < noy;
    if (in_x && in_y) return;
    if (!in_x) {
        if (!per_x) return;
        gi = ((gi % nox) + nox) % nox;
    }
    if (!in_y) {
        if (!per_y) return;
        gj = ((gj % noy) + noy) % noy;
    }
    g.at(i, j) = g.at(gi + CF_HALO, gj + CF_HALO);
}

// --------------------------------------------------------------------------
// FP64 spline sample (Cajita B-spline order 1 / 3, evaluated separably);
// the coordinate clamp and integer part come from the integer-pipe helpers
// (cf_internal.cuh).
template <int ORDER>
__device__ __forceinline__ void weights64(double xi, int ext, int& k0, double* w) {
    if (ORDER == 1) {
        xi = clamp_bits(xi, 0.0, exact_double(ext - 1));
        int k = trunc_bits(xi);
        if (k > ext - 2) k = ext - 2;
        double t = xi - exact_double(k);
        w[0] = 1.0 - t;
        w[1] = t;
        k0 = k;
    } else {
        xi = clamp_bits(xi, 1.0, exact_double(ext - 2));
        int k = trunc_bits(xi);
        if (k > ext - 3) k = ext - 3;
        double t = xi - exact_double(k);
        double s = 1.0 - t;
        double t2 = t * t;
        double t3 = t2 * t;
        double s3 = (s * s) * s;
        w[0] = s3 * (1.0 / 6.0);
        w[1] = fma(0.5, t3, -t2) + (2.0 / 3.0);
        w[2] = fma(0.5, (t + t2) - t3, 1.0 / 6.0);
        w[3] = t3 * (1.0 / 6.0);
        k0 = k - 1;
    }
}

template <int ORDER>
__device__ double sample64(const Grid<double>& g, double lx, double ly, double rdx, double x, double y) {
    constexpr int n = ORDER == 1 ? 2 : 4;
    double xi = (x - lx) * rdx;
    double yi = (y - ly) * rdx;
    int kx, ky;
    double wx[n], wy[n];
    weights64<ORDER>(xi, g.ex, kx, wx);
    weights64<ORDER>(yi, g.ey, ky, wy);
    double val = 0.0;
#pragma unroll
    for (int b = 0; b < n; ++b) {
        const double* row = g.o + (size_t)(ky + b) * g.pitch + kx;
        double rs = wx[0] * __ldg(row);
#pragma unroll
        for (int a = 1; a < n; ++a) rs = fma(wx[a], __ldg(row + a), rs);
        val = (b == 0) ? wy[0] * rs : fma(wy[b], rs, val);
    }
    return val;
}

__device__ __forceinline__ double entity_coord(const Phys& p, int ent, int axis, int idx) {
    double t = exact_double(idx) + ENT_OFF_D[ent][axis];
    return p.gl[axis] + t * p.dx;
}

// rk3 backtrace (src/TimeIntegrator.hpp:36-77), linear velocity samples.
__device__ void rk3_64(const Phys& p, const Grid<double>& u, const Grid<double>& v, double dt,
                       double x0, double y0, double& tx, double& ty) {
    const double ulx = p.low[E_FACEI][0], uly = p.low[E_FACEI][1];
    const double vlx = p.low[E_FACEJ][0], vly = p.low[E_FACEJ][1];
    double v0x = sample64<1>(u, ulx, uly, p.rdx, x0, y0);
    double v0y = sample64<1>(v, vlx, vly, p.rdx, x0, y0);
    // the reference's stage expressions as written, one rounding per
    // operation: x0 - 0.5 * dt * v0 is x0 - ((0.5 * dt) * v0)
    double h1 = 0.5 * dt;
    double x1 = __dsub_rn(x0, __dmul_rn(h1, v0x)), y1 = __dsub_rn(y0, __dmul_rn(h1, v0y));
    double v1x = sample64<1>(u, ulx, uly, p.rdx, x1, y1);
    double v1y = sample64<1>(v, vlx, vly, p.rdx, x1, y1);
    double h2 = 0.75 * dt;
    bool ralston = (p.quirks & 2u) != 0;
    double sx = ralston ? v1x : v0x, sy = ralston ? v1y : v0y;
    double x2 = __dsub_rn(x0, __dmul_rn(h2, sx)), y2 = __dsub_rn(y0, __dmul_rn(h2, sy));
    double v2x = sample64<1>(u, ulx, uly, p.rdx, x2, y2);
    double v2y = sample64<1>(v, vlx, vly, p.rdx, x2, y2);
    // x0 - dt * ((2/9) v0 + (3/9) v1 + (4/9) v2), summed left to right
    double ax = __dadd_rn(__dmul_rn(2.0 / 9.0, v0x), __dmul_rn(3.0 / 9.0, v1x));
    ax = __dadd_rn(ax, __dmul_rn(4.0 / 9.0, v2x));
    double ay = __dadd_rn(__dmul_rn(2.0 / 9.0, v0y), __dmul_rn(3.0 / 9.0, v1y));
    ay = __dadd_rn(ay, __dmul_rn(4.0 / 9.0, v2y));
    tx = __dsub_rn(x0, __dmul_rn(dt, ax));
    ty = __dsub_rn(y0, __dmul_rn(dt, ay));
}

// --------------------------------------------------------------------------
// Inputs (src/Solver.hpp:181-263) applied to one entity value.
__device__ __forceinline__ bool in_box(const Phys& p, double x, double y) {
    return x >= p.bbox[0] && x < p.bbox[2] && y >= p.bbox[1] && y < p.bbox[3];
}

__device__ __forceinline__ double inputs_cell_in(const Phys& p, double q, bool inbox, double dt) {
    if (inbox) {
        if (p.src_mode == 0) {
            if (q < p.src_q) q = p.src_q;
        } else {
            q = __dadd_rn(q, __dmul_rn(p.src_q, dt));  // rate form (extension)
        }
    }
    return q;
}

__device__ __forceinline__ double inputs_cell(const Phys& p, double q, double x, double y, double dt) {
    if (in_box(p, x, y)) {
        if (p.src_mode == 0) {
            if (q < p.src_q) q = p.src_q;
        } else {
            q = __dadd_rn(q, __dmul_rn(p.src_q, dt));  // rate form (extension)
        }
    }
    return q;
}

// axis 0: I-face (u), axis 1: J-face (v); rho is used only with a density-scaled force.
__device__ __forceinline__ double inputs_face_in(const Phys& p, int axis, double w, bool inbox, double dt, int gidx,
                                                 double rho) {
    if (inbox && fabs(w) < fabs(p.src_vel[axis])) w = p.src_vel[axis];
    // ux += _force[0] * delta_t (src/BodyForce.hpp:52, 61); the density-scaled
    // form (extension) scales the force first
    if (p.force_density)
        w = __dadd_rn(w, __dmul_rn(__dmul_rn(p.force[axis], rho), dt));
    else
        w = __dadd_rn(w, __dmul_rn(p.force[axis], dt));
    int per = axis == 0 ? p.per_x : p.per_y;
    int n = axis == 0 ? p.nx : p.ny;
    if (!per) {
        if (gidx <= 0 && p.bc[axis] == 0) w = 0.0;
        if (gidx > n - 1 && p.bc[axis + 2] == 0) w = 0.0;
    }
    return w;
}

__device__ __forceinline__ double inputs_face(const Phys& p, int axis, double w, double x, double y,
                                              double dt, int gidx, double rho) {
    if (in_box(p, x, y) && fabs(w) < fabs(p.src_vel[axis])) w = p.src_vel[axis];
    // ux += _force[0] * delta_t (src/BodyForce.hpp:52, 61); the density-scaled
    // form (extension) scales the force first
    if (p.force_density)
        w = __dadd_rn(w, __dmul_rn(__dmul_rn(p.force[axis], rho), dt));
    else
        w = __dadd_rn(w, __dmul_rn(p.force[axis], dt));
    int per = axis == 0 ? p.per_x : p.per_y;
    int n = axis == 0 ? p.nx : p.ny;
    if (!per) {
        if (gidx <= 0 && p.bc[axis] == 0) w = 0.0;
        if (gidx > n - 1 && p.bc[axis + 2] == 0) w = 0.0;
    }
    return w;
}

// --------------------------------------------------------------------------
// FP64 advection: one thread per owned entity; blockIdx.z selects the
// entity (cell q, I-face u, J-face v).  Reads Current, writes Next.
struct Adv64 {
    Phys p;
    Grid<double> q, u, v, qn, un, vn;
    double dt;
    int fuse;
    int ent0;  // entity of blockIdx.z == 0 (a launch may cover a subset)
};

template <int ORDER>
__global__ void __launch_bounds__(256) k_advect64(Adv64 a) {
    const Phys& p = a.p;
    int ent = blockIdx.z + a.ent0;
    int gi = blockIdx.x * blockDim.x + threadIdx.x;
    int gj = blockIdx.y * blockDim.y + threadIdx.y;
    int ox = p.nx + ((ent == E_FACEI && !p.per_x) ? 1 : 0);
    int oy = p.ny + ((ent == E_FACEJ && !p.per_y) ? 1 : 0);
    if (gi >= ox || gj >= oy) return;
    const Grid<double>& f = ent == E_CELL ? a.q : (ent == E_FACEI ? a.u : a.v);
    const Grid<double>& fn = ent == E_CELL ? a.qn : (ent == E_FACEI ? a.un : a.vn);
    double x0 = entity_coord(p, ent, 0, gi + CF_HALO);
    double y0 = entity_coord(p, ent, 1, gj + CF_HALO);
    double tx, ty;
    rk3_64(p, a.u, a.v, a.dt, x0, y0, tx, ty);
    double val = sample64<ORDER>(f, p.low[ent][0], p.low[ent][1], p.rdx, tx, ty);
    if (a.fuse) {
        const bool inbox = in_box_idx(p, ent, gi + CF_HALO, gj + CF_HALO);
        if (ent == E_CELL)
            val = inputs_cell_in(p, val, inbox, a.dt);
        else if (ent == E_FACEI)
            val = inputs_face_in(p, 0, val, inbox, a.dt, gi, 0.0);
        else
            val = inputs_face_in(p, 1, val, inbox, a.dt, gj, 0.0);
    }
    fn.at(gi + CF_HALO, gj + CF_HALO) = val;
}

// --------------------------------------------------------------------------
// FP32 advection (mixed precision).  Positions are kept as an integer base
// (the entity's local index) plus a small FP32 displacement in cell units,
// so FP32 keeps full relative precision at any grid size.  A mixed context
// stores u and v as double-float pairs (each 8-byte element holds hi =
// fl32(w), lo = fl32(w - hi) of the face velocity w, about 48 significant
// bits): the projection works on the pairs on the FP32 pipe, and the
// advection samples the hi parts; q is FP32.
// The inputs epilogue tests the inflow box on integer index ranges that the
// host evaluated with the FP64 coordinate test; a body force is added to the
// advected value as a pair (fdt2 = the pair of force * dt), and only a face
// inside the box takes FP64 arithmetic.
struct Adv32 {
    Phys p;
    Grid<float> q, qn;
    Grid<double> u, v;    // current velocities, double-float pairs
    Grid<double> un, vn;  // next velocities, written as pairs
    float c;      // dt / dx
    double dt;
    int fuse;
    int ent0;     // entity of blockIdx.x == 0 (a launch may cover a subset)
    int unstaged; // tests: every tile reads global memory (same bits)
    float2 fdt2[2];  // force[axis] * dt as pairs (zero without a force)
    int force_on[2]; // force[axis] != 0 (tested on the host: an FP64 compare per face
                     // would occupy GB300's FP64 pipe)
};


// The RK3 trace of one entity at ghosted (li, lj) and the value sampled at
// its foot, U and V the velocity taps, F the advected field's.
template <int ORDER, typename A>
__device__ __forceinline__ float advect_value(const Adv32& a, int ent, int li, int lj, const A& U, const A& V,
                                              const A& F) {
    // entity offset minus the velocity grids' offsets (u: (0, .5), v: (.5, 0))
    const float ox_e = ent == E_FACEI ? 0.f : 0.5f;
    const float oy_e = ent == E_FACEJ ? 0.f : 0.5f;
    const float uox = ox_e, uoy = oy_e - 0.5f, vox = ox_e - 0.5f, voy = oy_e;
    // first RK stage at the entity itself
    float v0x, v0y;
    stage0_32(ent, U, V, li, lj, v0x, v0y);
    const float h1 = -0.5f * a.c, h2 = -0.75f * a.c;
    const float d1x = h1 * v0x, d1y = h1 * v0y;
    const float v1x = lin32(U, li, lj, uox + d1x, uoy + d1y);
    const float v1y = lin32(V, li, lj, vox + d1x, voy + d1y);
    const bool ralston = (a.p.quirks & 2u) != 0;
    const float d2x = h2 * (ralston ? v1x : v0x), d2y = h2 * (ralston ? v1y : v0y);
    const float v2x = lin32(U, li, lj, uox + d2x, uoy + d2y);
    const float v2y = lin32(V, li, lj, vox + d2x, voy + d2y);
    const float ax = fmaf(4.f / 9.f, v2x, fmaf(3.f / 9.f, v1x, (2.f / 9.f) * v0x));
    const float ay = fmaf(4.f / 9.f, v2y, fmaf(3.f / 9.f, v1y, (2.f / 9.f) * v0y));
    const float dx = -a.c * ax, dy = -a.c * ay;
    return ORDER == 1 ? lin32(F, li, lj, dx, dy) : cub32(F, li, lj, dx, dy);
}

// max that keeps a NaN (so a NaN in a window sends its tile to the clamped path)
__device__ __forceinline__ float max_nan(float x, float y) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
    return r;
}

// One CTA per 32 x 32 tile and entity kind (blockIdx.x, fastest, so that the
// kinds of one tile run together and share its windows through L2; tiles
// along blockIdx.y, blockIdx.z).  The CTA copies the windows of u, v and
// (cells) q into shared memory, 16-byte rows, and takes the largest |u|, |v|
// in them, M.  Every RK velocity is a convex combination of window values,
// so while (dt / dx) M <= 0.99 no position moves a full cell and the traces
// read only the window; otherwise (or with a NaN, or when a test asks for
// it) the tile reads global memory with the clamped stencil.  Either way
// each entity gets the same bits.
template <int ORDER>
__global__ void __launch_bounds__(256, 8) k_advect32(Adv32 a) {
    __shared__ __align__(16) float sw[3 * AW_N];  // u, v, q windows
    __shared__ float red[8];
    const Phys& p = a.p;
    const int ent = blockIdx.x + a.ent0;
    const int gi0 = blockIdx.y * AT_X, gj0 = blockIdx.z * AT_Y;
    const int lane = threadIdx.x & 31, wrow = threadIdx.x >> 5;
    // The window's origin is ghosted (gi0 - 1, gj0 + 1); rows past an array
    // and chunks past its padded row read as zeros.  u, v: 16-byte chunks of
    // two pairs, their hi parts kept (chunk c2 ends at element CF_COL0 + gi0
    // - 1 + 2 c2 + 2 of the row); q: chunks of four floats (ending at element
    // CF_COL0 + gi0 - 1 + 4 c4 + 4).
    float m = 0.f;
    for (int arr = 0; arr < 2; ++arr) {
        const double* go = arr == 0 ? a.u.o : a.v.o;
        const int gp = arr == 0 ? a.u.pitch : a.v.pitch, gey = arr == 0 ? a.u.ey : a.v.ey;
        constexpr int kRowChunks = AW_X / 2, kChunks = AW_Y * kRowChunks;
        const float* src = reinterpret_cast<const float*>(go + (size_t)(gj0 + 1) * gp + (gi0 - 1));
        const int nrow = gey - (gj0 + 1), nc2 = (gp - CF_COL0 - gi0 + 1) >> 1;
        float* dst = sw + arr * AW_N;
        for (int k = threadIdx.x; k < kChunks; k += 256) {
            const int r = k / kRowChunks, c2 = k - r * kRowChunks;
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < nrow && c2 < nc2)
                w = __ldg(reinterpret_cast<const float4*>(src + 2 * ((size_t)r * gp + 2 * c2)));
            *reinterpret_cast<float2*>(dst + 2 * k) = make_float2(w.x, w.z);  // r AW_X + 2 c2 = 2 k
            m = max_nan(m, max_nan(fabsf(w.x), fabsf(w.z)));
        }
    }
    if (ent == E_CELL) {
        constexpr int kRowChunks = AW_X / 4, kChunks = AW_Y * kRowChunks;
        const float* src = a.q.o + (size_t)(gj0 + 1) * a.q.pitch + (gi0 - 1);
        const int nrow = a.q.ey - (gj0 + 1), nc4 = (a.q.pitch - CF_COL0 - gi0 + 1) >> 2;
        float* dst = sw + 2 * AW_N;
        for (int k = threadIdx.x; k < kChunks; k += 256) {
            const int r = k / kRowChunks, c4 = k - r * kRowChunks;
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < nrow && c4 < nc4) w = __ldg(reinterpret_cast<const float4*>(src + (size_t)r * a.q.pitch + 4 * c4));
            *reinterpret_cast<float4*>(dst + 4 * k) = w;  // r AW_X + 4 c4 = 4 k
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max_nan(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) red[wrow] = m;
    __syncthreads();
    float big = red[0];
#pragma unroll
    for (int w = 1; w < 8; ++w) big = max_nan(big, red[w]);
    const bool staged = !a.unstaged && a.c * big <= 0.99f;

    const int ox = p.nx + ((ent == E_FACEI && !p.per_x) ? 1 : 0);
    const int oy = p.ny + ((ent == E_FACEJ && !p.per_y) ? 1 : 0);
    const int fa = ent == E_CELL ? 2 : (ent == E_FACEI ? 0 : 1);
    const GlobalTaps gu{reinterpret_cast<const float*>(a.u.o), a.u.pitch, a.u.ex, a.u.ey, 2},
        gv{reinterpret_cast<const float*>(a.v.o), a.v.pitch, a.v.ex, a.v.ey, 2};
    const GlobalTaps gf =
        ent == E_CELL ? GlobalTaps{a.q.o, a.q.pitch, a.q.ex, a.q.ey, 1} : (ent == E_FACEI ? gu : gv);
#pragma unroll 1
    for (int k = 0; k < AT_Y / 8; ++k) {
        const int gi = gi0 + lane, gj = gj0 + wrow + 8 * k;
        if (gi >= ox || gj >= oy) continue;
        const int li = gi + CF_HALO, lj = gj + CF_HALO;
        float val;
        if (staged) {
            const WindowTaps U{sw, gi0 - 1, gj0 + 1}, V{sw + AW_N, gi0 - 1, gj0 + 1},
                F{sw + fa * AW_N, gi0 - 1, gj0 + 1};
            val = advect_value<ORDER>(a, ent, li, lj, U, V, F);
        } else {
            val = advect_value<ORDER>(a, ent, li, lj, gu, gv, gf);
        }
        if (ent == E_CELL) {
            // cell inputs (src/Solver.hpp:181-263): the clamp max(q, Q) rounds to
            // the same FP32 value when taken in FP32; the rate form in FP64
            if (a.fuse && in_box_idx(p, E_CELL, li, lj)) {
                if (p.src_mode == 0) {
                    const float qf = (float)p.src_q;
                    if (val < qf) val = qf;
                } else {
                    val = (float)__dadd_rn((double)val, __dmul_rn(p.src_q, a.dt));
                }
            }
            a.qn.at(li, lj) = val;
            continue;
        }
        // face inputs (src/Solver.hpp:181-263) on the pair (val, 0): the inflow
        // velocity where it is larger, then the body force, then the walls
        const int axis = ent == E_FACEI ? 0 : 1;
        float2 w = make_float2(val, 0.f);
        if (a.fuse) {
            if (in_box_idx(p, ent, li, lj) && fabs((double)val) < fabs(p.src_vel[axis])) w = df_split(p.src_vel[axis]);
            if (a.force_on[axis]) w = df_add(w, a.fdt2[axis]);
            const int per = axis == 0 ? p.per_x : p.per_y, n = axis == 0 ? p.nx : p.ny, gg = axis == 0 ? gi : gj;
            if (!per) {
                if (gg <= 0 && p.bc[axis] == 0) w = make_float2(0.f, 0.f);
                if (gg > n - 1 && p.bc[axis + 2] == 0) w = make_float2(0.f, 0.f);
            }
        }
        double& dst = axis == 0 ? a.un.at(li, lj) : a.vn.at(li, lj);
        reinterpret_cast<float2&>(dst) = w;
    }
}

// --------------------------------------------------------------------------
// Standalone inputs (Solver::setup and density-scaled body forces): pass 0
// updates cells, pass 1 updates faces reading the updated cells.  A mixed
// context (TQ = float) keeps u, v as double-float pairs: a face value is
// taken to FP64, the inputs applied in FP64 and the result split again.
template <typename TQ>
struct Inp {
    Phys p;
    Grid<TQ> q;
    Grid<double> u, v;
    double dt;
};

template <typename TQ>
__device__ __forceinline__ double cell_q(const Inp<TQ>& a, int gi, int gj) {
    int ci = wrap_index(gi, a.p.nx, a.p.per_x), cj = wrap_index(gj, a.p.ny, a.p.per_y);
    if (ci < 0 || cj < 0) return 0.0;
    return (double)a.q.at(ci + CF_HALO, cj + CF_HALO);
}

template <typename TQ>
__global__ void k_inputs_cells(Inp<TQ> a) {
    int gi = blockIdx.x * blockDim.x + threadIdx.x;
    int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= a.p.nx || gj >= a.p.ny) return;
    double x = entity_coord(a.p, E_CELL, 0, gi + CF_HALO), y = entity_coord(a.p, E_CELL, 1, gj + CF_HALO);
    TQ& q = a.q.at(gi + CF_HALO, gj + CF_HALO);
    q = (TQ)inputs_cell(a.p, (double)q, x, y, a.dt);
}

template <typename TQ>
__global__ void k_inputs_faces(Inp<TQ> a) {
    const Phys& p = a.p;
    int axis = blockIdx.z;
    int gi = blockIdx.x * blockDim.x + threadIdx.x;
    int gj = blockIdx.y * blockDim.y + threadIdx.y;
    int ox = p.nx + ((axis == 0 && !p.per_x) ? 1 : 0);
    int oy = p.ny + ((axis == 1 && !p.per_y) ? 1 : 0);
    if (gi >= ox || gj >= oy) return;
    int ent = axis == 0 ? E_FACEI : E_FACEJ;
    double x = entity_coord(p, ent, 0, gi + CF_HALO), y = entity_coord(p, ent, 1, gj + CF_HALO);
    double rho = 0.0;
    if (p.force_density)
        rho = axis == 0 ? (cell_q(a, gi - 1, gj) + cell_q(a, gi, gj)) * 0.5
                        : (cell_q(a, gi, gj - 1) + cell_q(a, gi, gj)) * 0.5;
    double& w = axis == 0 ? a.u.at(gi + CF_HALO, gj + CF_HALO) : a.v.at(gi + CF_HALO, gj + CF_HALO);
    if constexpr (sizeof(TQ) == sizeof(float)) {
        float2& wp = reinterpret_cast<float2&>(w);
        wp = df_split(inputs_face(p, axis, df_value(wp), x, y, a.dt, axis == 0 ? gi : gj, rho));
    } else {
        w = inputs_face(p, axis, w, x, y, a.dt, axis == 0 ? gi : gj, rho);
    }
}

// --------------------------------------------------------------------------
// Test exports and small utilities.
struct Pts {
    Phys p;
    Grid<double> f, u, v;
    int ent, order, n;
    const double* xy;
    double* out;
    double dt;
};

__global__ void k_interp_points(Pts a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    double x = a.xy[2 * k], y = a.xy[2 * k + 1];
    a.out[k] = a.order == 1 ? sample64<1>(a.f, a.p.low[a.ent][0], a.p.low[a.ent][1], a.p.rdx, x, y)
                            : sample64<3>(a.f, a.p.low[a.ent][0], a.p.low[a.ent][1], a.p.rdx, x, y);
}

__global__ void k_trace_points(Pts a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    double tx, ty;
    rk3_64(a.p, a.u, a.v, a.dt, a.xy[2 * k], a.xy[2 * k + 1], tx, ty);
    a.out[2 * k] = tx;
    a.out[2 * k + 1] = ty;
}

// SiloWriter::writeFile's cell-centred velocity (src/SiloWriter.hpp:177-191):
// interpolateVelocity<2, 1> (linear) of u and v at each owned cell centre,
// written owned-region, x fastest, into uc, vc (pitch nx)
__global__ void k_cell_velocity(Phys p, Grid<double> u, Grid<double> v, double* uc, double* vc) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    const int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= p.nx || gj >= p.ny) return;
    const double x = entity_coord(p, E_CELL, 0, gi + CF_HALO), y = entity_coord(p, E_CELL, 1, gj + CF_HALO);
    const size_t k = (size_t)gj * p.nx + gi;
    uc[k] = sample64<1>(u, p.low[E_FACEI][0], p.low[E_FACEI][1], p.rdx, x, y);
    vc[k] = sample64<1>(v, p.low[E_FACEJ][0], p.low[E_FACEJ][1], p.rdx, x, y);
}

// max |w| over the owned faces of one axis; non-negative doubles order like
// their bit patterns, so an integer atomicMax is exact and order-free.
__global__ void k_max_abs(Grid<double> g, int ox, int oy, unsigned long long* out) {
    int gi = blockIdx.x * blockDim.x + threadIdx.x;
    int gj = blockIdx.y * blockDim.y + threadIdx.y;
    double m = 0.0;
    if (gi < ox && gj < oy) m = fabs(g.at(gi + CF_HALO, gj + CF_HALO));
    if (m != m) m = INFINITY;
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// FP64 staging <-> FP32 quantity (owned region, staging row pitch = ox)
__global__ void k_q_convert(Grid<float> q, double* st, int nx, int ny, int to_device) {
    int gi = blockIdx.x * blockDim.x + threadIdx.x;
    int gj = blockIdx.y * blockDim.y + threadIdx.y;
    if (gi >= nx || gj >= ny) return;
    size_t k = (size_t)gj * nx + gi;
    if (to_device)
        q.at(gi + CF_HALO, gj + CF_HALO) = (float)st[k];
    else
        st[k] = (double)q.at(gi + CF_HALO, gj + CF_HALO);
}

// --------------------------------------------------------------------------
// launchers
static inline dim3 grid2(int ex, int ey, dim3 blk, int z = 1) {
    return dim3((ex + blk.x - 1) / blk.x, (ey + blk.y - 1) / blk.y, z);
}

cudaError_t launch_fill_ghosts(cf_ctx* c, int what, cudaStream_t stream) {
    const Phys& p = c->ph;
    if (!p.per_x && !p.per_y) return cudaSuccess;  // wall ghosts are never written
    if (!stream) stream = c->stream;
    int s = c->cur;
    int nqx = p.nx, nqy = p.ny;
    int nux = p.per_x ? p.nx : p.nx + 1, nvy = p.per_y ? p.ny : p.ny + 1;
    auto frame = [&](int ex, int ey, int nox, int noy) {
        const int n = CF_HALO * ex + noy * (ex - nox) + (ey - CF_HALO - noy) * ex;
        return (n + 255) / 256;
    };
    if (what & GHOSTS_Q) {
        if (c->precision == CF_PREC_FP64) {
            const Grid<double>& g = c->q64[s];
            k_fill_ghosts<double><<<frame(g.ex, g.ey, nqx, nqy), 256, 0, stream>>>(g, nqx, nqy, p.per_x, p.per_y);
        } else {
            const Grid<float>& g = c->q32[s];
            k_fill_ghosts<float><<<frame(g.ex, g.ey, nqx, nqy), 256, 0, stream>>>(g, nqx, nqy, p.per_x, p.per_y);
        }
        c->launches += 1;
    }
    if (what & GHOSTS_UV) {
        k_fill_ghosts<double><<<frame(c->u[s].ex, c->u[s].ey, nux, p.ny), 256, 0, stream>>>(c->u[s], nux, p.ny,
                                                                                         p.per_x, p.per_y);
        k_fill_ghosts<double><<<frame(c->v[s].ex, c->v[s].ey, p.nx, nvy), 256, 0, stream>>>(c->v[s], p.nx, nvy,
                                                                                         p.per_x, p.per_y);
        c->launches += 2;
    }
    return cudaGetLastError();
}

cudaError_t launch_advect(cf_ctx* c, double dt, int order, int fuse_inputs, int ent0, int nent, bool prep,
                          bool advance) {
    const Phys& p = c->ph;
    int s = c->cur, n = 1 - s;
    dim3 blk(32, 8);
    dim3 grd = grid2(p.nx + 1, p.ny + 1, blk, nent);
    if (c->precision == CF_PREC_FP64) {
        Adv64 a{p, c->q64[s], c->u[s], c->v[s], c->q64[n], c->u[n], c->v[n], dt, fuse_inputs, ent0};
        if (order == 1)
            k_advect64<1><<<grd, blk, 0, c->stream>>>(a);
        else
            k_advect64<3><<<grd, blk, 0, c->stream>>>(a);
    } else {
        // fused inputs with a density-scaled force are applied by the
        // standalone inputs kernels after the advection
        Adv32 a{p,   c->q32[s], c->q32[n], c->u[s], c->v[s], c->u[n], c->v[n], (float)(dt / p.dx), dt, fuse_inputs,
                ent0, c->test_unstaged, {}};
        for (int k = 0; k < 2; ++k) {
            const double f = p.force[k] * dt;
            const float hi = (float)f;
            a.fdt2[k] = make_float2(hi, (float)(f - (double)hi));
            a.force_on[k] = p.force[k] != 0.0 ? 1 : 0;
        }
        (void)prep;
        const dim3 tiles(nent, (p.nx + 1 + AT_X - 1) / AT_X, (p.ny + 1 + AT_Y - 1) / AT_Y);
        if (order == 1)
            k_advect32<1><<<tiles, 256, 0, c->stream>>>(a);
        else
            k_advect32<3><<<tiles, 256, 0, c->stream>>>(a);
    }
    c->launches += 1;
    if (advance) {
        c->cur = n;  // ProblemManager::advance for q, u, v
    }
    return cudaGetLastError();
}

cudaError_t launch_add_inputs(cf_ctx* c, double dt) {
    const Phys& p = c->ph;
    int s = c->cur;
    dim3 blk(32, 8);
    if (c->precision == CF_PREC_FP64) {
        Inp<double> a{p, c->q64[s], c->u[s], c->v[s], dt};
        k_inputs_cells<double><<<grid2(p.nx, p.ny, blk), blk, 0, c->stream>>>(a);
        k_inputs_faces<double><<<grid2(p.nx + 1, p.ny + 1, blk, 2), blk, 0, c->stream>>>(a);
    } else {
        Inp<float> a{p, c->q32[s], c->u[s], c->v[s], dt};
        k_inputs_cells<float><<<grid2(p.nx, p.ny, blk), blk, 0, c->stream>>>(a);
        k_inputs_faces<float><<<grid2(p.nx + 1, p.ny + 1, blk, 2), blk, 0, c->stream>>>(a);
    }
    c->launches += 2;
    return cudaGetLastError();
}

// Mixed storage of u, v: double-float pairs.  k_to_pairs turns the FP64
// values of the owned region in place into pairs; k_from_pairs writes the
// FP64 values of a region [i0, i0 + nx) x [j0, j0 + ny) of the ghosted array
// to dst (row pitch dp elements).
__global__ void k_to_pairs(Grid<double> g, int nx, int ny) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nx || j >= ny) return;
    double& e = g.at(i + CF_HALO, j + CF_HALO);
    reinterpret_cast<float2&>(e) = df_split(e);
}

__global__ void k_from_pairs(Grid<double> g, int i0, int j0, int nx, int ny, double* dst, int dp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nx || j >= ny) return;
    dst[(size_t)j * dp + i] = df_value(reinterpret_cast<const float2&>(g.at(i0 + i, j0 + j)));
}

static Grid<double> vel_grid(cf_ctx* c, int field, int version) {
    return field == CF_FIELD_U ? c->u[version] : c->v[version];
}

cudaError_t launch_to_pairs(cf_ctx* c, int field, int version, cudaStream_t stream) {
    const Phys& p = c->ph;
    const int ox = p.nx + ((field == CF_FIELD_U && !p.per_x) ? 1 : 0);
    const int oy = p.ny + ((field == CF_FIELD_V && !p.per_y) ? 1 : 0);
    dim3 blk(32, 8);
    k_to_pairs<<<grid2(ox, oy, blk), blk, 0, stream ? stream : c->stream>>>(vel_grid(c, field, version), ox, oy);
    c->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_from_pairs(cf_ctx* c, int field, int version, double* dst, cudaStream_t stream) {
    const Phys& p = c->ph;
    const int ox = p.nx + ((field == CF_FIELD_U && !p.per_x) ? 1 : 0);
    const int oy = p.ny + ((field == CF_FIELD_V && !p.per_y) ? 1 : 0);
    dim3 blk(32, 8);
    k_from_pairs<<<grid2(ox, oy, blk), blk, 0, stream ? stream : c->stream>>>(vel_grid(c, field, version), CF_HALO,
                                                                            CF_HALO, ox, oy, dst, ox);
    c->launches += 1;
    return cudaGetLastError();
}

// The current u, v as FP64 ghosted arrays: the state itself (FP64 context),
// or (mixed) FP64 copies of the pairs in arrays made on first use.
int velocity_f64(cf_ctx* c, Grid<double>* gu, Grid<double>* gv) {
    const int s = c->cur;
    if (c->precision != CF_PREC_MIXED) {
        *gu = c->u[s];
        *gv = c->v[s];
        return CF_OK;
    }
    for (int f = 0; f < 2; ++f) {
        const Grid<double>& g = f == 0 ? c->u[s] : c->v[s];
        if (!c->vel64[f].o) {
            const int rc = alloc_grid64(c, c->vel64[f], g.ex, g.ey);
            if (rc) return rc;
        }
        Grid<double>& d = c->vel64[f];
        dim3 blk(32, 8);
        k_from_pairs<<<grid2(g.ex, g.ey, blk), blk, 0, c->stream>>>(g, 0, 0, g.ex, g.ey, &d.at(0, 0), d.pitch);
        c->launches += 1;
    }
    *gu = c->vel64[0];
    *gv = c->vel64[1];
    return cuda_check(c, cudaGetLastError(), "velocity conversion");
}

cudaError_t launch_interp_points(cf_ctx* c, int field, int order, int n, const double* d_xy, double* d_out) {
    int s = c->cur;
    Grid<double> gu, gv;
    if (velocity_f64(c, &gu, &gv)) return cudaErrorMemoryAllocation;
    Grid<double> f = field == CF_FIELD_QUANTITY ? c->q64[s] : (field == CF_FIELD_U ? gu : gv);
    Pts a{c->ph, f, gu, gv, field, order, n, d_xy, d_out, 0.0};
    k_interp_points<<<(n + 127) / 128, 128, 0, c->stream>>>(a);
    c->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_cell_velocity(cf_ctx* c, double* d_uc, double* d_vc) {
    const Phys& p = c->ph;
    dim3 blk(32, 8);
    Grid<double> gu, gv;
    if (velocity_f64(c, &gu, &gv)) return cudaErrorMemoryAllocation;
    k_cell_velocity<<<grid2(p.nx, p.ny, blk), blk, 0, c->stream>>>(p, gu, gv, d_uc, d_vc);
    c->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_trace_points(cf_ctx* c, int n, const double* d_xy, double dt, double* d_out) {
    Grid<double> gu, gv;
    if (velocity_f64(c, &gu, &gv)) return cudaErrorMemoryAllocation;
    Pts a{c->ph, gu, gu, gv, 0, 1, n, d_xy, d_out, dt};
    k_trace_points<<<(n + 127) / 128, 128, 0, c->stream>>>(a);
    c->launches += 1;
    return cudaGetLastError();
}

// test export: the integer-pipe conversions applied to n values
__global__ void k_test_convert(int n, const double* d, float* f, double* w) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float v = d2f_rn(d[k]);
    f[k] = v;
    w[k] = f2d_exact(v);
}

cudaError_t launch_test_convert(cf_ctx* c, int n, const double* d, float* f, double* w) {
    if (n <= 0) return cudaSuccess;
    k_test_convert<<<(n + 255) / 256, 256, 0, c->stream>>>(n, d, f, w);
    c->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_max_velocity(cf_ctx* c, double* d_out) {
    const Phys& p = c->ph;
    Grid<double> gu, gv;
    if (velocity_f64(c, &gu, &gv)) return cudaErrorMemoryAllocation;
    cudaMemsetAsync(d_out, 0, sizeof(double), c->stream);
    dim3 blk(32, 8);
    int nux = p.per_x ? p.nx : p.nx + 1, nvy = p.per_y ? p.ny : p.ny + 1;
    k_max_abs<<<grid2(nux, p.ny, blk), blk, 0, c->stream>>>(gu, nux, p.ny, (unsigned long long*)d_out);
    k_max_abs<<<grid2(p.nx, nvy, blk), blk, 0, c->stream>>>(gv, p.nx, nvy, (unsigned long long*)d_out);
    c->launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_q_to_f64(cf_ctx* c, int version, double* dst, cudaStream_t stream) {
    dim3 blk(32, 8);
    k_q_convert<<<grid2(c->ph.nx, c->ph.ny, blk), blk, 0, stream>>>(c->q32[version], dst, c->ph.nx, c->ph.ny, 0);
    c->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_convert_q(cf_ctx* c, int to_device, int version, cudaStream_t stream) {
    dim3 blk(32, 8);
    if (!stream) stream = c->stream;
    k_q_convert<<<grid2(c->ph.nx, c->ph.ny, blk), blk, 0, stream>>>(c->q32[version], c->staging, c->ph.nx, c->ph.ny,
                                                                    to_device);
    c->launches += 1;
    return cudaGetLastError();
}

}  // namespace cf
