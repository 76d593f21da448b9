// FP32 samplers of the mixed-precision advection and of its transpose
// (cf_fields.cu, cf_adjoint.cu): tap access to ghosted arrays or staged
// windows, linear and cubic B-spline samples, the first RK stage.  Both
// directions use these functions, so the reverse sweep recomputes the
// forward trace bit for bit.  Arithmetic: src/Interpolation.hpp:30-54 (the
// spline weights), src/TimeIntegrator.hpp:36-77 (the RK3 trace).
#pragma once
#include "cf_internal.cuh"

namespace cf {

// Tap access for the FP32 samplers.  GlobalTaps reads a ghosted FP32 array
// and clamps the stencil to it, as the FP64 samplers do; WindowTaps reads a
// CTA's staged copy of part of the array in shared memory and does not
// clamp.  The advection uses a window only where no position of a trace
// moves a full cell from its entity; the taps then lie within two cells of
// the entity, inside the window and at least one cell inside the ghosted
// array, where the clamps cannot fire, so both give the same bits.
// A pair array is read as floats two apart (es = 2, the hi parts).
struct GlobalTaps {
    const float* o;
    int pitch, ex, ey;
    int es;  // floats per element: 1 (FP32 array), 2 (pair array)
    static constexpr bool kClamp = true;
    __device__ __forceinline__ const float* at(int ix, int iy) const {
        return o + ((size_t)iy * pitch + ix) * es;
    }
    __device__ __forceinline__ int stride() const { return pitch * es; }
    __device__ __forceinline__ int step() const { return es; }
    __device__ __forceinline__ static float ld(const float* p) { return __ldg(p); }
};

// Advection tiles: 32 x 32 entities per CTA of 256 threads (lane = column,
// four rows per thread).  An entity of the tile at ghosted (li, lj) has
// li in [gi0 + 3, gi0 + 35), lj in [gj0 + 3, gj0 + 35); with every RK
// position less than a cell from it, its taps lie in [li - 2, li + 2] x
// [lj - 2, lj + 2].  The window, ghosted columns [gi0 - 1, gi0 + 39) and rows
// [gj0 + 1, gj0 + 38), holds that with a cell to spare; its first column
// sits on a 16-byte boundary (ghosted column 3 of every row is on a
// 128-byte one), so rows are copied as float4.
constexpr int AT_X = 32;
constexpr int AT_Y = 32;
constexpr int AW_X = 40;
constexpr int AW_Y = AT_Y + 5;
constexpr int AW_N = AW_X * AW_Y;

struct WindowTaps {
    const float* s;  // ghosted (x0, y0)
    int x0, y0;
    int ex = 0, ey = 0;  // unused: a window does not clamp
    static constexpr bool kClamp = false;
    __device__ __forceinline__ const float* at(int ix, int iy) const { return s + ((iy - y0) * AW_X + (ix - x0)); }
    __device__ __forceinline__ int stride() const { return AW_X; }
    __device__ __forceinline__ static constexpr int step() { return 1; }
    __device__ __forceinline__ static float ld(const float* p) { return *p; }
};

template <typename A>
__device__ __forceinline__ float lin32(const A& g, int bi, int bj, float fx, float fy) {
    float flx = floorf(fx), fly = floorf(fy);
    int ix = bi + (int)flx, iy = bj + (int)fly;
    float tx = fx - flx, ty = fy - fly;
    if constexpr (A::kClamp) {
        if (ix < 0) { ix = 0; tx = 0.f; }
        if (ix > g.ex - 2) { ix = g.ex - 2; tx = 1.f; }
        if (iy < 0) { iy = 0; ty = 0.f; }
        if (iy > g.ey - 2) { iy = g.ey - 2; ty = 1.f; }
    }
    const float* r0 = g.at(ix, iy);
    const float* r1 = r0 + g.stride();
    const int e = g.step();
    const float2 lo = make_float2(A::ld(r0), A::ld(r1));           // (a0, b0)
    const float2 hi = make_float2(A::ld(r0 + e), A::ld(r1 + e));   // (a1, b1)
    // (s0, s1) = (fma(tx, a1 - a0, a0), fma(tx, b1 - b0, b0)), paired
    const float2 sp = f2_fma(make_float2(tx, tx), f2_sub(hi, lo), lo);
    return fmaf(ty, sp.y - sp.x, sp.x);
}

__device__ __forceinline__ void cubic_w32(float t, float* w) {
    float s = 1.f - t, t2 = t * t, t3 = t2 * t;
    w[0] = s * s * s * (1.f / 6.f);
    w[1] = fmaf(0.5f, t3, -t2) + (2.f / 3.f);
    w[2] = fmaf(0.5f, (t + t2) - t3, 1.f / 6.f);
    w[3] = t3 * (1.f / 6.f);
}

template <typename A>
__device__ __forceinline__ float cub32(const A& g, int bi, int bj, float fx, float fy) {
    float flx = floorf(fx), fly = floorf(fy);
    int ix = bi + (int)flx, iy = bj + (int)fly;
    float tx = fx - flx, ty = fy - fly;
    if constexpr (A::kClamp) {
        if (ix < 1) { ix = 1; tx = 0.f; }
        if (ix > g.ex - 3) { ix = g.ex - 3; tx = 1.f; }
        if (iy < 1) { iy = 1; ty = 0.f; }
        if (iy > g.ey - 3) { iy = g.ey - 3; ty = 1.f; }
    }
    float wx[4], wy[4];
    cubic_w32(tx, wx);
    cubic_w32(ty, wy);
    // Difference form: c + sum w (f - c) with c = the tap at (ix, iy).  The
    // FP32 weights do not sum to exactly 1 (2/3 and 1/6 both round up, so
    // the sum is about 1 + 2.5e-8 per axis); summing w * f directly would
    // scale the field by that much every step, a drift that grows linearly
    // over a run.  Against differences the weight error only touches the
    // local variation of the field, and a constant is reproduced exactly.
    const float* base = g.at(ix - 1, iy - 1);
    const int st = g.stride(), e = g.step();
    const float c = A::ld(base + st + e);
    // rows 0, 1 and rows 2, 3 as packed pairs: rs_b = wx0 (f_b0 - c), then
    // fma(wx_k, f_bk - c, rs_b) for k = 1 .. 3, each lane as the scalar form
    const float2 cc = make_float2(c, c);
    float2 rs01, rs23;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 wk = make_float2(wx[k], wx[k]);
        const float2 d01 = f2_sub(make_float2(A::ld(base + k * e), A::ld(base + st + k * e)), cc);
        const float2 d23 = f2_sub(make_float2(A::ld(base + 2 * st + k * e), A::ld(base + 3 * st + k * e)), cc);
        rs01 = k == 0 ? f2_mul(wk, d01) : f2_fma(wk, d01, rs01);
        rs23 = k == 0 ? f2_mul(wk, d23) : f2_fma(wk, d23, rs23);
    }
    float val = wy[0] * rs01.x;
    val = fmaf(wy[1], rs01.y, val);
    val = fmaf(wy[2], rs23.x, val);
    val = fmaf(wy[3], rs23.y, val);
    return c + val;
}

// First RK stage of the FP32 trace: the velocity at the entity itself.  The
// linear samples' integer cells and fractions (0 or 1/2) are known, so the
// taps are read directly (a zero-weight row is dropped: it only could turn a
// -0 into +0, which no later step can tell apart).  Taps by entity, as
// offsets from the entity's ghosted (li, lj), each weighted as listed:
//   cell:   u (0,0), (1,0) 1/2 each;       v (0,0), (0,1) 1/2 each
//   face i: u (0,0) 1;                      v (-1,0), (0,0), (-1,1), (0,1) 1/4 each
//   face j: u (0,-1), (1,-1), (0,0), (1,0) 1/4 each;   v (0,0) 1
// (the reverse sweep spreads the stage's adjoint with these weights).
template <typename A>
__device__ __forceinline__ void stage0_32(int ent, const A& U, const A& V, int li, int lj, float& v0x, float& v0y) {
    const float* u0 = U.at(li, lj);
    const float* w0 = V.at(li, lj);
    const int pu = U.stride(), pv = V.stride(), eu = U.step(), ev = V.step();
    if (ent == E_CELL) {
        v0x = fmaf(0.5f, A::ld(u0 + eu) - A::ld(u0), A::ld(u0));
        v0y = fmaf(0.5f, A::ld(w0 + pv) - A::ld(w0), A::ld(w0));
    } else if (ent == E_FACEI) {
        v0x = A::ld(u0);
        const float* r0 = w0 - ev;
        const float s0 = fmaf(0.5f, A::ld(r0 + ev) - A::ld(r0), A::ld(r0));
        const float s1 = fmaf(0.5f, A::ld(r0 + pv + ev) - A::ld(r0 + pv), A::ld(r0 + pv));
        v0y = fmaf(0.5f, s1 - s0, s0);
    } else {
        const float* r0 = u0 - pu;
        const float s0 = fmaf(0.5f, A::ld(r0 + eu) - A::ld(r0), A::ld(r0));
        const float s1 = fmaf(0.5f, A::ld(r0 + pu + eu) - A::ld(r0 + pu), A::ld(r0 + pu));
        v0x = fmaf(0.5f, s1 - s0, s0);
        v0y = A::ld(w0);
    }
}

// A linear sample with what its transpose needs: the value (the bits lin32
// returns while no clamp fires), the cell offset (ox, oy) of its stencil
// from (bi, bj), the fractions, and the derivatives of the value by the
// position's two coordinates (index units).  No clamp: callers keep every
// position within a cell of (bi, bj), inside the ghosted array.
struct Lin32 {
    float val, gx, gy, tx, ty;
    int ox, oy;
};
template <typename A>
__device__ __forceinline__ Lin32 lin32g(const A& g, int bi, int bj, float fx, float fy) {
    Lin32 r;
    const float flx = floorf(fx), fly = floorf(fy);
    r.ox = (int)flx;
    r.oy = (int)fly;
    r.tx = fx - flx;
    r.ty = fy - fly;
    const float* r0 = g.at(bi + r.ox, bj + r.oy);
    const float* r1 = r0 + g.stride();
    const int e = g.step();
    const float a0 = A::ld(r0), a1 = A::ld(r0 + e);
    const float b0 = A::ld(r1), b1 = A::ld(r1 + e);
    const float s0 = fmaf(r.tx, a1 - a0, a0);
    const float s1 = fmaf(r.tx, b1 - b0, b0);
    r.val = fmaf(r.ty, s1 - s0, s0);
    r.gx = fmaf(r.ty, (b1 - b0) - (a1 - a0), a1 - a0);
    r.gy = s1 - s0;
    return r;
}

// Derivatives of the cubic B-spline weights cubic_w32 by t.
__device__ __forceinline__ void cubic_dw32(float t, float* dw) {
    const float s = 1.f - t, t2 = t * t;
    dw[0] = -0.5f * s * s;
    dw[1] = fmaf(1.5f, t2, -2.f * t);
    dw[2] = fmaf(-1.5f, t2, t + 0.5f);
    dw[3] = 0.5f * t2;
}

}  // namespace cf
