// Internal declarations shared by the CUDA translation units of libcfgpu.
//
// Storage (one GPU holds the whole grid):
//   * q, u, v: ghosted arrays, ghost depth 3 (src/Solver.hpp:78), x fastest.
//     Local index (i, j) of the ghosted Cajita space maps to
//     origin[j * pitch + i]; the owned corner (3, 3) sits on a 256-byte
//     boundary.  Extents: cells (nx+6, ny+6), I-faces (nx+7, ny+6),
//     J-faces (nx+6, ny+7) (tests/tstMesh.cpp:61-68).
//   * solver vectors: owned cells only, row pitch a multiple of 32 words.
//
// FP64 kernels are compiled with --fmad=false; every fused multiply-add is
// an explicit fma() so that results are reproducible bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CF_HALO 3
// element offset of a ghosted array's local (0, 0) from its allocation: local
// column CF_HALO (owned column 0) of every row lands on a 128-byte boundary
#define CF_COL0 (32 - CF_HALO)
#define CF_UNIT_COLS 64   // columns per reduction unit (32 lanes x 2)
#define CF_BAND_ROWS 16   // rows per reduction unit
#define CF_RED_THREADS 256
#define CF_RED_WARPS (CF_RED_THREADS / 32)

namespace cf {

enum Entity { E_CELL = 0, E_FACEI = 1, E_FACEJ = 2 };
enum SolveStatus { ST_CONVERGED = 0, ST_MAXIT = 1, ST_BREAKDOWN = 2, ST_NAN = 3, ST_TIMEOUT = 4, ST_RUNNING = 100 };

template <typename T>
struct Grid {
    T* o;       // local (0, 0)
    int pitch;  // elements per row
    int ex, ey; // ghosted extents
    __host__ __device__ T& at(int i, int j) const { return o[(size_t)j * pitch + i]; }
};

// Physical setup shared by the kernels (passed by value).
struct Phys {
    int nx, ny;
    int per_x, per_y;
    double dx, rdx;
    double gl[2];       // low corner of the ghosted local mesh
    double low[3][2];   // coordinate of local index 0 per entity (spline origin)
    int bc[4];          // left, bottom, right, top
    double bbox[4];     // inflow box x0, y0, x1, y1
    // per entity (cell, I-face, J-face): local indices [i0, i1) x [j0, j1)
    // whose coordinates lie in the inflow box (the FP64 test, evaluated once
    // on the host)
    int box[3][4];
    double src_q;
    double src_vel[2];
    int src_mode;
    double force[2];
    int force_density;
    unsigned quirks;
};

// the inflow box test on local indices (ranges the host evaluated with the
// FP64 coordinate test, src/InflowSource.hpp:78-88)
__device__ __forceinline__ bool in_box_idx(const Phys& p, int ent, int li, int lj) {
    return li >= p.box[ent][0] && li < p.box[ent][1] && lj >= p.box[ent][2] && lj < p.box[ent][3];
}

// Matrix tables indexed by wall-adjacency bits (1 left, 2 right, 4 bottom, 8 top).
struct Stencil {
    double diag[16];
    double minv[16];
    double ms;          // -scale (off-diagonal legs)
    float diag32[16];
    float minv32[16];
    float ms32;
};

// Device-resident solver scalars.
struct SolverState {
    double bb, rr, rho, alpha, beta;
    double tol2, abs2, area;
    // mixed precision: inner solve
    double rr_in0, rr_in, rho_in, alpha_in, beta_in, tau2;
    double rr_out, inner_tol2, target2, rho_prev;
    int use_abs, restart;
    int refreshed;  // mixed MG: r was just re-formed from the FP64 solution
    int trips, trip_limit;  // device-resident loop: trips taken, and the bound
    int iter, max_iter, status;
    int inner_iter, inner_status;
    int outer_iter, max_outer;
    int test_stall;  // test knob (cf_test_stall_wait): see k_tma_dir_matvec32
    int xsel;        // mixed MG-PCG, fused x update: the x buffer holding the solution
    unsigned int ticket[8];
};

struct Vec64 {
    double* a;
    int pitch;
};
struct Vec32 {
    float* a;
    int pitch;
};

// --------------------------------------------------------------------------
// Fixed-order reductions.  One warp reduces one unit of 64 x 16 cells: lane l
// owns columns 64g + 2l, 64g + 2l + 1 and accumulates row by row; the lane
// sums are folded by a xor butterfly; the last block to finish folds all
// unit partials: 256 strided accumulators, a butterfly per warp, and the 8
// warp sums added in order.
// FP32 butterfly sum of a warp (fixed order); the FP32 kernels fold their
// per-lane partials this way and hand the warp total on as FP64, so that no
// FP64 operation (a slow pipe on GB300) sits in their inner loops
__device__ __forceinline__ float warp_fold_f(float s) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, m);
    return s;
}

__device__ __forceinline__ double warp_fold(double s) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, m);
    return s;
}

__device__ __forceinline__ double warp_max(double s) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, m));
    return s;
}

// Returns true in the block that arrives last.  Every thread fences its own
// global writes before the block takes its ticket.
__device__ __forceinline__ bool last_block_arrive(unsigned int* ticket) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(ticket, 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (am_last) __threadfence();
    return am_last;
}

// Canonical final sum over n partials; blockDim.x must be 256.  All threads
// return the same value.
// Each thread adds partial[t], partial[t + 256], ... in that order; the
// loads go out eight at a time ahead of the additions (one block does this
// at the end of a launch, so a chain of dependent loads would be its tail).
constexpr int CF_FOLD_BATCH = 8;
__device__ __forceinline__ double final_tree(const double* partial, int n) {
    __shared__ double ws[CF_RED_WARPS];
    double s = 0.0;
    int u = threadIdx.x;
    for (; u + (CF_FOLD_BATCH - 1) * CF_RED_THREADS < n; u += CF_FOLD_BATCH * CF_RED_THREADS) {
        double v[CF_FOLD_BATCH];
#pragma unroll
        for (int k = 0; k < CF_FOLD_BATCH; ++k) v[k] = __ldcg(partial + u + k * CF_RED_THREADS);
#pragma unroll
        for (int k = 0; k < CF_FOLD_BATCH; ++k) s = s + v[k];
    }
    for (; u < n; u += CF_RED_THREADS) s = s + __ldcg(partial + u);
    s = warp_fold(s);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    double tot = ws[0];
#pragma unroll
    for (int k = 1; k < CF_RED_WARPS; ++k) tot = tot + ws[k];
    __syncthreads();
    return tot;
}

__device__ __forceinline__ double final_max(const double* partial, int n) {
    __shared__ double ws[CF_RED_WARPS];
    double s = 0.0;
    int u = threadIdx.x;
    for (; u + (CF_FOLD_BATCH - 1) * CF_RED_THREADS < n; u += CF_FOLD_BATCH * CF_RED_THREADS) {
        double v[CF_FOLD_BATCH];
#pragma unroll
        for (int k = 0; k < CF_FOLD_BATCH; ++k) v[k] = __ldcg(partial + u + k * CF_RED_THREADS);
#pragma unroll
        for (int k = 0; k < CF_FOLD_BATCH; ++k) s = fmax(s, v[k]);
    }
    for (; u < n; u += CF_RED_THREADS) s = fmax(s, __ldcg(partial + u));
    s = warp_max(s);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    double tot = ws[0];
#pragma unroll
    for (int k = 1; k < CF_RED_WARPS; ++k) tot = fmax(tot, ws[k]);
    __syncthreads();
    return tot;
}

// Wall-adjacency bits of cell (gi, gj); periodic axes have no walls.
__device__ __forceinline__ int edge_bits(int gi, int gj, int nx, int ny, int per_x, int per_y) {
    int b = 0;
    if (!per_x) b |= (gi == 0 ? 1 : 0) | (gi == nx - 1 ? 2 : 0);
    if (!per_y) b |= (gj == 0 ? 4 : 0) | (gj == ny - 1 ? 8 : 0);
    return b;
}

// Wrap an index along a periodic axis; returns -1 outside a wall axis.
__device__ __forceinline__ int wrap_index(int g, int n, int per) {
    if (g >= 0 && g < n) return g;
    if (!per) return -1;
    g %= n;
    return g < 0 ? g + n : g;
}

// Asynchronous global -> shared copies (cp.async, completion by groups per
// thread: a thread that reads back only what it copied needs no barrier).
__device__ __forceinline__ void cpa16(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa8(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa4(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// FP32 <-> FP64 conversions by bit manipulation on the integer pipe (GB300's
// FP64 pipe, which executes the hardware conversions, is narrow).  Straight
// from the IEEE 754 binary32/binary64 layouts: a normal binary32 widens
// exactly by re-biasing the exponent (+896) and shifting the significand by
// 29 bits; a binary64 in the binary32 normal range narrows by keeping the top
// 23 significand bits and rounding on the 29 dropped ones, to nearest with
// ties to even (a carry out of the significand increments the exponent,
// which is the correctly rounded result up to infinity).  Zeros take the same
// path; a warp holding any other special value (subnormal, infinity, NaN,
// out of range) uses the hardware conversion.
__device__ __forceinline__ double f2d_exact(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    const bool fast = e != 0xffu && (e != 0u || m == 0u);
    if (__all_sync(__activemask(), fast)) {
        const unsigned hi = (u & 0x80000000u) | (e == 0u ? 0u : ((e + 896u) << 20) | (m >> 3));
        const unsigned lo = m << 29;
        return __hiloint2double((int)hi, (int)lo);
    }
    return (double)f;
}

__device__ __forceinline__ float d2f_rn(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned e = (hi >> 20) & 0x7ffu;
    const bool zero = (hi & 0x7fffffffu) == 0u && lo == 0u;
    const bool fast = zero || (e >= 897u && e <= 1150u);
    if (__all_sync(__activemask(), fast)) {
        const unsigned m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned rest = lo & 0x1fffffffu, half = 0x10000000u;
        const unsigned up = (rest > half || (rest == half && (m23 & 1u))) ? 1u : 0u;
        const unsigned fb = (hi & 0x80000000u) | (zero ? 0u : (((e - 896u) << 23) | m23) + up);
        return __uint_as_float(fb);
    }
    return __double2float_rn(d);
}

// Spline-coordinate helpers for the FP64 samplers.
// The clamp of the logical coordinate to [lo, hi] (lo, hi small non-negative
// integers), its integer part and that part as a double are done on the
// integer pipe: for doubles of one sign the IEEE 754 bit patterns order like
// the values (a set sign bit makes the signed pattern negative; patterns
// above +infinity's are NaNs), the integer part of x in [0, 2^31) is the
// significand with the hidden bit shifted right by 52 - exponent, and an int
// k > 0 is exactly the double with exponent 31 - clz(k) and k's bits below
// its top one as the significand.  The results are those of fmin/fmax, the
// truncating conversion and the int-to-double conversion, which run on
// GB300's narrow FP64 pipe.
__device__ __forceinline__ double exact_double(int k) {  // k >= 0
    if (k == 0) return 0.0;
    const int e = 31 - __clz(k);
    const unsigned long long m = ((unsigned long long)(unsigned)k << (52 - e)) & 0xFFFFFFFFFFFFFull;
    return __longlong_as_double((long long)(((unsigned long long)(e + 1023) << 52) | m));
}

// x's bit pattern for ordered comparisons with non-negative bounds (-0 as +0)
__device__ __forceinline__ long long order_bits(double x) {
    const long long b = __double_as_longlong(x);
    return b == (long long)0x8000000000000000ull ? 0 : b;
}

// !(lo <= x && x <= hi) for lo <= hi non-negative (true for NaN)
__device__ __forceinline__ bool outside_bits(double x, double lo, double hi) {
    const long long b = order_bits(x);
    return b < __double_as_longlong(lo) || b > __double_as_longlong(hi);
}

// fmin(fmax(x, lo), hi) for lo <= hi non-negative (NaN -> lo, as fmax gives)
__device__ __forceinline__ double clamp_bits(double x, double lo, double hi) {
    const long long b = order_bits(x);
    if (b < __double_as_longlong(lo) || b > 0x7FF0000000000000LL) return lo;
    if (b > __double_as_longlong(hi)) return hi;
    return x;
}

// (int)x for x in [0, 2^31)
__device__ __forceinline__ int trunc_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)(b >> 52) - 1023;
    if (e < 0) return 0;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    return (int)(m >> (52 - e));
}

// Double-float (hi + lo FP32 pair) error-free sums (Knuth two-sum, Dekker
// quick two-sum); exact with --fmad=false.
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return make_float2(s, e);
}
__device__ __forceinline__ float2 df_quick(float a, float b) {  // |a| >= |b|
    float s = a + b;
    return make_float2(s, b - (s - a));
}
// double-float + FP32
__device__ __forceinline__ float2 df_add_f(float2 x, float e) {
    float2 s = df_two_sum(x.x, e);
    s.y = s.y + x.y;
    return df_quick(s.x, s.y);
}
__device__ __forceinline__ float2 df_add(float2 x, float2 y) {
    float2 s = df_two_sum(x.x, y.x);
    float2 t = df_two_sum(x.y, y.y);
    s.y = s.y + t.x;
    s = df_quick(s.x, s.y);
    s.y = s.y + t.y;
    return df_quick(s.x, s.y);
}
__device__ __forceinline__ float2 df_mul(float2 x, float2 y) {
    float p = x.x * y.x;
    float e = fmaf(x.x, y.x, -p);
    e = fmaf(x.x, y.y, e);
    e = fmaf(x.y, y.x, e);
    return df_quick(p, e);
}
// Packed FP32 pairs: one f32x2 instruction (sm_100 and later) performs two
// independent FP32 operations, each rounded exactly as its scalar form, so
// pairing two rows of a stencil halves their instructions and keeps every bit.
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mov.b64 pc, {%6, %7};\n\tfma.rn.f32x2 pd, pa, pb, pc;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}

// An FP64 value as a pair: hi = the value rounded to FP32, lo = the rest
// rounded to FP32 (about 48 significant bits; one FP64 subtraction), and
// back (one FP64 addition, exact for pairs made this way).
__device__ __forceinline__ float2 df_split(double v) {
    const float hi = d2f_rn(v);
    return make_float2(hi, d2f_rn(v - f2d_exact(hi)));
}
__device__ __forceinline__ double df_value(float2 p) { return f2d_exact(p.x) + f2d_exact(p.y); }

}  // namespace cf

// Launch helpers implemented in the .cu files (called by cf_api.cu).
namespace cf {
struct Ctx;
}
