// FP32 inner Jacobi-PCG iteration of the mixed-precision projection, fed by
// TMA.
//
// The FP32 solver vectors (r, p twice) carry a one-cell ghost ring:
// element (i, j), i in [-1, nx], j in [-1, ny], lives at
// base[(j + 1) * pitch + i + 4], so owned column 0 sits on a 16-byte boundary.
// Wall ghosts stay zero; along a periodic axis the thread that writes an
// edge cell also writes its ghost copy, so every halo a kernel reads was
// written by an earlier launch.
//
// Each kernel is persistent (two CTAs per SM).  A CTA walks tiles of 128 x 16
// owned cells; for each tile a single thread issues 2-D TMA copies
// (cp.async.bulk.tensor) of 136 x 18 boxes -- the tile, one halo row above and
// below and a 4-column (16-byte) pad on each side -- into one of three
// shared-memory stages, completing on an mbarrier.  While a tile is computed
// from shared memory the next two are in flight.  Stores go straight from
// registers (float4 where a full vector is owned).
//
//   K1  p <- M^-1 r + beta p (halo too, in shared memory) ; q <- A p ; p.q
//   K2  q <- A p (recomputed) ; x += alpha p (double-float) ; r -= alpha q ;
//       r.z , r.r
//
// Dot products: FP32 per thread within a tile, FP64 across tiles, warps and
// CTAs; the last CTA finishes the sum and advances the solver state.
// mbarrier waits are bounded: on timeout the CTA records ST_TIMEOUT, waits
// (bounded) for its own copies still in flight, and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <math.h>

#include "cf_ctx.cuh"

namespace cf {

#define FULLMASK32 0xffffffffu

constexpr int kTW = 128;                 // owned columns per tile
constexpr int kTH = 16;                  // owned rows per tile
constexpr int kBX = kTW + 8;             // box columns
constexpr int kBY = kTH + 2;             // box rows
constexpr int kBoxBytes = kBX * kBY * 4; // 9792
constexpr int kSlot = 9856;              // 128-byte aligned slot
constexpr int kStages = 3;
constexpr int kThreads = 256;
constexpr unsigned kWaitLimit = 1u << 22;
// the drain after a timeout waits longer than any tile wait: a CTA must not
// exit while one of its bulk copies may still be writing its shared memory
constexpr unsigned kDrainLimit = 1u << 24;
// the stalled wait of the timeout-path test (cf_test_stall_wait)
constexpr unsigned kStallLimit = 1u << 10;

struct Cg32T {
    int nx, ny, per_x, per_y, tiles_x, tiles, pitch;
    int mg;  // MG-PCG: K1 reads z (minv = 1), K2 leaves beta and rho to k_mg_rz32
    Stencil st;
    float *r, *pa, *pb;  // element (0, 0)
    float2* x;           // the solution as double-float pairs (owned cells, row pitch xpitch)
    int xpitch;
    double *part0, *part1;
    SolverState* S;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; true when the phase completed
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned limit) {
    for (unsigned k = 0; k < limit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ int ebits32t(const Cg32T& a, int i, int j) {
    int ci = wrap_index(i, a.nx, a.per_x), cj = wrap_index(j, a.ny, a.per_y);
    if (ci < 0) ci = 0;
    if (cj < 0) cj = 0;
    return edge_bits(ci, cj, a.nx, a.ny, a.per_x, a.per_y);
}

// store one owned value and, along a periodic axis, its ghost copy
__device__ __forceinline__ void put_ghosted(const Cg32T& a, float* o, int i, int j, float val) {
    const ptrdiff_t row = (ptrdiff_t)j * a.pitch;
    o[row + i] = val;
    if (a.per_x) {
        if (i == 0) o[row + a.nx] = val;
        if (i == a.nx - 1) o[row - 1] = val;
    }
    if (a.per_y) {
        if (j == 0) o[(ptrdiff_t)a.ny * a.pitch + i] = val;
        if (j == a.ny - 1) o[-(ptrdiff_t)a.pitch + i] = val;
    }
}

// store four consecutive owned values starting at column i
__device__ __forceinline__ void put4(const Cg32T& a, float* o, int i, int j, float4 v, bool ghosts) {
    if (i + 3 < a.nx) {
        *reinterpret_cast<float4*>(o + (ptrdiff_t)j * a.pitch + i) = v;
        if (ghosts && ((a.per_x && (i == 0 || i + 3 == a.nx - 1)) || (a.per_y && (j == 0 || j == a.ny - 1)))) {
            put_ghosted(a, o, i, j, v.x);
            put_ghosted(a, o, i + 1, j, v.y);
            put_ghosted(a, o, i + 2, j, v.z);
            put_ghosted(a, o, i + 3, j, v.w);
        }
        return;
    }
    float vv[4] = {v.x, v.y, v.z, v.w};
    for (int k = 0; k < 4; ++k)
        if (i + k < a.nx) {
            if (ghosts)
                put_ghosted(a, o, i + k, j, vv[k]);
            else
                o[(ptrdiff_t)j * a.pitch + i + k] = vv[k];
        }
}

__device__ __forceinline__ float stencil1(const Cg32T& a, int i, int j, float c, float w, float e, float s, float n) {
    float q = a.st.diag32[ebits32t(a, i, j)] * c;
    q = fmaf(a.st.ms32, w, q);
    q = fmaf(a.st.ms32, e, q);
    q = fmaf(a.st.ms32, s, q);
    q = fmaf(a.st.ms32, n, q);
    return q;
}

// A p for the four cells (i0..i0+3, j) of a lane from the shared tile P
// (row stride kBX, owned (c, r) at [r + 1][c + 4]).
template <bool INTERIOR>
__device__ __forceinline__ float4 apply4(const Cg32T& a, const float* P, int lane, int row, int i0, int j,
                                         float4& pc) {
    const float* rc = P + (row + 1) * kBX + 4 + 4 * lane;
    pc = *reinterpret_cast<const float4*>(rc);
    float4 pu = *reinterpret_cast<const float4*>(rc - kBX);
    float4 pd = *reinterpret_cast<const float4*>(rc + kBX);
    float left = __shfl_up_sync(FULLMASK32, pc.w, 1);
    float right = __shfl_down_sync(FULLMASK32, pc.x, 1);
    if (lane == 0) left = rc[-1];
    if (lane == 31) right = rc[4];
    float4 q;
    if (INTERIOR) {
        const float d0 = a.st.diag32[0], ms = a.st.ms32;
        q.x = fmaf(ms, pd.x, fmaf(ms, pu.x, fmaf(ms, pc.y, fmaf(ms, left, d0 * pc.x))));
        q.y = fmaf(ms, pd.y, fmaf(ms, pu.y, fmaf(ms, pc.z, fmaf(ms, pc.x, d0 * pc.y))));
        q.z = fmaf(ms, pd.z, fmaf(ms, pu.z, fmaf(ms, pc.w, fmaf(ms, pc.y, d0 * pc.z))));
        q.w = fmaf(ms, pd.w, fmaf(ms, pu.w, fmaf(ms, right, fmaf(ms, pc.z, d0 * pc.w))));
    } else {
        q.x = stencil1(a, i0, j, pc.x, left, pc.y, pu.x, pd.x);
        q.y = stencil1(a, i0 + 1, j, pc.y, pc.x, pc.z, pu.y, pd.y);
        q.z = stencil1(a, i0 + 2, j, pc.z, pc.y, pc.w, pu.z, pd.z);
        q.w = stencil1(a, i0 + 3, j, pc.w, pc.z, right, pu.w, pd.w);
    }
    return q;
}

// true when no cell of the tile or of its halo is next to a wall: every
// diagonal and preconditioner entry is then the interior value
__device__ __forceinline__ bool interior_tile(const Cg32T& a, int i0, int j0) {
    bool wx = !a.per_x && (i0 <= 1 || i0 + kTW >= a.nx - 1);
    bool wy = !a.per_y && (j0 <= 1 || j0 + kTH >= a.ny - 1);
    bool full = i0 + kTW <= a.nx && j0 + kTH <= a.ny;
    return full && !(wx || wy);
}

__device__ __forceinline__ bool running(const SolverState* S) {
    return *(volatile const int*)&S->status == ST_RUNNING && *(volatile const int*)&S->inner_status == ST_RUNNING;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
    v = warp_fold(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = red[0];
    for (int k = 1; k < kThreads / 32; ++k) t = t + red[k];
    __syncthreads();
    return t;
}

// Timeout path: record the status and wait (bounded, with the longer drain
// limit) for this CTA's copies still in flight.
__device__ void abandon(SolverState* S, const uint64_t* bars, int kfirst, int ktiles) {
    if (threadIdx.x == 0) {
        atomicExch(&S->status, (int)ST_TIMEOUT);
        for (int k = kfirst; k < ktiles && k < kfirst + kStages; ++k)
            mbar_wait(smem_u32(&bars[k % kStages]), (uint32_t)((k / kStages) & 1), kDrainLimit);
    }
    __syncthreads();
}

// K1: new direction (with halo) in shared memory, stencil, p.q
__global__ void __launch_bounds__(kThreads, 2)
    k_tma_dir_matvec32(const __grid_constant__ CUtensorMap map_r, const __grid_constant__ CUtensorMap map_pa,
                       const __grid_constant__ CUtensorMap map_pb, Cg32T a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[kStages];
    // test knob: an mbarrier that nothing arrives on (cf_test_stall_wait)
    __shared__ __align__(8) uint64_t never;
    __shared__ double red[kThreads / 32];
    SolverState* S = a.S;
    if (!running(S)) return;
    const int it = S->inner_iter;
    const bool first = it == 0 || S->restart;
    const bool stall = S->test_stall != 0 && blockIdx.x == 0;
    const float beta = (float)S->beta_in;
    const CUtensorMap* map_old = (it & 1) ? &map_pb : &map_pa;
    float* pnew = (it & 1) ? a.pa : a.pb;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ntile = (a.tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    unsigned char* sb = smem + ((128u - (smem_u32(smem) & 127u)) & 127u);  // TMA wants 128-byte slots
    auto stage_ptr = [&](int s, int arr) { return reinterpret_cast<float*>(sb + (s * 2 + arr) * kSlot); };
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(smem_u32(&bars[s]), 1);
        mbar_init(smem_u32(&never), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int k) {
        int t = (int)blockIdx.x + k * (int)gridDim.x;
        int s = k % kStages;
        int x = (t % a.tiles_x) * kTW, y = (t / a.tiles_x) * kTH;
        uint32_t bar = smem_u32(&bars[s]);
        mbar_expect_tx(bar, 2 * kBoxBytes);
        tma_load_2d(smem_u32(stage_ptr(s, 0)), &map_r, x, y, bar);
        tma_load_2d(smem_u32(stage_ptr(s, 1)), map_old, x, y, bar);
    };
    if (tid == 0)
        for (int k = 0; k < kStages && k < ntile; ++k) issue(k);
    float acc = 0.f;  // FP32 over this block's tiles (no FP64 in the loop)
    for (int k = 0; k < ntile; ++k) {
        const int s = k % kStages;
        const int t = (int)blockIdx.x + k * (int)gridDim.x;
        const int i0 = (t % a.tiles_x) * kTW, j0 = (t / a.tiles_x) * kTH;
        // with the test knob, block 0's first wait is on the barrier nothing
        // arrives on, with a short limit: it times out, and the drain below
        // waits for the real copies of stages 0..2
        bool ok = (stall && k == 0) ? mbar_wait(smem_u32(&never), 0u, kStallLimit)
                                    : mbar_wait(smem_u32(&bars[s]), (uint32_t)((k / kStages) & 1), kWaitLimit);
        if (__syncthreads_or(!ok)) {
            abandon(S, bars, k, ntile);
            return;
        }
        float* R = stage_ptr(s, 0);
        float* P = stage_ptr(s, 1);
        const bool inner = interior_tile(a, i0, j0);
        // phase 1: P <- M^-1 R + beta P over the whole box (halo included)
        for (int v = tid; v < kBY * (kBX / 4); v += kThreads) {
            float4 rv = reinterpret_cast<float4*>(R)[v];
            float4 pv = reinterpret_cast<float4*>(P)[v];
            float4 o;
            if (inner) {
                const float m0 = a.st.minv32[0];
                o.x = m0 * rv.x;
                o.y = m0 * rv.y;
                o.z = m0 * rv.z;
                o.w = m0 * rv.w;
            } else {
                int row = v / (kBX / 4), c4 = v % (kBX / 4);
                int j = j0 - 1 + row, i = i0 - 4 + 4 * c4;
                o.x = a.st.minv32[ebits32t(a, i, j)] * rv.x;
                o.y = a.st.minv32[ebits32t(a, i + 1, j)] * rv.y;
                o.z = a.st.minv32[ebits32t(a, i + 2, j)] * rv.z;
                o.w = a.st.minv32[ebits32t(a, i + 3, j)] * rv.w;
            }
            if (!first) {
                o.x = fmaf(beta, pv.x, o.x);
                o.y = fmaf(beta, pv.y, o.y);
                o.z = fmaf(beta, pv.z, o.z);
                o.w = fmaf(beta, pv.w, o.w);
            }
            reinterpret_cast<float4*>(P)[v] = o;
        }
        __syncthreads();
        // phase 2: q = A p on the owned cells, p.q, store p
        float part = 0.f;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const int row = 2 * warp + rr, j = j0 + row, i = i0 + 4 * lane;
            float4 pc;
            float4 q = inner ? apply4<true>(a, P, lane, row, i, j, pc) : apply4<false>(a, P, lane, row, i, j, pc);
            if (j < a.ny && i < a.nx) {
                part = fmaf(pc.x, q.x, part);
                if (i + 1 < a.nx) part = fmaf(pc.y, q.y, part);
                if (i + 2 < a.nx) part = fmaf(pc.z, q.z, part);
                if (i + 3 < a.nx) part = fmaf(pc.w, q.w, part);
                put4(a, pnew, i, j, pc, true);
            }
        }
        acc = acc + part;
        fence_proxy_async();
        __syncthreads();
        if (tid == 0 && k + kStages < ntile) issue(k + kStages);
    }
    double tot = block_sum((double)acc, red);
    if (tid == 0) a.part0[blockIdx.x] = tot;
    if (last_block_arrive(&S->ticket[5])) {
        double pq = final_tree(a.part0, gridDim.x);
        if (tid == 0) {
            S->ticket[5] = 0;
            S->restart = 0;
            if (isnan(pq))
                S->status = ST_NAN;
            else if (!(pq > 0.0))
                S->inner_status = ST_BREAKDOWN;  // FP32 noise floor: refine and restart
            else
                S->alpha_in = S->rho_in / pq;
        }
    }
}

// K2: recompute A p, update x (double-float) and r, r.z and r.r.  x is read
// with plain loads issued before the tile's copies are awaited.
__global__ void __launch_bounds__(kThreads, 2)
    k_tma_update32(const __grid_constant__ CUtensorMap map_r, const __grid_constant__ CUtensorMap map_pa,
                   const __grid_constant__ CUtensorMap map_pb, Cg32T a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[kStages];
    __shared__ double red[kThreads / 32];
    SolverState* S = a.S;
    if (!running(S)) return;
    const int it = S->inner_iter;
    const CUtensorMap* map_p = (it & 1) ? &map_pa : &map_pb;
    const float alpha = (float)S->alpha_in, malpha = -alpha;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ntile = (a.tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    unsigned char* sb = smem + ((128u - (smem_u32(smem) & 127u)) & 127u);  // TMA wants 128-byte slots
    auto stage_ptr = [&](int s, int arr) { return reinterpret_cast<float*>(sb + (s * 2 + arr) * kSlot); };
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(smem_u32(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int k) {
        int t = (int)blockIdx.x + k * (int)gridDim.x;
        int s = k % kStages;
        int x = (t % a.tiles_x) * kTW, y = (t / a.tiles_x) * kTH;
        uint32_t bar = smem_u32(&bars[s]);
        mbar_expect_tx(bar, 2 * kBoxBytes);
        tma_load_2d(smem_u32(stage_ptr(s, 0)), map_p, x, y, bar);
        tma_load_2d(smem_u32(stage_ptr(s, 1)), &map_r, x, y, bar);
    };
    if (tid == 0)
        for (int k = 0; k < kStages && k < ntile; ++k) issue(k);
    float arz = 0.f, arr = 0.f;  // FP32 over this block's tiles (no FP64 in the loop)
    for (int k = 0; k < ntile; ++k) {
        const int s = k % kStages;
        const int t = (int)blockIdx.x + k * (int)gridDim.x;
        const int i0 = (t % a.tiles_x) * kTW, j0 = (t / a.tiles_x) * kTH;
        const bool inner = interior_tile(a, i0, j0);
        // x of the lane's cells (i .. i + 3) on its two rows
        float4 xv[2][2];
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const int j = j0 + 2 * warp + rr, i = i0 + 4 * lane;
            const float2* xp = a.x + (size_t)j * a.xpitch + i;
            if (inner) {
                xv[rr][0] = reinterpret_cast<const float4*>(xp)[0];
                xv[rr][1] = reinterpret_cast<const float4*>(xp)[1];
            } else {
                float* xf = reinterpret_cast<float*>(xv[rr]);
                for (int c = 0; c < 4; ++c) {
                    const bool in = j < a.ny && i + c < a.nx;
                    const float2 v = in ? xp[c] : make_float2(0.f, 0.f);
                    xf[2 * c] = v.x;
                    xf[2 * c + 1] = v.y;
                }
            }
        }
        bool ok = mbar_wait(smem_u32(&bars[s]), (uint32_t)((k / kStages) & 1), kWaitLimit);
        if (__syncthreads_or(!ok)) {
            abandon(S, bars, k, ntile);
            return;
        }
        const float* P = stage_ptr(s, 0);
        const float* R = stage_ptr(s, 1);
        float prz = 0.f, prr = 0.f;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const int row = 2 * warp + rr, j = j0 + row, i = i0 + 4 * lane;
            float4 pc;
            float4 q = inner ? apply4<true>(a, P, lane, row, i, j, pc) : apply4<false>(a, P, lane, row, i, j, pc);
            const int off = (row + 1) * kBX + 4 + 4 * lane;
            float4 rv = *reinterpret_cast<const float4*>(R + off);
            float2 x0 = df_add_f(make_float2(xv[rr][0].x, xv[rr][0].y), alpha * pc.x);
            float2 x1 = df_add_f(make_float2(xv[rr][0].z, xv[rr][0].w), alpha * pc.y);
            float2 x2 = df_add_f(make_float2(xv[rr][1].x, xv[rr][1].y), alpha * pc.z);
            float2 x3 = df_add_f(make_float2(xv[rr][1].z, xv[rr][1].w), alpha * pc.w);
            rv.x = fmaf(malpha, q.x, rv.x);
            rv.y = fmaf(malpha, q.y, rv.y);
            rv.z = fmaf(malpha, q.z, rv.z);
            rv.w = fmaf(malpha, q.w, rv.w);
            if (inner) {
                const float m0 = a.st.minv32[0];
                float s2 = fmaf(rv.w, rv.w, fmaf(rv.z, rv.z, fmaf(rv.y, rv.y, rv.x * rv.x)));
                prr += s2;
                prz = fmaf(m0, s2, prz);
                float4* xo = reinterpret_cast<float4*>(a.x + (size_t)j * a.xpitch + i);
                xo[0] = make_float4(x0.x, x0.y, x1.x, x1.y);
                xo[1] = make_float4(x2.x, x2.y, x3.x, x3.y);
                put4(a, a.r, i, j, rv, true);
            } else if (j < a.ny && i < a.nx) {
                float rvs[4] = {rv.x, rv.y, rv.z, rv.w};
                const float2 xs[4] = {x0, x1, x2, x3};
                float2* xo = a.x + (size_t)j * a.xpitch + i;
                for (int c = 0; c < 4; ++c)
                    if (i + c < a.nx) {
                        float z = a.st.minv32[ebits32t(a, i + c, j)] * rvs[c];
                        prz = fmaf(rvs[c], z, prz);
                        prr = fmaf(rvs[c], rvs[c], prr);
                        xo[c] = xs[c];
                    }
                put4(a, a.r, i, j, rv, true);
            }
        }
        arz = arz + prz;
        arr = arr + prr;
        __syncthreads();
        if (tid == 0 && k + kStages < ntile) issue(k + kStages);
    }
    double trz = block_sum((double)arz, red);
    double trr = block_sum((double)arr, red);
    if (tid == 0) {
        a.part0[blockIdx.x] = trz;
        a.part1[blockIdx.x] = trr;
    }
    if (last_block_arrive(&S->ticket[6])) {
        double rz = final_tree(a.part0, gridDim.x);
        double rr = final_tree(a.part1, gridDim.x);
        if (tid == 0) {
            S->ticket[6] = 0;
            S->rho_prev = S->rho_in;
            if (!a.mg) {
                S->beta_in = rz / S->rho_in;
                S->rho_in = rz;
            }
            S->rr_in = rr;
            if (rr > S->rr_in0) S->rr_in0 = rr;
            S->inner_iter = it + 1;
            S->iter = S->iter + 1;
            // reliable update when the recursive residual fell by delta since
            // the last one, or already looks converged
            if (isnan(rr))
                S->status = ST_NAN;
            else if (rr <= S->tau2 * S->rr_in0 || rr <= S->target2)
                S->inner_status = ST_CONVERGED;
            else if (S->iter >= S->max_iter)
                S->inner_status = ST_MAXIT;
        }
    }
}

// --------------------------------------------------------------------------
// Mixed MG-PCG helpers.  z = V-cycle(r) is written to the owned cells of z32;
// along periodic axes its ghost ring is refreshed here (wall ghosts stay 0).
__global__ void k_z32_ghosts(float* z, int nx, int ny, int pitch, int per_x, int per_y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (per_x && t < ny) {
        float* row = z + (ptrdiff_t)t * pitch;
        row[-1] = row[nx - 1];
        row[nx] = row[0];
    }
    if (per_y && t < nx) {
        z[-(ptrdiff_t)pitch + t] = z[(ptrdiff_t)(ny - 1) * pitch + t];
        z[(ptrdiff_t)ny * pitch + t] = z[t];
    }
}

// rho = r.z (FP32 per lane over a 64 x 16 unit, FP64 beyond).  After an
// inner iteration: beta = rho_new / rho.  After the residual was re-formed
// from the FP64 solution (S->refreshed): beta = rho_new / rho_prev, which
// keeps the search direction across a reliable update (ignored on a restart).
__global__ void __launch_bounds__(CF_RED_THREADS)
    k_mg_rz32(const float* r, const float* z, int nx, int ny, int pitch, int G, int U, double* part,
              SolverState* S) {
    if (!running(S)) return;
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    float arz = 0.f;
    if (unit < U) {
        const int g = unit % G, band = unit / G;
        const int c0 = g * CF_UNIT_COLS + 2 * lane;
        const int j0 = band * CF_BAND_ROWS;
        const int j1 = min(j0 + CF_BAND_ROWS, ny);
        for (int j = j0; j < j1; ++j)
            for (int s = 0; s < 2; ++s) {
                const int c = c0 + s;
                if (c >= nx) continue;
                const ptrdiff_t k = (ptrdiff_t)j * pitch + c;
                arz = fmaf(r[k], z[k], arz);
            }
    }
    double drz = warp_fold((double)arz);
    if (unit < U && lane == 0) part[unit] = drz;
    if (last_block_arrive(&S->ticket[7])) {
        double rz = final_tree(part, U);
        if (threadIdx.x == 0) {
            S->ticket[7] = 0;
            double den = S->refreshed ? S->rho_prev : S->rho_in;
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

// --------------------------------------------------------------------------
// host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D map over a ghosted FP32 vector's storage (pitch x (ny + 2) floats)
static int make_map(cf_ctx* c, CUtensorMap* m, float* base) {
    auto fn = encode_fn();
    if (!fn) return fail(c, CF_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    cuuint64_t dims[2] = {(cuuint64_t)c->p32, (cuuint64_t)(c->ph.ny + 2)};
    cuuint64_t strides[1] = {(cuuint64_t)c->p32 * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)kBX, (cuuint32_t)kBY};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(c, CF_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return CF_OK;
}

int cg32_setup(cf_ctx* c) {
    int rc = make_map(c, &c->map_r, c->r32b);
    if (!rc) rc = make_map(c, &c->map_pa, c->pa32b);
    if (!rc) rc = make_map(c, &c->map_pb, c->pb32b);
    if (rc) return rc;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c->tiles_x = (c->ph.nx + kTW - 1) / kTW;
    c->tiles = c->tiles_x * ((c->ph.ny + kTH - 1) / kTH);
    rc = cuda_check(c, cudaFuncSetAttribute(k_tma_dir_matvec32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            kStages * 2 * kSlot + 128),
                    "smem attribute");
    if (!rc)
        rc = cuda_check(c, cudaFuncSetAttribute(k_tma_update32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                kStages * 2 * kSlot + 128),
                        "smem attribute");
    // persistent grids: as many CTAs as fit on the GPU at once
    int occ1 = 0, occ2 = 0;
    if (!rc)
        rc = cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, k_tma_dir_matvec32, kThreads,
                                                                         kStages * 2 * kSlot + 128),
                        "occupancy");
    if (!rc)
        rc = cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, k_tma_update32, kThreads,
                                                                         kStages * 2 * kSlot + 128),
                        "occupancy");
    if (rc) return rc;
    occ1 = occ1 < 1 ? 1 : occ1;
    occ2 = occ2 < 1 ? 1 : occ2;
    c->cta32 = c->tiles < occ1 * sms ? c->tiles : occ1 * sms;
    c->cta32b = c->tiles < occ2 * sms ? c->tiles : occ2 * sms;
    return rc;
}

// z32 (ghosted, zero) and its tensor map, for the mixed MG-PCG
int cg32_mg_setup(cf_ctx* c) {
    if (c->z32b) return CF_OK;
    size_t n32 = (size_t)c->p32 * (c->ph.ny + 2);
    cudaError_t e = cudaMalloc(&c->z32b, n32 * sizeof(float));
    if (e != cudaSuccess) return fail(c, CF_ERR_NOMEM, "z32: cudaMalloc failed");
    c->allocs.push_back(c->z32b);
    int rc = cuda_check(c, cudaMemsetAsync(c->z32b, 0, n32 * sizeof(float), c->stream), "z32 memset");
    c->z32.a = c->z32b + c->p32 + 4;
    c->z32.pitch = c->p32;
    if (!rc) rc = make_map(c, &c->map_z, c->z32b);
    return rc;
}

static Cg32T cg32_args(cf_ctx* c, const Stencil& st) {
    Cg32T a{};
    a.nx = c->ph.nx;
    a.ny = c->ph.ny;
    a.per_x = c->ph.per_x;
    a.per_y = c->ph.per_y;
    a.tiles_x = c->tiles_x;
    a.tiles = c->tiles;
    a.pitch = c->p32;
    a.st = st;
    a.x = reinterpret_cast<float2*>(c->x.a);
    a.xpitch = c->vpitch;
    a.r = c->r32.a;
    a.pa = c->pa32.a;
    a.pb = c->pb32.a;
    a.part0 = c->partials;
    a.part1 = c->partials + c->n_units;
    a.S = c->S;
    return a;
}

void cg32_launch_iteration(cf_ctx* c, const Stencil& st) {
    Cg32T a = cg32_args(c, st);
    k_tma_dir_matvec32<<<c->cta32, kThreads, kStages * 2 * kSlot + 128, c->stream>>>(c->map_r, c->map_pa, c->map_pb, a);
    k_tma_update32<<<c->cta32b, kThreads, kStages * 2 * kSlot + 128, c->stream>>>(c->map_r, c->map_pa, c->map_pb,
                                                                            a);
}

// z = V-cycle(r32), its periodic ghosts, rho = r.z; returns kernels launched
int cg32_mg_precondition(cf_ctx* c, double scale) {
    bool done = false;
    int n = mg_vcycle(c, scale, &done);
    if (done) return n;  // r.z, the scalars and z's ghosts came with the finest post-smoothing
    if (c->ph.per_x || c->ph.per_y) {
        int m = c->ph.nx > c->ph.ny ? c->ph.nx : c->ph.ny;
        k_z32_ghosts<<<(m + 255) / 256, 256, 0, c->stream>>>(c->z32.a, c->ph.nx, c->ph.ny, c->p32, c->ph.per_x,
                                                             c->ph.per_y);
        n += 1;
    }
    k_mg_rz32<<<(c->n_units + CF_RED_WARPS - 1) / CF_RED_WARPS, CF_RED_THREADS, 0, c->stream>>>(
        c->r32.a, c->z32.a, c->ph.nx, c->ph.ny, c->p32, c->G, c->n_units, c->partials, c->S);
    return n + 1;
}

// K1 on z (M^-1 = 1) and K2 of one MG-PCG inner iteration.  When every
// iteration ends with a reliable update (c->x_only), K2 reduces to the x
// update, which the fused reliable update does (k_outer_resid<true>), so K1
// runs alone.
void cg32_launch_pair_mg(cf_ctx* c, const Stencil& st) {
    Stencil stz = st;
    for (int b = 0; b < 16; ++b) stz.minv32[b] = 1.0f;
    Cg32T a = cg32_args(c, stz);
    a.mg = 1;
    k_tma_dir_matvec32<<<c->cta32, kThreads, kStages * 2 * kSlot + 128, c->stream>>>(c->map_z, c->map_pa, c->map_pb, a);
    if (!c->x_only) {
        k_tma_update32<<<c->cta32b, kThreads, kStages * 2 * kSlot + 128, c->stream>>>(c->map_r, c->map_pa, c->map_pb,
                                                                                a);
    }
}

}  // namespace cf
