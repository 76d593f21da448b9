// Allocation-free divergence norms: cf_div_norms_noalloc.
//
// Who needs this: callers that own their velocity arrays and cannot (or may
// not) allocate device memory at the point where they want the norm, e.g. a
// host code whose device memory is entirely owned by its own pool allocator
// (a Kokkos/Cabana application with a fixed memory budget), or a monitoring
// hook that runs inside a latency-critical loop where cudaMalloc/cudaFree
// would synchronise the device.  The regular entry point needs a cf_ctx,
// and creating one allocates every field and solver vector.
//
// The variant computes what cf_div_norms computes for an FP64 context (same
// per-cell divergence, same fixed reduction order, so the results are bit
// for bit equal; a mixed context squares in FP32 and can differ in the last
// bits of the L2 norm) but keeps its reduction scratch -- one partial sum and one partial
// max per 64 x 16-cell unit, plus the last-block ticket -- in the
// file-scope device array below, which every GPU that loads this library
// holds until the process exits (1 MiB).
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "../../include/cajitafluids_gb300.h"
#include "cf_internal.cuh"

namespace {

// [0, MAX): per-unit sums of b^2; [MAX, 2 MAX): per-unit max |b|;
// slot 2 MAX: last-block ticket (an unsigned int in the first 4 bytes).
static __device__ __align__(256) double g_noalloc_scratch[2 * CF_NOALLOC_MAX_UNITS + 32];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Once per device, with that device current: the device address of the
// scratch array (the host-side symbol is only a stand-in, never a pointer a
// kernel may use).  The cached address is that of the primary context's
// module; it goes stale after cudaDeviceReset, which callers must not mix
// with this entry point.
int scratch_for_current_device(double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return CF_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return CF_OK;
}

struct NoAllocArgs {
    const double *u, *v;
    long long u_pitch, v_pitch;
    int nx, ny, per_x, per_y, G, U;
    double mscale, dx;
    double* scratch;
    double* out;
};

__device__ __forceinline__ double div_cell(const NoAllocArgs& a, int gi, int gj) {
    int ie = gi + 1, jn = gj + 1;
    if (a.per_x && ie == a.nx) ie = 0;
    if (a.per_y && jn == a.ny) jn = 0;
    double u0 = a.u[gj * a.u_pitch + gi], u1 = a.u[gj * a.u_pitch + ie];
    double v0 = a.v[gj * a.v_pitch + gi], v1 = a.v[jn * a.v_pitch + gi];
    double t = u1 - u0;
    t = t + v1;
    t = t - v0;
    return a.mscale * t;
}

__global__ void __launch_bounds__(CF_RED_THREADS) k_div_norms_noalloc(NoAllocArgs a) {
    double* part_sum = a.scratch;
    double* part_max = a.scratch + CF_NOALLOC_MAX_UNITS;
    unsigned int* ticket = reinterpret_cast<unsigned int*>(a.scratch + 2 * CF_NOALLOC_MAX_UNITS);
    const int lane = threadIdx.x & 31;
    const int unit = blockIdx.x * CF_RED_WARPS + (threadIdx.x >> 5);
    double ass = 0.0, amx = 0.0;
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
                double b = div_cell(a, c, j);
                ass = fma(b, b, ass);
                amx = fmax(amx, fabs(b));
            }
    }
    ass = cf::warp_fold(ass);
    amx = cf::warp_max(amx);
    if (unit < a.U && lane == 0) {
        part_sum[unit] = ass;
        part_max[unit] = amx;
    }
    if (cf::last_block_arrive(ticket)) {
        double ss = cf::final_tree(part_sum, a.U);
        double mx = cf::final_max(part_max, a.U);
        if (threadIdx.x == 0) {
            *ticket = 0;
            a.out[0] = sqrt(ss) * a.dx;
            a.out[1] = mx;
        }
    }
}

}  // namespace

extern "C" int cf_div_norms_noalloc(const double* u, ptrdiff_t u_pitch, const double* v, ptrdiff_t v_pitch, int nx,
                                    int ny, int periodic_x, int periodic_y, double dx, double* out, void* stream) {
    if (!u || !v || !out || nx <= 0 || ny <= 0 || !(dx > 0.0)) return CF_ERR_INVALID;
    const int ux = periodic_x ? nx : nx + 1;
    if (u_pitch < ux || v_pitch < nx) return CF_ERR_INVALID;
    const long long G = (nx + CF_UNIT_COLS - 1) / CF_UNIT_COLS;
    const long long B = (ny + CF_BAND_ROWS - 1) / CF_BAND_ROWS;
    if (G * B > CF_NOALLOC_MAX_UNITS) return CF_ERR_TOO_LARGE;
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the ticket must start at zero; the partials are fully rewritten
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch + 2 * CF_NOALLOC_MAX_UNITS);
    if (cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s) != cudaSuccess) return CF_ERR_CUDA;
    NoAllocArgs a;
    a.u = u;
    a.v = v;
    a.u_pitch = u_pitch;
    a.v_pitch = v_pitch;
    a.nx = nx;
    a.ny = ny;
    a.per_x = periodic_x ? 1 : 0;
    a.per_y = periodic_y ? 1 : 0;
    a.G = (int)G;
    a.U = (int)(G * B);
    a.mscale = -(1.0 / dx);
    a.dx = dx;
    a.scratch = scratch;
    a.out = out;
    int blocks = (a.U + CF_RED_WARPS - 1) / CF_RED_WARPS;
    k_div_norms_noalloc<<<blocks, CF_RED_THREADS, 0, s>>>(a);
    return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}
