// measure_static.cu — the FP64 energy/virial/momentum reduction of
// mdg_system_measure, for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs while
// another component owns the device heap (a custom pool allocator that must
// see every allocation), latency-critical loops where an allocation's implicit
// synchronisation is not allowed, and sandboxed plug-in hosts that only hand
// out pre-registered device buffers. mdg_measure_static gives them the same
// reduction on arrays they already own: the only scratch it needs, the
// per-block partial sums, lives in the file-scope device array below.
//
// Limits and sharing:
//  - kStaticParts blocks of kStaticItems atoms each, so at most
//    kStaticMaxAtoms atoms per call; larger inputs are rejected.
//  - The array exists once per GPU that loads the library and is held until
//    the process exits (kStaticBytes bytes).
//  - Every call on a device uses the same array. Calls whose kernels overlap
//    on the GPU (different streams, or different host threads) race on it;
//    order such calls on one stream. Each call writes every partial it reads,
//    so nothing has to be cleared between calls.
//  - The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it. With
//    lazy module loading (the CUDA default) that lookup also loads this
//    module on the device, which creates the array and can synchronise:
//    make the first call on each device at set-up, as a warm-up, before any
//    stream capture and outside any loop that must not wait.
//  - An error already pending on the calling thread (from an earlier CUDA
//    call) is reported as such before anything is launched; errors of this
//    call's own launches are reported after them.
#include <cuda_runtime.h>

#include <mutex>

#include "mdg_host.h"

namespace mdg {

constexpr int kStaticThreads = 256;
constexpr int kStaticItems = 8;                       // atoms per thread
constexpr int kStaticParts = 4096;                    // blocks (partials)
constexpr size_t kStaticMaxAtoms = (size_t)kStaticParts * kStaticThreads * kStaticItems;  // 8,388,608
constexpr int kStaticSlots = 8;                       // doubles per partial
constexpr size_t kStaticBytes = ((size_t)kStaticParts * kStaticSlots + 16) * sizeof(double);

// partials [kStaticParts][8], then 16 doubles: totals and the COM velocity
static __device__ __align__(256) double g_measure_scratch[(size_t)kStaticParts * kStaticSlots + 16];
static_assert(sizeof(g_measure_scratch) == kStaticBytes, "static scratch size (262,272 bytes per device)");

struct StaticMeasureArgs {
    size_t n;
    const double *m, *vx, *vy, *vz, *Ep, *Em, *V0, *V4, *V8;
};

__device__ void static_block_sum(double* sh, double* vals, int nv) {
    int t = threadIdx.x;
    for (int k = 0; k < nv; ++k) sh[k * kStaticThreads + t] = vals[k];
    __syncthreads();
    for (int s = kStaticThreads / 2; s > 0; s >>= 1) {
        if (t < s)
            for (int k = 0; k < nv; ++k) sh[k * kStaticThreads + t] += sh[k * kStaticThreads + t + s];
        __syncthreads();
    }
}

// Pass 1: Ep, Em, virial trace, momentum and mass per block.
__global__ void __launch_bounds__(kStaticThreads) k_static_measure1(StaticMeasureArgs A, double* scratch) {
    __shared__ double sh[7 * kStaticThreads];
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    size_t base = (size_t)blockIdx.x * kStaticThreads * kStaticItems + threadIdx.x;
    for (int q = 0; q < kStaticItems; ++q) {
        size_t i = base + (size_t)q * kStaticThreads;
        if (i >= A.n) break;
        v[0] += A.Ep[i];
        v[1] += A.Em[i];
        v[2] += A.V0[i] + A.V4[i] + A.V8[i];
        v[3] += A.m[i] * A.vx[i];
        v[4] += A.m[i] * A.vy[i];
        v[5] += A.m[i] * A.vz[i];
        v[6] += A.m[i];
    }
    static_block_sum(sh, v, 7);
    if (threadIdx.x < 7) scratch[(size_t)blockIdx.x * kStaticSlots + threadIdx.x] = sh[threadIdx.x * kStaticThreads];
}

// Totals of pass 1 in a fixed order; COM velocity into the tail slots.
__global__ void k_static_measure_total1(int nparts, double* scratch) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nparts; ++b)
        for (int k = 0; k < 7; ++k) s[k] += scratch[(size_t)b * kStaticSlots + k];
    double* tail = scratch + (size_t)kStaticParts * kStaticSlots;
    for (int k = 0; k < 7; ++k) tail[k] = s[k];
    double tm = s[6];
    tail[8] = tm > 0.0 ? s[3] / tm : 0.0;
    tail[9] = tm > 0.0 ? s[4] / tm : 0.0;
    tail[10] = tm > 0.0 ? s[5] / tm : 0.0;
}

// Pass 2: kinetic energy relative to the COM velocity.
__global__ void __launch_bounds__(kStaticThreads) k_static_measure2(StaticMeasureArgs A, double* scratch) {
    __shared__ double sh[kStaticThreads];
    const double* com = scratch + (size_t)kStaticParts * kStaticSlots + 8;
    double ke = 0.0;
    size_t base = (size_t)blockIdx.x * kStaticThreads * kStaticItems + threadIdx.x;
    for (int q = 0; q < kStaticItems; ++q) {
        size_t i = base + (size_t)q * kStaticThreads;
        if (i >= A.n) break;
        double dx = A.vx[i] - com[0], dy = A.vy[i] - com[1], dz = A.vz[i] - com[2];
        ke += 0.5 * A.m[i] * (dx * dx + dy * dy + dz * dz);
    }
    double v[1] = {ke};
    static_block_sum(sh, v, 1);
    if (threadIdx.x == 0) scratch[(size_t)blockIdx.x * kStaticSlots + 7] = sh[0];
}

// Final: {Ep, Em, KE, Etot, virial, vcom x, y, z} into the caller's array.
__global__ void k_static_measure_total2(int nparts, const double* scratch, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double ke = 0.0;
    for (int b = 0; b < nparts; ++b) ke += scratch[(size_t)b * kStaticSlots + 7];
    const double* tail = scratch + (size_t)kStaticParts * kStaticSlots;
    out[0] = tail[0];
    out[1] = tail[1];
    out[2] = ke;
    out[3] = tail[0] + tail[1] + ke;
    out[4] = tail[2];
    out[5] = tail[8];
    out[6] = tail[9];
    out[7] = tail[10];
}

// Device address of g_measure_scratch, looked up once per device.
static double* static_scratch_ptr(int device, int* rc) {
    static std::mutex mu;
    static double* ptrs[64] = {};
    *rc = MDG_OK;
    if (device < 0 || device >= 64) {
        set_error("device index out of range");
        *rc = MDG_ERR_INVALID;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_measure_scratch);
        if (e != cudaSuccess) {
            *rc = cuda_status(e, "cudaGetSymbolAddress(g_measure_scratch)");
            return nullptr;
        }
        ptrs[device] = static_cast<double*>(p);
    }
    return ptrs[device];
}

}  // namespace mdg

extern "C" int mdg_measure_static(const double* d_m, const double* d_v, const double* d_Ep, const double* d_Em,
                                  const double* d_V, size_t n, double* d_out, void* stream) {
    using namespace mdg;
    if (!d_out || (n && (!d_m || !d_v || !d_Ep || !d_Em || !d_V))) {
        set_error("mdg_measure_static: null array");
        return MDG_ERR_INVALID;
    }
    if (n > kStaticMaxAtoms) {
        set_error("mdg_measure_static: at most 8,388,608 atoms per call (static scratch size)");
        return MDG_ERR_INVALID;
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    int rc;
    double* scratch = static_scratch_ptr(device, &rc);
    if (!scratch) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) return cuda_status(e, "mdg_measure_static: error pending from an earlier CUDA call");
    StaticMeasureArgs A;
    A.n = n;
    A.m = d_m;
    A.vx = d_v;
    A.vy = d_v + n;
    A.vz = d_v + 2 * n;
    A.Ep = d_Ep;
    A.Em = d_Em;
    A.V0 = d_V;
    A.V4 = d_V + 4 * n;
    A.V8 = d_V + 8 * n;
    size_t per = (size_t)kStaticThreads * kStaticItems;
    int nparts = n ? (int)((n + per - 1) / per) : 1;
    k_static_measure1<<<nparts, kStaticThreads, 0, st>>>(A, scratch);
    k_static_measure_total1<<<1, 32, 0, st>>>(nparts, scratch);
    k_static_measure2<<<nparts, kStaticThreads, 0, st>>>(A, scratch);
    k_static_measure_total2<<<1, 32, 0, st>>>(nparts, scratch, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "mdg_measure_static launch");
    return MDG_OK;
}
