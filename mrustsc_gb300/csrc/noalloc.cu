// noalloc.cu -- umap's smooth_knn_dist on device-resident data through an
// entry point that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: processes that hand all
// of a GPU's memory to their own pool allocator (a framework's caching
// allocator, a query service that reserves its HBM budget at start-up and
// must never grow), and latency-critical loops where cudaMalloc's implicit
// device-wide synchronisation would stall every other stream.  For them this
// file provides scrust_cuda_smooth_knn_distances_noalloc: the caller passes
// the distances, sigmas and rhos buffers, and the only scratch the
// computation needs -- one FP64 partial sum per 4096 distances, then the
// global mean -- lives in a file-scope device array of fixed size.
//
// That array is part of the loaded module: every GPU that loads the library
// holds its 33 KB until the process exits.  Its device address is looked up
// once per device with cudaGetSymbolAddress (host code cannot use the
// array's name as a device address) on the first call that works on that
// device, and kept for the life of the process, so the entry point must not
// be used across a cudaDeviceReset of that device.  The device is the one
// that holds the caller's buffers (all three must be on the same device, and
// a non-default stream must belong to it); the calling thread's current
// device is set to it for the call and given back afterwards.  Every call on
// a device shares the one array; calls whose work overlaps on the GPU
// (different streams, no ordering between them) race on it and may read each
// other's partial sums.  Each call writes every scratch entry it reads before
// reading it, so nothing needs clearing between calls.
//
// The global mean (used only for the sigma of a row whose neighbours all sit
// at distance 0) is summed here in FP64 from per-chunk partials, while the
// reference sums in f32 in ndarray's unrolled order (which the regular entry
// point reproduces); the two means differ by a few 1e-6 relative at the
// largest accepted size, inside the 1e-5 sigma tolerance.
#include <math.h>

#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int64_t kChunk = (int64_t)kThreads * kItems;     // distances per partial sum
constexpr int kMaxPartials = 4096;
constexpr int64_t kMaxEntries = kChunk * kMaxPartials;     // 16,777,216 = largest n * k
constexpr int kMeanSlot = kMaxPartials;
constexpr int kMaxDevices = 64;

// Partial sums [0, kMaxPartials) and the global mean at kMeanSlot.
static __device__ __align__(256) double g_smooth_scratch[kMaxPartials + 32];

std::mutex g_setup_mu;
double* g_scratch_ptr[kMaxDevices] = {};

__global__ void __launch_bounds__(kThreads) noalloc_partial_kernel(const float* __restrict__ dist, int64_t total,
                                                                   double* __restrict__ scratch) {
    __shared__ double warp_sum[kThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kChunk;
    double s = 0.0;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int64_t i = base + (int64_t)it * kThreads + threadIdx.x;
        if (i < total) s += (double)dist[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += warp_sum[w];
        scratch[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kThreads) noalloc_mean_kernel(double* __restrict__ scratch, int partials,
                                                                int64_t total) {
    __shared__ double warp_sum[kThreads / 32];
    double s = 0.0;
    for (int p = threadIdx.x; p < partials; p += kThreads) s += scratch[p];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += warp_sum[w];
        scratch[kMeanSlot] = (double)__fdiv_rn(__double2float_rn(t), (float)total);
    }
}

// ndarray 0.16.1 unrolled_fold order for a row sum.
__device__ float row_sum_unrolled(const float* xs, int len) {
    float acc = 0.f;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f, p4 = 0.f, p5 = 0.f, p6 = 0.f, p7 = 0.f;
    while (len >= 8) {
        p0 = __fadd_rn(p0, xs[0]);
        p1 = __fadd_rn(p1, xs[1]);
        p2 = __fadd_rn(p2, xs[2]);
        p3 = __fadd_rn(p3, xs[3]);
        p4 = __fadd_rn(p4, xs[4]);
        p5 = __fadd_rn(p5, xs[5]);
        p6 = __fadd_rn(p6, xs[6]);
        p7 = __fadd_rn(p7, xs[7]);
        xs += 8;
        len -= 8;
    }
    acc = __fadd_rn(acc, __fadd_rn(p0, p4));
    acc = __fadd_rn(acc, __fadd_rn(p1, p5));
    acc = __fadd_rn(acc, __fadd_rn(p2, p6));
    acc = __fadd_rn(acc, __fadd_rn(p3, p7));
    for (int i = 0; i < len; i++) acc = __fadd_rn(acc, xs[i]);
    return acc;
}

// The per-row rho / bisection / sigma floor of crates/scrust-core/src/neighbors.rs:252-296,
// reading the global mean from the scratch array.
__global__ void noalloc_smooth_kernel(const float* __restrict__ dist, int64_t n, int k, double target,
                                      const double* __restrict__ scratch, float* __restrict__ sigmas,
                                      float* __restrict__ rhos) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* row = dist + i * k;
    float rho = 0.f;
    for (int j = 0; j < k; j++) {
        const float v = row[j];
        if (v > 0.f) {
            rho = v;
            break;
        }
    }
    const float fmax = 3.40282346638528859812e+38f;
    float low = 0.f, high = fmax, mid = 1.f;
    for (int it = 0; it < 64; it++) {
        float card = 0.f;
        for (int j = 0; j < k; j++) {
            const float offset = __fsub_rn(row[j], rho);
            const float term = offset > 0.f ? expf(__fdiv_rn(-offset, mid)) : 1.0f;
            card = __fadd_rn(card, term);
        }
        const double c64 = (double)card;
        if (fabs(c64 - target) < 1e-5) break;
        if (c64 > target) {
            high = mid;
            mid = __fdiv_rn(__fadd_rn(low, high), 2.0f);
        } else {
            low = mid;
            mid = high >= fmax ? __fmul_rn(mid, 2.0f) : __fdiv_rn(__fadd_rn(low, high), 2.0f);
        }
    }
    const float mean = (float)scratch[kMeanSlot];
    const float reference = rho > 0.f ? __fdiv_rn(row_sum_unrolled(row, k), (float)(k + 1)) : mean;
    sigmas[i] = fmaxf(mid, __fmul_rn(1e-3f, reference));
    rhos[i] = rho;
}

// The device that holds a caller buffer, or -1 when it is not device memory.
int device_of(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? a.device : -1;
}

// The scratch array's device address on device `dev` (which is current),
// looked up on the first call that works on that device.
int32_t scratch_for_device(int dev, double** out, scrust_status* st) {
    cudaError_t e = cudaSuccess;
    if (dev < 0 || dev >= kMaxDevices)
        return fail(st, SCRUST_NO_GPU, "device %d is beyond the %d devices this entry point tracks", dev,
                    kMaxDevices);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        double* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_smooth_scratch);
        if (e != cudaSuccess) return cuda_fail(st, e, "smooth_knn_noalloc: scratch address");
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return SCRUST_OK;
}

}  // namespace

}  // namespace scrust

using namespace scrust;

extern "C" int32_t scrust_cuda_smooth_knn_distances_noalloc(const float* distances, uint64_t n, uint32_t k,
                                                            float* sigmas, float* rhos, void* stream,
                                                            scrust_status* st) {
    if (n == 0 || k == 0)
        return fail(st, SCRUST_SHAPE, "expected a distance matrix with at least one cell and one neighbour, got %llu x %u",
                    (unsigned long long)n, k);
    if (!distances || !sigmas || !rhos) return fail(st, SCRUST_SHAPE, "expected non-null device pointers");
    const uint64_t total = n * (uint64_t)k;
    if (total / k != n || total > (uint64_t)kMaxEntries)
        return fail(st, SCRUST_INVALID_PARAMETER,
                    "n * k must be at most %lld for the allocation-free entry point (its scratch is a fixed "
                    "device array), got %llu x %u",
                    (long long)kMaxEntries, (unsigned long long)n, k);
    const int dev = device_of(distances);
    if (dev < 0 || device_of(sigmas) != dev || device_of(rhos) != dev)
        return fail(st, SCRUST_INVALID_PARAMETER,
                    "expected distances, sigmas and rhos in the device memory of one GPU, got buffers on devices "
                    "%d, %d and %d (-1: not device memory)",
                    dev, device_of(sigmas), device_of(rhos));
    cudaStream_t s = (cudaStream_t)stream;
    if (s) {
        int sdev = -1;
        if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
            cudaGetLastError();
            return fail(st, SCRUST_INVALID_PARAMETER, "expected a valid CUDA stream");
        }
        if (sdev != dev)
            return fail(st, SCRUST_INVALID_PARAMETER,
                        "expected a stream of device %d, which holds the buffers, got a stream of device %d", dev,
                        sdev);
    }
    DeviceGuard device_guard(dev);
    double* scratch = nullptr;
    int32_t rc = scratch_for_device(dev, &scratch, st);
    if (rc) return rc;
    const int partials = (int)((total + kChunk - 1) / kChunk);
    noalloc_partial_kernel<<<partials, kThreads, 0, s>>>(distances, (int64_t)total, scratch);
    noalloc_mean_kernel<<<1, kThreads, 0, s>>>(scratch, partials, (int64_t)total);
    noalloc_smooth_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(distances, (int64_t)n, (int)k,
                                                                      log2((double)(k + 1)), scratch, sigmas,
                                                                      rhos);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(st, e, "smooth_knn_noalloc");
    return ok(st);
}
