// selftest.cu -- a self-test of the bounded device waits.
//
// Every mbarrier wait of the sweep kernels is bounded by a wall-clock limit
// (tma.cuh: mbar_wait_bounded); on timeout the waiting thread sets the
// device error block's timeout flag, the kernel returns, and the host maps
// the flag to SCRUST_TIMEOUT.  Running that path inside a sweep would need a
// copy or an MMA that never completes, which is not something to do to a
// GPU.  This kernel exercises the same wait and the same mapping on an
// mbarrier that nothing ever arrives on: one thread, no bulk copy and no
// tensor-core work in flight, and a limit of at most 100 ms.
#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "tma.cuh"

namespace scrust {

namespace {

__global__ void bounded_wait_kernel(int* err, unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    fence_barrier_init();
    // Phase 0 never completes: no thread arrives.
    mbar_wait_bounded(&bar, 0u, err, limit_ns);
}

}  // namespace

}  // namespace scrust

using namespace scrust;

extern "C" {

int32_t scrust_cuda_selftest_bounded_wait(scrust_context* ctx, uint64_t limit_ns, scrust_status* st) {
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (limit_ns == 0 || limit_ns > 100000000ull)
        return fail(st, SCRUST_INVALID_PARAMETER, "expected a wait limit in (0, 100 ms], got %llu ns",
                    (unsigned long long)limit_ns);
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    bounded_wait_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_err, (unsigned long long)limit_ns);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(st, e, "bounded wait self-test");
    ctx->launches += 1;
    return collect_device_errors(ctx, st);
}

}  // extern "C"
