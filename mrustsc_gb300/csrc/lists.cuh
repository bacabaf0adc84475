// lists.cuh -- per-row candidate lists shared by the candidate kernels and the
// rerank: the thresholds that bound them and the warp-cooperative prune.
//
// A list holds (column id, s) pairs with s = |b|^2 - 2 a.b (the row's own
// |a|^2 is a constant shift).  Its threshold theta only ever decreases; a
// column is admitted while s < theta.  A prune sets theta from the k-th
// smallest s in the list through the form's error bound and drops entries at
// or above it.
#pragma once

#include <math.h>
#include <stdint.h>

#include "common.cuh"

namespace scrust {

constexpr int kListMaxEntriesPerLane = 16;  // list storage per (row, segment) <= 512

// Plain (FP32) form: additive margin 2 beta.
struct PlainBound {
    float margin;
    __device__ __forceinline__ float theta(float kth) const { return kth + margin; }
};

// Tensor (16-bit operand) form.  With Q the squared distance between the
// quantised points (Q = s + A, A = |a_hat|^2, computed within +-delta) and
// |sqrt(Q) - sqrt(D)| <= eps for the caller's squared distance D, a column
// whose lower bound on D is above the k-th smallest upper bound cannot be a
// neighbour: theta = (sqrt(kth + A + delta) + 2 eps)^2 + delta - A, where eps2
// carries 2 eps.
struct TensorBound {
    float A, delta, eps2;
    __device__ __forceinline__ float theta(float kth) const {
        const double q = fmax(0.0, (double)kth + (double)A) + (double)delta;
        const double r = sqrt(q) + (double)eps2;
        const double th = r * r + (double)delta - (double)A;
        return __double2float_ru(th + 1e-6 * fabs(th) + 1e-30);
    }
    // The same bound in f32 with every step rounded towards +inf, then
    // raised past itself: never at or below the exact bound.
    __device__ __forceinline__ float theta_f32(float kth) const {
        const float q = __fadd_ru(fmaxf(0.f, __fadd_ru(kth, A)), delta);
        const float r = __fadd_ru(__fsqrt_ru(q), eps2);
        const float th = __fsub_ru(__fadd_ru(__fmul_ru(r, r), delta), A);
        return __fadd_ru(__fadd_ru(th, __fmul_ru(fabsf(th), 1e-6f)), 1e-30f);
    }
};

struct PruneResult {
    float theta;   // new threshold (warp-uniform)
    uint32_t cnt;  // entries kept (warp-uniform)
};

// Prunes one row's list with the whole warp: theta <- min(old, bound.theta(k-th
// smallest value)), entries at or above theta dropped (compacted in place).
// Every lane returns the same result.
template <class Bound>
__device__ PruneResult prune_core(uint32_t* ids, float* vals, uint32_t cnt, int k, const Bound& bound,
                                  float theta_old) {
    // Fewer than k entries: there is no k-th smallest to bound the row by.
    if ((int)cnt < k) return PruneResult{theta_old, cnt};
    const int lane = threadIdx.x & 31;
    float v[kListMaxEntriesPerLane];
    uint32_t id[kListMaxEntriesPerLane];
#pragma unroll
    for (int e = 0; e < kListMaxEntriesPerLane; e++) {
        const int p = e * 32 + lane;
        if (p < (int)cnt) {
            v[e] = vals[p];
            id[e] = ids[p];
        } else {
            v[e] = __int_as_float(0x7f800000);
            id[e] = 0xffffffffu;
        }
    }
    // k-th smallest key by binary radix selection over the bits below the
    // keys' common prefix; each step is one warp-wide count.
    uint32_t kmin = 0xffffffffu, kmax = 0u;
#pragma unroll
    for (int e = 0; e < kListMaxEntriesPerLane; e++) {
        if (e * 32 + lane < (int)cnt) {
            const uint32_t key = float_key(v[e]);
            kmin = min(kmin, key);
            kmax = max(kmax, key);
        }
    }
    kmin = __reduce_min_sync(0xffffffffu, kmin);
    kmax = __reduce_max_sync(0xffffffffu, kmax);
    const uint32_t diff = kmin ^ kmax;
    const int top = diff ? 31 - __clz(diff) : -1;
    const uint32_t low = top >= 0 ? (uint32_t)((2ull << top) - 1ull) : 0u;
    uint32_t prefix = kmin & ~low, decided = ~low;
    int rank = k;
#pragma unroll 1
    for (int bit = top; bit >= 0; --bit) {
        const uint32_t b = 1u << bit;
        int c0 = 0;
#pragma unroll
        for (int e = 0; e < kListMaxEntriesPerLane; e++) {
            const uint32_t key = float_key(v[e]);
            c0 += (e * 32 + lane < (int)cnt) && ((key & decided) == prefix) && !(key & b);
        }
        const int total = __reduce_add_sync(0xffffffffu, c0);
        if (rank > total) {
            rank -= total;
            prefix |= b;
        }
        decided |= b;
    }
    const float theta = fminf(theta_old, bound.theta(key_float(prefix)));
    uint32_t out = 0;
#pragma unroll
    for (int e = 0; e < kListMaxEntriesPerLane; e++) {
        const bool keep = (e * 32 + lane < (int)cnt) && (v[e] < theta);
        const uint32_t ballot = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const uint32_t pos = out + __popc(ballot & lanemask_lt());
            ids[pos] = id[e];
            vals[pos] = v[e];
        }
        out += __popc(ballot);
    }
    __syncwarp();
    return PruneResult{theta, out};
}

// prune_core for a list whose threshold and count live in shared memory:
// lane 0 writes them back.  A row with `cap` or more entries inside its own
// threshold overflows: its list is emptied, its threshold set to -inf and
// *overflow_flag raised, so the exact fallback finishes it.
template <class Bound>
__device__ void prune_list(uint32_t* ids, float* vals, uint32_t cnt, int k, int cap, const Bound& bound,
                           float* thr, uint32_t* cnt_out, uint32_t* overflow_flag) {
    const PruneResult r = prune_core(ids, vals, cnt, k, bound, *thr);
    if ((threadIdx.x & 31) == 0) {
        if ((int)r.cnt >= cap) {
            *overflow_flag = 1u;
            *thr = __int_as_float(0xff800000);
            *cnt_out = 0;
        } else {
            *thr = r.theta;
            *cnt_out = r.cnt;
        }
    }
    __syncwarp();
}

}  // namespace scrust
