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
// The k-th smallest comes from a four-pass 8-bit radix select over a
// 256-bin histogram `hist` in shared memory owned by this warp.  Every lane
// returns the same result.
template <class Bound>
__device__ PruneResult prune_core(uint32_t* ids, float* vals, uint32_t cnt, int k, const Bound& bound,
                                  float theta_old, uint32_t* hist) {
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
    const int live = ((int)cnt + 31) / 32;  // entry slots that can hold data
    uint32_t prefix = 0, decided = 0;
    int rank = k;
#pragma unroll 1
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 24 - 8 * pass;
#pragma unroll
        for (int b = 0; b < 8; b++) hist[lane * 8 + b] = 0;
        __syncwarp();
#pragma unroll
        for (int e = 0; e < kListMaxEntriesPerLane; e++) {
            if (e < live && e * 32 + lane < (int)cnt) {
                const uint32_t key = float_key(v[e]);
                if ((key & decided) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
            }
        }
        __syncwarp();
        uint32_t c[8];
        uint32_t own = 0;
#pragma unroll
        for (int b = 0; b < 8; b++) {
            c[b] = hist[lane * 8 + b];
            own += c[b];
        }
        uint32_t incl = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int L = __ffs(__ballot_sync(0xffffffffu, (int)incl >= rank)) - 1;
        uint32_t digit = 0;
        int new_rank = 0;
        if (lane == L) {
            int r = rank - (int)(incl - own);
            int b = 0;
            for (; b < 7; b++) {
                if ((int)c[b] >= r) break;
                r -= (int)c[b];
            }
            digit = (uint32_t)(lane * 8 + b);
            new_rank = r;
        }
        digit = __shfl_sync(0xffffffffu, digit, L);
        rank = __shfl_sync(0xffffffffu, new_rank, L);
        prefix |= digit << shift;
        decided |= 255u << shift;
        __syncwarp();
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
                           float* thr, uint32_t* cnt_out, uint32_t* overflow_flag, uint32_t* hist) {
    const PruneResult r = prune_core(ids, vals, cnt, k, bound, *thr, hist);
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
