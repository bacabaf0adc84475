// common.cuh -- device utilities shared by the kNN and connectivities kernels.
//
// Numerical contract (kept identical in the oracle, oracle/neighbors_oracle.c):
//   * FP32 difference form:  r = sum_t (a_t - b_t)^2 with four interleaved
//     fused accumulators (dimension t goes to accumulator t mod 4) joined as
//     (acc0 + acc1) + (acc2 + acc3).  Relative error <= (ceil(D/4) + 4) * 2^-24.
//   * FP64 adjudication: s = s + (a_t - b_t) * (a_t - b_t) in dimension order
//     with no fused operations, then sqrt -- the rounding of
//     oracle_knn_fp64_rows, bit for bit.
//   * Reference-snap form: the sequential fma chain on centred coordinates and
//     the ((D + 2) * eps) * (|q|^2 + |c|^2) snap of the reference Metal kernel
//     (crates/scrust-gpu/src/kernels/knn.rs:223-240).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace scrust {

constexpr float kF32Eps = 1.1920928955078125e-07f;  // 2^-23
constexpr double kUnit32 = 5.9604644775390625e-08;  // 2^-24
constexpr float kTieAbs = 1e-37f;                    // covers f32 underflow of squared differences

// Error flags written by kernels into the context's device error block.
enum DeviceError : int {
    DERR_TIMEOUT = 0,        // a bounded mbarrier / flag wait ran out
    DERR_CANDIDATES = 1,     // a row's candidate set was inconsistent (fewer than k)
    DERR_TIE_OVERFLOW = 2,   // more equidistant candidates than the fallback holds
    DERR_ZERO_ROW = 3,       // cosine metric given an all-zero row
    DERR_BAD_INDEX = 4,      // connectivities given an id >= n
    DERR_COUNT = 8
};

__device__ __forceinline__ uint32_t float_key(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_float(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------------------
// Distances.

// FP32 difference form with four interleaved fused accumulators.
__device__ __forceinline__ float dist2_f32(const float* __restrict__ a, const float* __restrict__ b,
                                           int d) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int t = 0;
    for (; t + 3 < d; t += 4) {
        float d0 = __fsub_rn(__ldg(a + t), __ldg(b + t));
        float d1 = __fsub_rn(__ldg(a + t + 1), __ldg(b + t + 1));
        float d2 = __fsub_rn(__ldg(a + t + 2), __ldg(b + t + 2));
        float d3 = __fsub_rn(__ldg(a + t + 3), __ldg(b + t + 3));
        s0 = __fmaf_rn(d0, d0, s0);
        s1 = __fmaf_rn(d1, d1, s1);
        s2 = __fmaf_rn(d2, d2, s2);
        s3 = __fmaf_rn(d3, d3, s3);
    }
    if (t < d) {
        float d0 = __fsub_rn(__ldg(a + t), __ldg(b + t));
        s0 = __fmaf_rn(d0, d0, s0);
    }
    if (t + 1 < d) {
        float d1 = __fsub_rn(__ldg(a + t + 1), __ldg(b + t + 1));
        s1 = __fmaf_rn(d1, d1, s1);
    }
    if (t + 2 < d) {
        float d2 = __fsub_rn(__ldg(a + t + 2), __ldg(b + t + 2));
        s2 = __fmaf_rn(d2, d2, s2);
    }
    return __fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3));
}

// dist2_f32 on rows padded with zeros to d4 float4 words: the same
// accumulators in the same order (the padding adds exact zeros), so the same
// value, with a quarter of the loads.
__device__ __forceinline__ float dist2_f32_v4(const float4* __restrict__ a, const float4* __restrict__ b, int d4) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll 4
    for (int t = 0; t < d4; ++t) {
        const float4 x = __ldg(a + t), y = __ldg(b + t);
        const float d0 = __fsub_rn(x.x, y.x), d1 = __fsub_rn(x.y, y.y), d2 = __fsub_rn(x.z, y.z),
                    d3 = __fsub_rn(x.w, y.w);
        s0 = __fmaf_rn(d0, d0, s0);
        s1 = __fmaf_rn(d1, d1, s1);
        s2 = __fmaf_rn(d2, d2, s2);
        s3 = __fmaf_rn(d3, d3, s3);
    }
    return __fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3));
}

// 32 bytes from global memory in one load (32-byte aligned; read-only path).
__device__ __forceinline__ void ldg_v8(const float* p, float (&r)[8]) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7])
        : "l"(p));
}

// dist2_f32 on rows padded with zeros to d8 32-byte words (32-byte aligned):
// the same accumulators in the same order (the padding adds exact zeros), so
// the same value; a lane's loads then use whole 32-byte sectors.
__device__ __forceinline__ float dist2_f32_v8(const float* __restrict__ a, const float* __restrict__ b, int d8) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll 1
    for (int t = 0; t < d8; ++t) {
        float x[8], y[8];
        ldg_v8(a + 8 * t, x);
        ldg_v8(b + 8 * t, y);
#pragma unroll
        for (int h = 0; h < 8; h += 4) {
            const float d0 = __fsub_rn(x[h], y[h]), d1 = __fsub_rn(x[h + 1], y[h + 1]),
                        d2 = __fsub_rn(x[h + 2], y[h + 2]), d3 = __fsub_rn(x[h + 3], y[h + 3]);
            s0 = __fmaf_rn(d0, d0, s0);
            s1 = __fmaf_rn(d1, d1, s1);
            s2 = __fmaf_rn(d2, d2, s2);
            s3 = __fmaf_rn(d3, d3, s3);
        }
    }
    return __fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3));
}

// Relative error bound of dist2_f32 with a 1.5x safety factor.
__host__ __device__ __forceinline__ float dist2_f32_gamma(int d) {
    return (float)(1.5 * ((double)((d + 3) / 4) + 5.0) * kUnit32);
}

// The reference Metal kernel's value: sequential fma on centred coordinates,
// snapped to 0 below ((D + 2) * eps) * (|q|^2 + |c|^2).
__device__ __forceinline__ float dist2_reference_snap(const float* __restrict__ a,
                                                      const float* __restrict__ b, int d,
                                                      float na, float nb) {
    float s = 0.f;
    for (int t = 0; t < d; t++) {
        float delta = __fsub_rn(__ldg(a + t), __ldg(b + t));
        s = __fmaf_rn(delta, delta, s);
    }
    float threshold = __fmul_rn(__fmul_rn(__fadd_rn((float)d, 2.0f), kF32Eps), __fadd_rn(na, nb));
    return s < threshold ? 0.0f : s;
}

// FP64 squared distance, dimension order, no fused operations.
__device__ __forceinline__ double dist2_f64(const float* __restrict__ a, const float* __restrict__ b,
                                            int d) {
    double s = 0.0;
    for (int t = 0; t < d; t++) {
        double diff = __dsub_rn((double)__ldg(a + t), (double)__ldg(b + t));
        s = __dadd_rn(s, __dmul_rn(diff, diff));
    }
    return s;
}

// FP64 cosine distance 1 - a.b / (|a| |b|) with precomputed FP64 norms.
__device__ __forceinline__ double cosine_f64(const float* __restrict__ a, const float* __restrict__ b,
                                             int d, double na, double nb) {
    double dot = 0.0;
    for (int t = 0; t < d; t++) dot = __dadd_rn(dot, __dmul_rn((double)__ldg(a + t), (double)__ldg(b + t)));
    return __dsub_rn(1.0, __ddiv_rn(dot, __dmul_rn(na, nb)));
}

// ---------------------------------------------------------------------------
// Teams: the same selection / sort / adjudication code runs on one warp per
// row (the common case) or one block per row (the fallback for rows with
// very many equidistant candidates).

struct WarpTeam {
    int rank;
    __device__ WarpTeam() : rank(threadIdx.x & 31) {}
    __device__ __forceinline__ int size() const { return 32; }
    __device__ __forceinline__ void sync() const { __syncwarp(); }
    __device__ __forceinline__ int count(bool p) const { return __popc(__ballot_sync(0xffffffffu, p)); }
    __device__ __forceinline__ int any(bool p) const { return __any_sync(0xffffffffu, p); }
    __device__ __forceinline__ int sum(int v) const { return __reduce_add_sync(0xffffffffu, v); }
};

struct BlockTeam {
    int rank;
    int* scratch;  // one shared int
    __device__ explicit BlockTeam(int* s) : rank(threadIdx.x), scratch(s) {}
    __device__ __forceinline__ int size() const { return blockDim.x; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ int count(bool p) const { return __syncthreads_count(p); }
    __device__ __forceinline__ int any(bool p) const { return __syncthreads_or(p); }
    __device__ __forceinline__ int sum(int v) const {
        __syncthreads();
        if (rank == 0) *scratch = 0;
        __syncthreads();
        if (v) atomicAdd(scratch, v);
        __syncthreads();
        return *(volatile int*)scratch;
    }
};

// The rank-th smallest (1-based) of the high 32 bits of keys[0..m).
template <class Team>
__device__ uint32_t team_select_hi(const Team& team, const unsigned long long* keys, int m, int rank) {
    uint32_t prefix = 0, decided = 0;
    for (int bit = 31; bit >= 0; --bit) {
        const uint32_t b = 1u << bit;
        int c0 = 0;
        for (int p = team.rank; p < m; p += team.size()) {
            uint32_t hk = (uint32_t)(keys[p] >> 32);
            c0 += ((hk & decided) == prefix) && !(hk & b);
        }
        int total = team.sum(c0);
        if (rank > total) {
            rank -= total;
            prefix |= b;
        }
        decided |= b;
    }
    return prefix;
}

// Ascending bitonic sort of keys[0..P), P a power of two.
template <class Team>
__device__ void team_bitonic_sort(const Team& team, unsigned long long* keys, int P) {
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = team.rank; t < (P >> 1); t += team.size()) {
                int i = 2 * t - (t & (stride - 1));
                int j = i + stride;
                bool up = (i & size) == 0;
                unsigned long long a = keys[i], b = keys[j];
                if ((a > b) == up) {
                    keys[i] = b;
                    keys[j] = a;
                }
            }
            team.sync();
        }
    }
}

__host__ __device__ __forceinline__ int next_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

}  // namespace scrust
