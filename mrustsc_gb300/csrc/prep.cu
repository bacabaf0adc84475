// prep.cu -- per-row preparation before candidate generation.
//
//   column means     f64, as crates/scrust-core/src/neighbors.rs:144-154 forms
//                    them (the sequential variant reproduces that order bit for
//                    bit; the parallel one is a deterministic two-level sum)
//   normalise rows   cosine metric: rows divided by their FP64 norm
//   centre/transpose centred f32 coordinates, (D_pad x n_pad) for the plain
//                    form's TMA tiles, squared norms by an fma chain
//                    (crates/scrust-gpu/src/kernels/knn.rs:148-155) and the
//                    largest centred norm
//   margins          per-row candidate margin from the derived error bound
//
// All kernels here are HBM-bound single passes over n x D floats.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

constexpr int kMeanRowsPerBlock = 2048;

__global__ void means_sequential_kernel(const float* __restrict__ x, int64_t n, int d,
                                        double* __restrict__ means) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d) return;
    double s = 0.0;
    for (int64_t r = 0; r < n; r++) s = __dadd_rn(s, (double)__ldg(x + r * d + c));
    means[c] = __ddiv_rn(s, (double)n);
}

__global__ void means_partial_kernel(const float* __restrict__ x, int64_t n, int d,
                                     double* __restrict__ partial) {
    int64_t r0 = (int64_t)blockIdx.x * kMeanRowsPerBlock;
    int64_t r1 = min(n, r0 + kMeanRowsPerBlock);
    for (int c = threadIdx.x; c < d; c += blockDim.x) {
        double s = 0.0;
        for (int64_t r = r0; r < r1; r++) s = __dadd_rn(s, (double)__ldg(x + r * d + c));
        partial[(int64_t)blockIdx.x * d + c] = s;
    }
}

__global__ void means_final_kernel(const double* __restrict__ partial, int blocks, int64_t n, int d,
                                   double* __restrict__ means) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d) return;
    double s = 0.0;
    for (int b = 0; b < blocks; b++) s = __dadd_rn(s, partial[(int64_t)b * d + c]);
    means[c] = __ddiv_rn(s, (double)n);
}

__global__ void normalise_rows_kernel(const float* __restrict__ x, int64_t n, int d,
                                      float* __restrict__ xn, double* __restrict__ norm64,
                                      int* __restrict__ err) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* row = x + i * d;
    double s = 0.0;
    for (int t = 0; t < d; t++) {
        double v = (double)__ldg(row + t);
        s = __dadd_rn(s, __dmul_rn(v, v));
    }
    double nrm = sqrt(s);
    norm64[i] = nrm;
    if (!(nrm > 0.0)) {
        atomicExch(err + DERR_ZERO_ROW, 1);
        nrm = 1.0;
    }
    for (int t = 0; t < d; t++) xn[i * d + t] = __double2float_rn(__ddiv_rn((double)__ldg(row + t), nrm));
}

// One thread per (padded) row: centred coordinates written transposed so the
// plain form's TMA boxes are [64 dims][128 rows]; the squared norm is the
// reference's fma chain; padding rows get +inf so their candidates are never
// admitted.
__global__ void centre_transpose_kernel(const float* __restrict__ x, int64_t n, int64_t n_pad, int d,
                                        int dp, const double* __restrict__ means,
                                        float* __restrict__ coords_t, float* __restrict__ norm2,
                                        float* __restrict__ cnorm, float* __restrict__ xcentred,
                                        uint32_t* __restrict__ max_norm_bits) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    const bool valid = i < n;
    float acc = 0.f;
    for (int t = 0; t < dp; t++) {
        float c = 0.f;
        if (valid && t < d) c = __double2float_rn(__dsub_rn((double)__ldg(x + i * d + t), means[t]));
        if (coords_t) coords_t[(int64_t)t * n_pad + i] = c;
        if (valid && t < d) {
            if (xcentred) xcentred[i * d + t] = c;
            acc = __fmaf_rn(c, c, acc);
        }
    }
    if (norm2) norm2[i] = valid ? acc : __int_as_float(0x7f800000);
    if (valid) {
        // sqrt rounded up by a relative 2^-20 so it bounds the true norm.
        float nrm = __fmul_ru(__fsqrt_ru(acc), 1.0f + 9.5367431640625e-07f);
        cnorm[i] = nrm;
        atomicMax(max_norm_bits, __float_as_uint(nrm));
    } else {
        cnorm[i] = 0.f;
    }
}

// Per-row candidate margin in s-space (s = |b|^2 - 2 a.b; the row's own |a|^2
// is a constant shift and cancels in every comparison made within the row).
//
// For every column j the computed s_ij differs from d_ij^2 - |a_i|^2 (d the
// distance between the caller's rows) by at most beta_i, so a column whose
// lower bound s - beta exceeds the k-th smallest upper bound s + beta cannot
// be among the k nearest: the margin is 2 * beta_i.  beta_i collects
//   plain form (FP32 fused dot, D terms):
//     (gamma_D + u) (M^2 + 2 |a| M)             expansion rounding, gamma_D = (D + 2) u
//     2.01 u (|a| + M)^2                        centring rounding of both rows
//   tensor form (16-bit operands, FP32 accumulate, scale 2^s applied):
//     2 (|e_a| M + |a| E + |e_a| E)             operand quantisation (exact error norms)
//     64 * 2^-24 (2 |a| M + M^2) + (gamma_D + u) M^2 + 2^-30 M^2   accumulation, norm split
//     2.01 u (|a| + M)^2                        centring
//   cosine adds 4.01 u + 1e-12 (f32 rounding of the normalised rows, FP64 noise);
//   reference-snap adds the snap floor ((D+2) 2u)(|a|^2 + M^2) and the
//   sequential chain's (D + 2) u (|a| + M)^2.
// M and E are the largest centred norm and quantisation error norm over all
// reference rows; u = 2^-24.  A 1.5x safety factor is applied.
__global__ void margins_kernel(const float* __restrict__ cnorm, const float* __restrict__ norm2,
                               int64_t n, int d, int mode, int metric, int form,
                               const uint32_t* __restrict__ max_norm_bits,
                               const float* __restrict__ qerr, const uint32_t* __restrict__ max_qerr_bits,
                               float scale2, float* __restrict__ margin) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double u = kUnit32;
    const double M = (double)__uint_as_float(*max_norm_bits);
    const double a = (double)cnorm[i];
    const double gammaD = (double)(d + 2) * u;
    double beta;
    if (form == SCRUST_FORM_PLAIN) {
        beta = (gammaD + u) * (M * M + 2.0 * a * M);
    } else {
        const double E = (double)__uint_as_float(*max_qerr_bits);
        const double ea = (double)qerr[i];
        beta = 2.0 * (ea * M + a * E + ea * E) + 64.0 * u * (2.0 * a * M + M * M) +
               (gammaD + u) * M * M + 9.313225746154785e-10 * M * M;
    }
    beta += 2.01 * u * (a + M) * (a + M);
    if (metric == SCRUST_METRIC_COSINE) beta += (4.01 * u + 1e-12) * (double)scale2;
    if (mode == SCRUST_MODE_REFERENCE_SNAP) {
        const double na = (double)norm2[i];
        beta += (double)(d + 2) * 2.0 * u * (na + M * M) + gammaD * (a + M) * (a + M);
    }
    margin[i] = __double2float_ru(2.0 * 1.5 * beta + 1e-30);
}

}  // namespace

cudaError_t launch_column_means(const float* x, int64_t n, int d, bool sequential, double* means,
                                double* partial, cudaStream_t s) {
    if (sequential) {
        means_sequential_kernel<<<(d + 63) / 64, 64, 0, s>>>(x, n, d, means);
        return cudaGetLastError();
    }
    int blocks = (int)((n + kMeanRowsPerBlock - 1) / kMeanRowsPerBlock);
    int threads = d >= 256 ? 256 : ((d + 31) / 32) * 32;
    means_partial_kernel<<<blocks, threads, 0, s>>>(x, n, d, partial);
    means_final_kernel<<<(d + 127) / 128, 128, 0, s>>>(partial, blocks, n, d, means);
    return cudaGetLastError();
}

namespace {

// Column means for the tensor form, where they only fix a centre (any
// centre serves, as long as every row and query is centred on the same
// one): f32 partial sums over 1024-row blocks, one warp per row at a time,
// then an f64 sum of the partials.  d <= 64.
constexpr int kMeanRowsF32 = 1024;
__global__ void __launch_bounds__(256) means_partial_f32_kernel(const float* __restrict__ x, int64_t n, int d,
                                                                float* __restrict__ partial) {
    __shared__ float acc_s[8][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.x * kMeanRowsF32;
    const int64_t r1 = min(n, r0 + kMeanRowsF32);
    float a0 = 0.f, a1 = 0.f;
    for (int64_t r = r0 + w; r < r1; r += 8) {
        if (lane < d) a0 += __ldg(x + r * d + lane);
        if (lane + 32 < d) a1 += __ldg(x + r * d + lane + 32);
    }
    acc_s[w][lane] = a0;
    acc_s[w][lane + 32] = a1;
    __syncthreads();
    if (threadIdx.x < d) {
        float t = 0.f;
        for (int q = 0; q < 8; ++q) t += acc_s[q][threadIdx.x];
        partial[(int64_t)blockIdx.x * d + threadIdx.x] = t;
    }
}

// One block of 256 threads per column: strided f32 sums of the partials,
// then a tree.
__global__ void __launch_bounds__(256) means_final_f32_kernel(const float* __restrict__ partial, int blocks,
                                                              int64_t n, int d, double* __restrict__ means) {
    __shared__ float ws[8];
    const int c = blockIdx.x;
    float t = 0.f;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) t += partial[(int64_t)b * d + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < 8; ++w) s += ws[w];
        means[c] = (double)s / (double)n;
    }
}

}  // namespace

// `partial` is the d * (ceil(n / 2048) + 1) doubles that launch_column_means
// takes; the f32 partials of 1024-row blocks fit in it.
cudaError_t launch_column_means_centre(const float* x, int64_t n, int d, double* means, double* partial,
                                       cudaStream_t s) {
    const int blocks = (int)((n + kMeanRowsF32 - 1) / kMeanRowsF32);
    means_partial_f32_kernel<<<blocks, 256, 0, s>>>(x, n, d, reinterpret_cast<float*>(partial));
    means_final_f32_kernel<<<d, 256, 0, s>>>(reinterpret_cast<const float*>(partial), blocks, n, d, means);
    return cudaGetLastError();
}

cudaError_t launch_normalise_rows(const float* x, int64_t n, int d, float* xn, double* norm64,
                                  int* d_err, cudaStream_t s) {
    normalise_rows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, n, d, xn, norm64, d_err);
    return cudaGetLastError();
}

// The largest norm of a row centred on the f32-rounded column means (as
// the tensor operands centre them), bounded from above; one warp per row,
// lanes over the coordinates (d <= 64).
__global__ void __launch_bounds__(256) max_centred_norm_kernel(const float* __restrict__ x, int64_t n, int d,
                                                               const double* __restrict__ means,
                                                               uint32_t* __restrict__ max_norm_bits) {
    __shared__ float m32[64];
    if (threadIdx.x < 64) m32[threadIdx.x] = threadIdx.x < d ? __double2float_rn(means[threadIdx.x]) : 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    float best = 0.f;
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
        float acc = 0.f;
        if (lane < d) {
            const float c = __fsub_rn(__ldg(x + r * d + lane), m32[lane]);
            acc = c * c;
        }
        if (lane + 32 < d) {
            const float c = __fsub_rn(__ldg(x + r * d + lane + 32), m32[lane + 32]);
            acc = __fmaf_rn(c, c, acc);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        best = fmaxf(best, acc);
    }
    if (lane == 0 && best > 0.f) {
        // A sum of d rounded non-negative terms, scaled past its rounding.
        const float grow = 1.0f + (float)(d + 4) * 1.1920929e-07f;
        atomicMax(max_norm_bits, __float_as_uint(__fmul_ru(__fsqrt_ru(__fmul_ru(best, grow)), 1.0f + 9.5367431640625e-07f)));
    }
}

cudaError_t launch_max_centred_norm(const float* x, int64_t n, int d, const double* means, uint32_t* max_norm_bits,
                                    int sm_count, cudaStream_t s) {
    const int64_t want = (n + 7) / 8;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count * 16));
    max_centred_norm_kernel<<<blocks, 256, 0, s>>>(x, n, d, means, max_norm_bits);
    return cudaGetLastError();
}

cudaError_t launch_centre_transpose(const float* x, int64_t n, int64_t n_pad, int d, int dp,
                                    const double* means, float* coords_t, float* norm2,
                                    float* cnorm, float* xcentred, uint32_t* max_norm_bits,
                                    cudaStream_t s) {
    centre_transpose_kernel<<<(unsigned)((n_pad + 255) / 256), 256, 0, s>>>(
        x, n, n_pad, d, dp, means, coords_t, norm2, cnorm, xcentred, max_norm_bits);
    return cudaGetLastError();
}

cudaError_t launch_margins(const float* cnorm, const float* norm2, int64_t n, int d, int mode,
                           int metric, int form, const uint32_t* max_norm_bits,
                           const float* qerr, const uint32_t* max_qerr_bits, float scale2,
                           float* margin, cudaStream_t s) {
    margins_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        cnorm, norm2, n, d, mode, metric, form, max_norm_bits, qerr, max_qerr_bits, scale2, margin);
    return cudaGetLastError();
}

}  // namespace scrust
