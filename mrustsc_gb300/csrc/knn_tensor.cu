// knn_tensor.cu -- the tensor form: candidate generation as a 16-bit
// tcgen05 GEMM with FP32 accumulation in TMEM, fused with per-row candidate
// selection.  The exact rerank (rerank.cu) then turns the candidates into the
// same FP64-equal neighbour lists the plain form produces.
//
// Operands (K = 64 halves per row, one 128-byte swizzle row):
//   A_i = [ a_hat_i (D), 1, 1, 1, 0 ... ]
//   B_j = [ -2 b_hat_j (D), n1_j, n2_j, n3_j, 0 ... ]
// where a_hat = fp16/bf16(scale * (x - mean)) and n1 + n2 + n3 is
// |b_hat_j|^2 split into three 16-bit parts, so one MMA chain yields
// t_ij = |b_hat_j|^2 - 2 a_hat_i . b_hat_j = |a_hat_i - b_hat_j|^2 - |a_hat_i|^2.
// Because the norm is the quantised vector's own, the quantisation error of a
// pair's squared distance scales with the pair's distance, not with the
// norms (see TensorBound in lists.cuh).
//
// Kernel layout (persistent, one CTA per SM, 320 threads):
//   warp 0      TMA producer: A (256 query rows) per work item, B (256
//               reference rows) per tile, 4-stage ring
//   warp 1      TMEM owner and MMA issuer: per B tile, two M=128 x N=256 x
//               K=16 x4 chains into two TMEM accumulators (query halves)
//   warps 2-9   epilogue: warp w reads TMEM lanes 32*(w%4).. of half (w-2)/4;
//               each thread owns one query row, tests 32 columns at a time
//               against its threshold (3-input min), appends survivors to
//               its list and prunes full lists warp-cooperatively
// The two accumulators ping-pong: the epilogue drains half 0 of tile j while
// the tensor core computes half 1 of tile j, so each B tile is read once per
// 256 query rows.  Every wait is bounded (tma.cuh).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "lists.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace scrust {

namespace {

constexpr int TBM = 128;               // rows per accumulator (MMA M)
constexpr int TBN = 256;               // reference rows per tile (MMA N)
constexpr int TK = 64;                 // halves per operand row
constexpr int HALVES = 2;              // query halves per work item
constexpr int ROWS = TBM * HALVES;     // 256 query rows per work item
constexpr int STAGES = 4;
constexpr int EPI_WARPS = 8;
constexpr int THREADS = (2 + EPI_WARPS) * 32;
constexpr uint32_t A_BYTES = ROWS * TK * 2;
constexpr uint32_t B_BYTES = TBN * TK * 2;
constexpr uint32_t TMEM_COLS = 512;
constexpr size_t SMEM_BYTES = 2 * A_BYTES + STAGES * B_BYTES + 1024;

struct TensorArgs {
    Lists lists;
    const float* bA;
    const float* bdelta;
    const float* beps2;
    int64_t nq, nr;
    int k;
    int self;
    int col_tiles;
    int tiles_per_seg;
    int items;
    uint32_t idesc;
    int* err;
};

__device__ __forceinline__ float f_of(uint32_t u) { return __uint_as_float(u); }

__device__ __forceinline__ float min32(const uint32_t (&v)[32]) {
    float m[11];
#pragma unroll
    for (int i = 0; i < 10; i++) m[i] = min3f(f_of(v[3 * i]), f_of(v[3 * i + 1]), f_of(v[3 * i + 2]));
    m[10] = fminf(f_of(v[30]), f_of(v[31]));
    const float a = min3f(m[0], m[1], m[2]);
    const float b = min3f(m[3], m[4], m[5]);
    const float c = min3f(m[6], m[7], m[8]);
    const float d = fminf(m[9], m[10]);
    return fminf(min3f(a, b, c), d);
}

// Appends the columns of one 32-column chunk that pass the row's threshold.
__device__ __forceinline__ void append_chunk(const uint32_t (&v)[32], int64_t colbase, float th, int64_t row,
                                             const TensorArgs& a, uint32_t* ids, float* vals, uint32_t& cnt) {
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const float t = f_of(v[j]);
        const int64_t col = colbase + j;
        if (t < th && col < a.nr && !(a.self && col == row)) {
            ids[cnt] = (uint32_t)col;
            vals[cnt] = t;
            cnt++;
        }
    }
}

__global__ void __launch_bounds__(THREADS, 1)
    tensor_candidates_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                             TensorArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = base;
    unsigned char* sB = base + 2 * A_BYTES;

    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], afull[2], aempty[2], tfull[HALVES],
        tempty[HALVES];
    __shared__ uint32_t tmem_slot;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int segs = a.lists.segments;

    if (threadIdx.x == 0) {
        prefetch_tensormap(&ta);
        prefetch_tensormap(&tb);
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&afull[b], 1);
            mbar_init(&aempty[b], 1);
        }
        for (int h = 0; h < HALVES; h++) {
            mbar_init(&tfull[h], 1);
            mbar_init(&tempty[h], 32 * (EPI_WARPS / HALVES));
        }
        fence_barrier_init();
    }
    if (warp == 1) {
        tmem_alloc(&tmem_slot, TMEM_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t sc = 0, ac = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < a.items && ok; w += gridDim.x) {
                const int qt = w / segs, seg = w % segs;
                const int ct0 = seg * a.tiles_per_seg;
                const int ct1 = min(a.col_tiles, ct0 + a.tiles_per_seg);
                const uint32_t ab = ac & 1, au = ac >> 1;
                if (!mbar_wait_bounded(&aempty[ab], (au & 1) ^ 1, a.err)) {
                    ok = false;
                    break;
                }
                mbar_arrive_expect_tx(&afull[ab], A_BYTES);
                tma_load_2d(sA + ab * A_BYTES, &ta, 0, qt * ROWS, &afull[ab]);
                ac++;
                for (int ct = ct0; ct < ct1; ++ct) {
                    const uint32_t st = sc % STAGES, su = sc / STAGES;
                    if (!mbar_wait_bounded(&empty[st], (su & 1) ^ 1, a.err)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&full[st], B_BYTES);
                    tma_load_2d(sB + st * B_BYTES, &tb, 0, ct * TBN, &full[st]);
                    sc++;
                }
            }
            // Copies still in flight complete on their barriers; wait for the
            // most recent phase of every stage (bounded) before leaving.
            for (uint32_t i = 0; i < STAGES && i < sc; i++) {
                const uint32_t idx = sc - 1 - i;
                mbar_wait_bounded(&full[idx % STAGES], (idx / STAGES) & 1, a.err, 100000000ull);
            }
            if (ac) mbar_wait_bounded(&afull[(ac - 1) & 1], ((ac - 1) >> 1) & 1, a.err, 100000000ull);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t sc = 0, ac = 0, tc = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < a.items && ok; w += gridDim.x) {
                const int seg = w % segs;
                const int ct0 = seg * a.tiles_per_seg;
                const int ct1 = min(a.col_tiles, ct0 + a.tiles_per_seg);
                const uint32_t ab = ac & 1, au = ac >> 1;
                if (!mbar_wait_bounded(&afull[ab], au & 1, a.err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a_base = smem_addr(sA + ab * A_BYTES);
                for (int ct = ct0; ct < ct1 && ok; ++ct) {
                    const uint32_t st = sc % STAGES, su = sc / STAGES;
                    if (!mbar_wait_bounded(&full[st], su & 1, a.err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t b_base = smem_addr(sB + st * B_BYTES);
                    for (int h = 0; h < HALVES; ++h) {
                        if (!mbar_wait_bounded(&tempty[h], (tc & 1) ^ 1, a.err)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t d = tmem + (uint32_t)(h * TBN);
#pragma unroll
                        for (int kk = 0; kk < TK / 16; ++kk) {
                            const uint64_t ad = umma_desc_sw128(a_base + (uint32_t)(h * TBM * 128 + kk * 32));
                            const uint64_t bd = umma_desc_sw128(b_base + (uint32_t)(kk * 32));
                            umma_f16(d, ad, bd, a.idesc, kk > 0 ? 1u : 0u);
                        }
                        umma_commit(&tfull[h]);
                    }
                    if (!ok) break;
                    umma_commit(&empty[st]);
                    sc++;
                    tc++;
                }
                if (!ok) break;
                umma_commit(&aempty[ab]);
                ac++;
            }
        }
    } else {
        // ---------------- epilogue ----------------
        const int e = warp - 2;
        const int h = e / (EPI_WARPS / HALVES);
        const int quarter = warp & 3;
        const int r_local = quarter * 32 + lane;
        const int cap = a.lists.cap;
        uint32_t tc = 0;
        bool ok = true;
        for (int w = blockIdx.x; w < a.items && ok; w += gridDim.x) {
            const int qt = w / segs, seg = w % segs;
            const int ct0 = seg * a.tiles_per_seg;
            const int ct1 = min(a.col_tiles, ct0 + a.tiles_per_seg);
            const int64_t row = (int64_t)qt * ROWS + h * TBM + r_local;
            const bool valid = row < a.nq;
            float th = valid ? __int_as_float(0x7f800000) : __int_as_float(0xff800000);
            uint32_t cnt = 0;
            TensorBound bnd{0.f, 0.f, 0.f};
            if (valid) bnd = TensorBound{a.bA[row], a.bdelta[row], a.beps2[row]};
            const int64_t lbase = (row * segs + seg) * (int64_t)a.lists.ctot;
            uint32_t* ids = a.lists.ids + lbase;
            float* vals = a.lists.vals + lbase;
            for (int ct = ct0; ct < ct1; ++ct) {
                if (!mbar_wait_bounded(&tfull[h], tc & 1, a.err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int64_t col0 = (int64_t)ct * TBN;
                const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(h * TBN);
#pragma unroll 1
                for (int c2 = 0; c2 < TBN / 64; ++c2) {
                    uint32_t v0[32], v1[32];
                    tmem_ld32(tbase + c2 * 64, v0);
                    tmem_ld32(tbase + c2 * 64 + 32, v1);
                    tmem_ld_wait2(v0, v1);
                    if (min32(v0) < th) append_chunk(v0, col0 + c2 * 64, th, row, a, ids, vals, cnt);
                    if (min32(v1) < th) append_chunk(v1, col0 + c2 * 64 + 32, th, row, a, ids, vals, cnt);
                    uint32_t need = __ballot_sync(0xffffffffu, cnt >= (uint32_t)cap);
                    while (need) {
                        const int l = __ffs(need) - 1;
                        need &= need - 1;
                        const uint32_t lc = __shfl_sync(0xffffffffu, cnt, l);
                        const float lth = __shfl_sync(0xffffffffu, th, l);
                        const TensorBound lb{__shfl_sync(0xffffffffu, bnd.A, l),
                                             __shfl_sync(0xffffffffu, bnd.delta, l),
                                             __shfl_sync(0xffffffffu, bnd.eps2, l)};
                        const int64_t lrow = __shfl_sync(0xffffffffu, row, l);
                        const int64_t lb_off = (lrow * segs + seg) * (int64_t)a.lists.ctot;
                        const PruneResult r = prune_core(a.lists.ids + lb_off, a.lists.vals + lb_off,
                                                         min(lc, (uint32_t)a.lists.ctot), a.k, lb, lth);
                        if (lane == l) {
                            if ((int)r.cnt >= cap) {
                                a.lists.overflow[row] = 1u;
                                th = __int_as_float(0xff800000);
                                cnt = 0;
                            } else {
                                th = r.theta;
                                cnt = r.cnt;
                            }
                        }
                    }
                }
                tc_fence_before();
                mbar_arrive(&tempty[h]);
                tc++;
            }
            if (valid && ok) a.lists.cnt[row * segs + seg] = min(cnt, (uint32_t)a.lists.ctot);
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ---- operand preparation ---------------------------------------------------------

template <class T>
__device__ __forceinline__ T to16(float v);
template <>
__device__ __forceinline__ __half to16<__half>(float v) {
    return __float2half_rn(v);
}
template <>
__device__ __forceinline__ __nv_bfloat16 to16<__nv_bfloat16>(float v) {
    return __float2bfloat16_rn(v);
}
__device__ __forceinline__ double f64_of(__half v) { return (double)__half2float(v); }
__device__ __forceinline__ double f64_of(__nv_bfloat16 v) { return (double)__bfloat162float(v); }

// One thread per padded row: writes A_i and B_i (64 16-bit values each), the
// quantised squared norm A = |a_hat|^2, the per-row error radius
// eps = |a_hat - scale*c| + scale*u*|c| (+ scale*u for normalised rows), and
// the running maxima of eps and |b_hat|.
template <class T>
__global__ void tensor_operands_kernel(const float* __restrict__ x, int64_t n, int64_t n_pad, int d,
                                       const double* __restrict__ means, const uint32_t* __restrict__ max_norm_bits,
                                       int cosine, T* __restrict__ A16, T* __restrict__ B16,
                                       float* __restrict__ bA, float* __restrict__ eps,
                                       uint32_t* __restrict__ max_eps_bits, uint32_t* __restrict__ max_bhat_bits) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    const float M = __uint_as_float(*max_norm_bits);
    // Power-of-two scale so every |scale * c| <= 64 (and |b_hat|^2 < 65504).
    int sexp = M > 0.f ? (int)floorf(log2f(64.0f / M)) : 0;
    sexp = max(-100, min(100, sexp));
    const float scale = ldexpf(1.0f, sexp);
    __align__(16) T arow[TK];
    __align__(16) T brow[TK];
    const T zero = to16<T>(0.f);
#pragma unroll
    for (int t = 0; t < TK; t++) {
        arow[t] = zero;
        brow[t] = zero;
    }
    if (i < n) {
        double hh = 0.0, e2 = 0.0, c2 = 0.0;
        for (int t = 0; t < d; t++) {
            const float c = __double2float_rn(__dsub_rn((double)__ldg(x + i * d + t), means[t]));
            const float y = c * scale;
            const T q = to16<T>(y);
            const double qd = f64_of(q);
            arow[t] = q;
            brow[t] = to16<T>(-2.0f * (float)qd);
            hh += qd * qd;
            const double err = qd - (double)y;
            e2 += err * err;
            c2 += (double)c * (double)c;
        }
        const T one = to16<T>(1.0f);
        arow[d] = one;
        arow[d + 1] = one;
        arow[d + 2] = one;
        const T n1 = to16<T>((float)hh);
        const double r1 = hh - f64_of(n1);
        const T n2 = to16<T>((float)r1);
        const double r2 = r1 - f64_of(n2);
        const T n3 = to16<T>((float)r2);
        brow[d] = n1;
        brow[d + 1] = n2;
        brow[d + 2] = n3;
        bA[i] = (float)hh;
        double ep = sqrt(e2) + 1.01 * (double)scale * kUnit32 * sqrt(c2);
        if (cosine) ep += 1.01 * (double)scale * kUnit32;
        ep += 1e-30;
        const float epf = __double2float_ru(ep);
        eps[i] = epf;
        atomicMax(max_eps_bits, __float_as_uint(epf));
        atomicMax(max_bhat_bits, __float_as_uint(__double2float_ru(sqrt(hh))));
    } else {
        bA[i] = 0.f;
        eps[i] = 0.f;
    }
    uint4* ad = reinterpret_cast<uint4*>(A16 + i * TK);
    uint4* bd = reinterpret_cast<uint4*>(B16 + i * TK);
    const uint4* as = reinterpret_cast<const uint4*>(arow);
    const uint4* bs = reinterpret_cast<const uint4*>(brow);
#pragma unroll
    for (int t = 0; t < TK * 2 / 16; t++) {
        ad[t] = as[t];
        bd[t] = bs[t];
    }
}

// delta: bound on the FP32 accumulation error of the 64-term MMA chain,
// 8 * 64 * 2^-24 * (2 |a_hat| Mb + Mb^2 + 3), plus the rounding of A to f32
// and the residual of the three-part 16-bit split of |b_hat|^2 (at most
// 2^-24 |b_hat|^2 for bf16 parts, far less for fp16); eps2 = 2 (eps_i + E).
__global__ void tensor_bounds_kernel(int64_t n, const float* __restrict__ bA, const float* __restrict__ eps,
                                     const uint32_t* __restrict__ max_eps_bits,
                                     const uint32_t* __restrict__ max_bhat_bits, float* __restrict__ bdelta,
                                     float* __restrict__ beps2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double Mb = (double)__uint_as_float(*max_bhat_bits);
    const double E = (double)__uint_as_float(*max_eps_bits);
    const double A = (double)bA[i];
    const double a = sqrt(A);
    const double delta = 8.0 * 64.0 * kUnit32 * (2.0 * a * Mb + Mb * Mb + 3.0) + 2.0 * kUnit32 * A +
                         4.0 * kUnit32 * Mb * Mb + 1e-7;
    bdelta[i] = __double2float_ru(delta);
    beps2[i] = __double2float_ru(2.0 * ((double)eps[i] + E));
}

}  // namespace

size_t tensor_smem_bytes() { return SMEM_BYTES; }

cudaError_t launch_tensor_operands(const float* x, int64_t n, int64_t n_pad, int d, const double* means,
                                   const uint32_t* max_norm_bits, bool cosine, bool bf16, void* A16, void* B16,
                                   float* bA, float* eps, uint32_t* max_eps_bits, uint32_t* max_bhat_bits,
                                   cudaStream_t s) {
    const unsigned blocks = (unsigned)((n_pad + 127) / 128);
    if (bf16)
        tensor_operands_kernel<__nv_bfloat16><<<blocks, 128, 0, s>>>(
            x, n, n_pad, d, means, max_norm_bits, cosine ? 1 : 0, (__nv_bfloat16*)A16, (__nv_bfloat16*)B16, bA,
            eps, max_eps_bits, max_bhat_bits);
    else
        tensor_operands_kernel<__half><<<blocks, 128, 0, s>>>(x, n, n_pad, d, means, max_norm_bits,
                                                              cosine ? 1 : 0, (__half*)A16, (__half*)B16, bA, eps,
                                                              max_eps_bits, max_bhat_bits);
    return cudaGetLastError();
}

cudaError_t launch_tensor_bounds(int64_t n, const float* bA, const float* eps, const uint32_t* max_eps_bits,
                                 const uint32_t* max_bhat_bits, float* bdelta, float* beps2, cudaStream_t s) {
    tensor_bounds_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, bA, eps, max_eps_bits, max_bhat_bits,
                                                                      bdelta, beps2);
    return cudaGetLastError();
}

cudaError_t launch_tensor_candidates(scrust_context* ctx, const KnnPlan& plan, const void* A16, int64_t nq_pad,
                                     const void* B16, int64_t nr_pad, const float* bA, const float* bdelta,
                                     const float* beps2, const Lists& lists, bool bf16, int* grid_out) {
    if (nq_pad % ROWS || nr_pad % TBN) return cudaErrorInvalidValue;
    CUtensorMap ta, tb;
    const CUtensorMapDataType dt = bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    if (!encode_2d(ctx, &ta, dt, (void*)A16, TK, (uint64_t)nq_pad, TK * 2, TK, ROWS, CU_TENSOR_MAP_SWIZZLE_128B))
        return cudaErrorInvalidValue;
    if (!encode_2d(ctx, &tb, dt, (void*)B16, TK, (uint64_t)nr_pad, TK * 2, TK, TBN, CU_TENSOR_MAP_SWIZZLE_128B))
        return cudaErrorInvalidValue;
    TensorArgs a;
    a.lists = lists;
    a.bA = bA;
    a.bdelta = bdelta;
    a.beps2 = beps2;
    a.nq = plan.nq;
    a.nr = plan.nr;
    a.k = plan.k;
    a.self = plan.self ? 1 : 0;
    a.col_tiles = (int)(nr_pad / TBN);
    a.tiles_per_seg = (a.col_tiles + lists.segments - 1) / lists.segments;
    if ((a.col_tiles + a.tiles_per_seg - 1) / a.tiles_per_seg != lists.segments) return cudaErrorInvalidValue;
    if (lists.ctot < lists.cap + 64 || lists.ctot > 32 * kListMaxEntriesPerLane) return cudaErrorInvalidValue;
    a.items = (int)(nq_pad / ROWS) * lists.segments;
    a.idesc = umma_idesc_f16(TBM, TBN, bf16);
    a.err = ctx->d_err;
    cudaError_t e =
        cudaFuncSetAttribute(tensor_candidates_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (e != cudaSuccess) return e;
    const int grid = std::min(a.items, ctx->sm_count);
    if (grid_out) *grid_out = grid;
    tensor_candidates_kernel<<<grid, THREADS, SMEM_BYTES, ctx->stream>>>(ta, tb, a);
    return cudaGetLastError();
}

}  // namespace scrust
