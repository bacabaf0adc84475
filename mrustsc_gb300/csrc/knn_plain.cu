// knn_plain.cu -- the plain form: FP32 tiled expansion distances on CUDA
// cores, fused with per-row candidate selection.
//
// Reference: the fused distance + top-k of the Metal kernel
// (crates/scrust-gpu/src/kernels/knn.rs:203-270) and the tiled expansion of
// crates/scrust-core/src/neighbors.rs:69-96.  Here a CTA owns 128 query rows
// and streams 128-column reference tiles through a two-stage TMA pipeline
// (boxes of [64 dims][128 rows] from the transposed centred coordinates).
// 256 threads each hold an 8x8 register tile of s = |b|^2 - 2 a.b.  A value
// below its row's threshold is appended to the row's candidate list in global
// memory; when a list reaches `cap` entries one warp prunes it: the k-th
// smallest value plus the row's margin becomes the new threshold, and entries
// above it are dropped.  The exact rerank later turns the lists into the
// neighbour rows.
#include "common.cuh"
#include "internal.h"
#include "lists.cuh"
#include "tma.cuh"

namespace scrust {

namespace {

constexpr int BM = 128, BN = 128, KC = 64, THREADS = 256;

struct PlainArgs {
    const float* r_norm2;
    const float* margin;
    Lists lists;
    int64_t nq;
    int nch;          // 64-dim chunks
    int dp;
    int kbox;         // dims per TMA box: min(64, dp)
    int k;
    int self;
    int col_tiles;
    int tiles_per_seg;
    int* err;
};

__global__ void __launch_bounds__(THREADS, 2)
    plain_candidates_kernel(const __grid_constant__ CUtensorMap tq, const __grid_constant__ CUtensorMap tr,
                            PlainArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const bool reload_a = a.nch > 1;
    float* sA[2];
    float* sB[2];
    sA[0] = (float*)base;
    sA[1] = reload_a ? sA[0] + KC * BM : sA[0];
    sB[0] = (reload_a ? sA[1] : sA[0]) + KC * BM;
    sB[1] = sB[0] + KC * BN;

    __shared__ __align__(8) uint64_t bars[3];
    __shared__ float thr_s[BM];
    __shared__ uint32_t cnt_s[BM];
    __shared__ float margin_s[BM];

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int warp = tid >> 5;
    const int64_t row0 = (int64_t)blockIdx.x * BM;
    const int seg = blockIdx.y;
    const int ct_begin = seg * a.tiles_per_seg;
    const int ct_end = min(a.col_tiles, ct_begin + a.tiles_per_seg);
    const int nsteps = (ct_end - ct_begin) * a.nch;

    if (tid == 0) {
        prefetch_tensormap(&tq);
        prefetch_tensormap(&tr);
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_init(&bars[2], 1);
        fence_barrier_init();
    }
    if (tid < BM) {
        const int64_t row = row0 + tid;
        const bool valid = row < a.nq;
        thr_s[tid] = valid ? __int_as_float(0x7f800000) : __int_as_float(0xff800000);
        cnt_s[tid] = 0;
        margin_s[tid] = valid ? a.margin[row] : 0.f;
    }
    __syncthreads();
    if (nsteps <= 0) {
        if (tid < BM && row0 + tid < a.nq) a.lists.cnt[(row0 + tid) * a.lists.segments + seg] = 0;
        return;
    }

    const uint32_t box_bytes = (uint32_t)a.kbox * BM * sizeof(float);
    auto issue = [&](int step) {
        const int st = step & 1;
        const int ct = ct_begin + step / a.nch;
        const int ch = step % a.nch;
        const uint32_t bytes = box_bytes * (reload_a ? 2u : 1u);
        mbar_arrive_expect_tx(&bars[st], bytes);
        if (reload_a) tma_load_2d(sA[st], &tq, (int)row0, ch * KC, &bars[st]);
        tma_load_2d(sB[st], &tr, ct * BN, ch * KC, &bars[st]);
    };
    if (tid == 0) {
        if (!reload_a) {
            mbar_arrive_expect_tx(&bars[2], box_bytes);
            tma_load_2d(sA[0], &tq, (int)row0, 0, &bars[2]);
        }
        issue(0);
    }
    if (!reload_a) {
        bool okA = mbar_wait_bounded(&bars[2], 0, a.err);
        if (__syncthreads_or(!okA)) return;
    }

    float acc[8][8];
    for (int step = 0; step < nsteps; ++step) {
        const int st = step & 1;
        const int ct = ct_begin + step / a.nch;
        const int ch = step % a.nch;
        if (tid == 0 && step + 1 < nsteps) issue(step + 1);
        bool okB = mbar_wait_bounded(&bars[st], (uint32_t)((step >> 1) & 1), a.err);
        if (__syncthreads_or(!okB)) return;

        if (ch == 0) {
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
        }
        const float* As = sA[reload_a ? st : 0];
        const float* Bs = sB[st];
        const int kc = min(KC, a.dp - ch * KC);
        for (int t = 0; t < kc; ++t) {
            const float4 a0 = *reinterpret_cast<const float4*>(As + t * BM + ty * 4);
            const float4 a1 = *reinterpret_cast<const float4*>(As + t * BM + 64 + ty * 4);
            const float4 b0 = *reinterpret_cast<const float4*>(Bs + t * BN + tx * 4);
            const float4 b1 = *reinterpret_cast<const float4*>(Bs + t * BN + 64 + tx * 4);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = __fmaf_rn(av[i], bv[j], acc[i][j]);
        }

        if (ch == a.nch - 1) {
            // Epilogue: s = |b|^2 - 2 a.b, threshold test, appends.
            const int64_t col0 = (int64_t)ct * BN;
            float nb[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int lc = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
                nb[j] = __ldg(a.r_norm2 + col0 + lc);
            }
            const bool diag = a.self && (col0 == row0);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int lr = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
                const float th = thr_s[lr];
                float s[8];
#pragma unroll
                for (int j = 0; j < 8; j++) s[j] = __fmaf_rn(-2.0f, acc[i][j], nb[j]);
                if (diag) {
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const int lc = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
                        if (lc == lr) s[j] = __int_as_float(0x7f800000);
                    }
                }
                const float m = fminf(min3f(s[0], s[1], s[2]), min3f(s[3], min3f(s[4], s[5], s[6]), s[7]));
                if (m < th) {
                    const int64_t lbase = ((row0 + lr) * a.lists.segments + seg) * (int64_t)a.lists.ctot;
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        if (s[j] < th) {
                            const int lc = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
                            uint32_t pos = atomicAdd(&cnt_s[lr], 1u);
                            if (pos < (uint32_t)a.lists.ctot) {
                                a.lists.ids[lbase + pos] = (uint32_t)(col0 + lc);
                                a.lists.vals[lbase + pos] = s[j];
                            }
                        }
                    }
                }
            }
            __syncthreads();
            // Prune every list that reached its capacity.
            for (int lr = warp * (BM / 8); lr < (warp + 1) * (BM / 8); ++lr) {
                uint32_t c = cnt_s[lr];
                if (c >= (uint32_t)a.lists.cap) {
                    const int64_t row = row0 + lr;
                    const int64_t lbase = (row * a.lists.segments + seg) * (int64_t)a.lists.ctot;
                    prune_list(a.lists.ids + lbase, a.lists.vals + lbase, min(c, (uint32_t)a.lists.ctot), a.k,
                               a.lists.cap, PlainBound{margin_s[lr]}, &thr_s[lr], &cnt_s[lr],
                               a.lists.overflow + row);
                }
            }
        }
        __syncthreads();
    }
    if (tid < BM) {
        const int64_t row = row0 + tid;
        if (row < a.nq)
            a.lists.cnt[row * a.lists.segments + seg] = min(cnt_s[tid], (uint32_t)a.lists.ctot);
    }
}

}  // namespace

size_t plain_smem_bytes(int dp) {
    const bool reload_a = dp > KC;
    return (size_t)(reload_a ? 4 : 3) * KC * BM * sizeof(float) + 1024;
}

cudaError_t launch_plain_candidates(scrust_context* ctx, const KnnPlan& plan, const float* q_t,
                                    int64_t nq_pad, const float* r_t, int64_t nr_pad, int dp,
                                    const float* r_norm2, const float* margin, const Lists& lists) {
    CUtensorMap tq, tr;
    // dp is a multiple of 4 up to 64 and a multiple of 64 beyond, so a box
    // of min(64, dp) dims never reaches past the tensor.
    if (dp > KC && dp % KC) return cudaErrorInvalidValue;
    const int kbox = dp < KC ? dp : KC;
    if (!encode_2d(ctx, &tq, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (void*)q_t, (uint64_t)nq_pad,
                   (uint64_t)dp, (uint64_t)nq_pad * sizeof(float), BM, (uint32_t)kbox,
                   CU_TENSOR_MAP_SWIZZLE_NONE))
        return cudaErrorInvalidValue;
    if (!encode_2d(ctx, &tr, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (void*)r_t, (uint64_t)nr_pad,
                   (uint64_t)dp, (uint64_t)nr_pad * sizeof(float), BN, (uint32_t)kbox,
                   CU_TENSOR_MAP_SWIZZLE_NONE))
        return cudaErrorInvalidValue;
    PlainArgs a;
    a.r_norm2 = r_norm2;
    a.margin = margin;
    a.lists = lists;
    a.nq = plan.nq;
    a.nch = (dp + KC - 1) / KC;
    a.dp = dp;
    a.kbox = kbox;
    a.k = plan.k;
    a.self = plan.self ? 1 : 0;
    a.col_tiles = (int)(nr_pad / BN);
    a.tiles_per_seg = (a.col_tiles + lists.segments - 1) / lists.segments;
    if ((a.col_tiles + a.tiles_per_seg - 1) / a.tiles_per_seg != lists.segments) return cudaErrorInvalidValue;
    a.err = ctx->d_err;
    const size_t smem = plain_smem_bytes(dp);
    cudaError_t e = set_smem_limit(ctx, (const void*)plain_candidates_kernel, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)(nq_pad / BM), (unsigned)lists.segments);
    plain_candidates_kernel<<<grid, THREADS, smem, ctx->stream>>>(tq, tr, a);
    return cudaGetLastError();
}

}  // namespace scrust
