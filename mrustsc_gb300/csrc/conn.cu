// conn.cu -- UMAP connectivities on the device, following
// crates/scrust-core/src/neighbors.rs:208-372:
//   smooth_knn_distances (:239-298)  one thread per row: rho, the 64-step f32
//                                    bisection with f64 tolerance test, sigma floor
//   directed_weights (:300-327)      one thread per row, sorted by column
//   symmetrise (:329-372)            transpose by a stable LSD radix sort of the
//                                    directed edges keyed by target row, then a
//                                    per-row sorted merge with (w + r) - (w * r)
// Every f32 operation is written with explicit round-to-nearest intrinsics so
// nothing is contracted into an fma, matching the reference's uncontracted Rust
// arithmetic; exp is CUDA's expf.  Sums of a row use ndarray 0.16.1's
// unrolled_fold order (crates/scrust-core/src/neighbors.rs:248,290), the global
// mean included (unrolled_mean_kernel).
#include <math.h>

#include <algorithm>
#include <utility>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

// ndarray 0.16.1 numeric_util::unrolled_fold with f32 addition.
__device__ float unrolled_sum(const float* xs, int len) {
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

__global__ void check_ids_kernel(const uint32_t* __restrict__ idx, int64_t total, int64_t n, int* err) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x)
        if ((int64_t)idx[i] >= n) atomicExch(err + DERR_BAD_INDEX, 1);
}

// The global mean distance of crates/scrust-core/src/neighbors.rs:248,
// `distances.sum() / (n * k) as f32`, in the reference's own rounding: ndarray
// 0.16.1 sums a contiguous array with unrolled_fold, eight sequential f32
// chains over the elements i = j (mod 8) of the first 8 * floor(len / 8),
// combined as ((p0+p4), (p1+p5), (p2+p6), (p3+p7)) into the accumulator, then
// the tail added in order.  Eight dependent chains cannot be split without
// changing the rounding, so one block runs them: lanes 0..7 of warp 0 add
// from shared memory while the other warps stage the next tile.
constexpr int FOLD_THREADS = 256;
constexpr int FOLD_TILE = 8192;  // floats per staged tile; two tiles of shared memory
constexpr size_t FOLD_SMEM_BYTES = sizeof(float) * 2 * FOLD_TILE;

__device__ __forceinline__ void fold_stage(const float* __restrict__ x, int64_t t0, int cnt, float* dst, int tid,
                                           int nthreads, bool vec) {
    if (vec) {
        const int c4 = cnt >> 2;
        const float4* src = reinterpret_cast<const float4*>(x + t0);
        float4* d4 = reinterpret_cast<float4*>(dst);
        for (int i = tid; i < c4; i += nthreads) d4[i] = __ldg(src + i);
        for (int i = (c4 << 2) + tid; i < cnt; i += nthreads) dst[i] = __ldg(x + t0 + i);
    } else {
        for (int i = tid; i < cnt; i += nthreads) dst[i] = __ldg(x + t0 + i);
    }
}

__global__ void __launch_bounds__(FOLD_THREADS) unrolled_mean_kernel(const float* __restrict__ x, int64_t len,
                                                                     float* __restrict__ mean) {
    extern __shared__ float fold_buf[];  // 2 * FOLD_TILE
    const int tid = threadIdx.x;
    const int64_t body = len & ~(int64_t)7;
    const int64_t tiles = (body + FOLD_TILE - 1) / FOLD_TILE;
    const bool vec = (reinterpret_cast<uintptr_t>(x) & 15) == 0;
    float p = 0.f;  // chain tid of the fold (lanes 0..7 of warp 0)
    if (tiles > 0) fold_stage(x, 0, (int)min((int64_t)FOLD_TILE, body), fold_buf, tid, FOLD_THREADS, vec);
    __syncthreads();
    for (int64_t t = 0; t < tiles; ++t) {
        const float* cur = fold_buf + (t & 1) * FOLD_TILE;
        const int cnt = (int)min((int64_t)FOLD_TILE, body - t * FOLD_TILE);
        if (tid >= 32) {
            if (t + 1 < tiles)
                fold_stage(x, (t + 1) * FOLD_TILE, (int)min((int64_t)FOLD_TILE, body - (t + 1) * FOLD_TILE),
                           fold_buf + ((t + 1) & 1) * FOLD_TILE, tid - 32, FOLD_THREADS - 32, vec);
        } else if (tid < 8) {
            // cnt is a multiple of 8: FOLD_TILE is, and so is body.
#pragma unroll 8
            for (int j = tid; j < cnt; j += 8) p = __fadd_rn(p, cur[j]);
        }
        __syncthreads();
    }
    if (tid < 32) {
        const float q = __shfl_down_sync(0xffffffffu, p, 4);  // lane j < 4 gets p_{j+4}
        const float pair = __fadd_rn(p, q);
        float acc = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) acc = __fadd_rn(acc, __shfl_sync(0xffffffffu, pair, j));
        if (tid == 0) {
            for (int64_t i = body; i < len; ++i) acc = __fadd_rn(acc, x[i]);
            *mean = __fdiv_rn(acc, __ll2float_rn(len));
        }
    }
}

__global__ void smooth_knn_kernel(const float* __restrict__ dist, int64_t n, int k, double target,
                                  const float* __restrict__ mean, float* __restrict__ sigmas,
                                  float* __restrict__ rhos) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* row = dist + i * k;
    float rho = 0.f;
    for (int j = 0; j < k; j++) {
        float v = row[j];
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
            float offset = __fsub_rn(row[j], rho);
            float term = offset > 0.f ? expf(__fdiv_rn(-offset, mid)) : 1.0f;
            card = __fadd_rn(card, term);
        }
        double c64 = (double)card;
        if (fabs(c64 - target) < 1e-5) break;
        if (c64 > target) {
            high = mid;
            mid = __fdiv_rn(__fadd_rn(low, high), 2.0f);
        } else {
            low = mid;
            mid = high >= fmax ? __fmul_rn(mid, 2.0f) : __fdiv_rn(__fadd_rn(low, high), 2.0f);
        }
    }
    // Only rows whose neighbours all sit at distance 0 use the global mean;
    // their weights are 1 whatever sigma is, so callers that report no sigma
    // pass no mean (such a row's sigma is then the bisection's last mid).
    float reference = rho > 0.f ? __fdiv_rn(unrolled_sum(row, k), (float)(k + 1)) : (mean ? *mean : 0.f);
    sigmas[i] = fmaxf(mid, __fmul_rn(1e-3f, reference));
    rhos[i] = rho;
}

// Directed weights of one row, sorted by column (a stable insertion sort in
// the row's own output slots, so equal columns keep their input order); also
// emits the row's k edge slots for the transpose sort (invalid slots keyed
// past n so they sort last).
__global__ void directed_kernel(const uint32_t* __restrict__ idx, const float* __restrict__ dist,
                                int64_t n, int k, const float* __restrict__ sigmas,
                                const float* __restrict__ rhos, uint32_t* __restrict__ dcol,
                                float* __restrict__ dw, uint32_t* __restrict__ dcnt,
                                uint32_t* __restrict__ ekey, unsigned long long* __restrict__ eval) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // Rows of up to 32 neighbours are sorted in thread-local storage; wider
    // rows in place in dcol/dw.
    uint32_t lcol[32];
    float lw[32];
    const bool local = k <= 32;
    uint32_t* col = local ? lcol : dcol + i * k;
    float* w = local ? lw : dw + i * k;
    int m = 0;
    const float sigma = sigmas[i], rho = rhos[i];
    for (int j = 0; j < k; j++) {
        const uint32_t nb = idx[i * k + j];
        if ((int64_t)nb == i) continue;
        const float offset = __fsub_rn(dist[i * k + j], rho);
        const float wt = (offset <= 0.f || sigma == 0.f) ? 1.0f : expf(__fdiv_rn(-offset, sigma));
        if (wt == 0.f) continue;
        int s = m;
        while (s > 0 && col[s - 1] > nb) {
            col[s] = col[s - 1];
            w[s] = w[s - 1];
            s--;
        }
        col[s] = nb;
        w[s] = wt;
        m++;
    }
    dcnt[i] = (uint32_t)m;
    for (int t = 0; t < k; t++) {
        const int64_t slot = i * k + t;
        if (t < m) {
            if (local) {
                dcol[slot] = col[t];
                dw[slot] = w[t];
            }
            ekey[slot] = col[t];
            eval[slot] = ((unsigned long long)(uint32_t)i << 32) | __float_as_uint(w[t]);
        } else {
            ekey[slot] = (uint32_t)n;
            eval[slot] = 0ull;
        }
    }
}

// directed_kernel for k <= G (G = 16 or 32): G lanes per row, one neighbour
// each.  A lane's place in the sorted row is the number of the row's kept
// entries before it in (column, input position) order, found with G
// shuffles; the same weights, the same stable order, no local memory.
template <int G>
__global__ void __launch_bounds__(256) directed_group_kernel(const uint32_t* __restrict__ idx,
                                                             const float* __restrict__ dist, int64_t n, int k,
                                                             const float* __restrict__ sigmas,
                                                             const float* __restrict__ rhos,
                                                             uint32_t* __restrict__ dcol, float* __restrict__ dw,
                                                             uint32_t* __restrict__ dcnt,
                                                             uint32_t* __restrict__ ekey,
                                                             unsigned long long* __restrict__ eval) {
    const int lane = threadIdx.x & 31;
    const int g = lane / G, j = lane % G;
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const bool row_ok = i < n;
    uint32_t nb = 0;
    float wt = 0.f;
    bool kept = false;
    if (row_ok && j < k) {
        nb = idx[i * k + j];
        if ((int64_t)nb != i) {
            const float sigma = sigmas[i], rho = rhos[i];
            const float offset = __fsub_rn(dist[i * k + j], rho);
            wt = (offset <= 0.f || sigma == 0.f) ? 1.0f : expf(__fdiv_rn(-offset, sigma));
            kept = wt != 0.f;
        }
    }
    const unsigned long long key = kept ? ((unsigned long long)nb << 32) | (uint32_t)j : ~0ull;
    int rank = 0;
#pragma unroll
    for (int o = 0; o < G; ++o) rank += __shfl_sync(0xffffffffu, key, g * G + o) < key;
    const uint32_t group_bits = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (G * g));
    const int m = __popc(__ballot_sync(0xffffffffu, kept) & group_bits);
    if (!row_ok) return;
    if (j == 0) dcnt[i] = (uint32_t)m;
    if (kept) {
        const int64_t slot = i * k + rank;
        dcol[slot] = nb;
        dw[slot] = wt;
        ekey[slot] = nb;
        eval[slot] = ((unsigned long long)(uint32_t)i << 32) | __float_as_uint(wt);
    }
    if (j < k && j >= m) {  // unused slots sort last
        ekey[i * k + j] = (uint32_t)n;
        eval[i * k + j] = 0ull;
    }
}

// directed_group_kernel for graphs whose rows hold distinct ids (every kNN
// graph this library builds): the same weights and sorted rows, and for the
// transpose each kept edge takes its place in its target row's bucket with one
// atomic increment of that row's in-degree (the order inside a bucket is
// arbitrary; the merge kernels order it by source row, which is unique there).
template <int G>
__global__ void __launch_bounds__(256) directed_bucket_kernel(const uint32_t* __restrict__ idx,
                                                              const float* __restrict__ dist, int64_t n, int k,
                                                              const float* __restrict__ sigmas,
                                                              const float* __restrict__ rhos,
                                                              uint32_t* __restrict__ dcol, float* __restrict__ dw,
                                                              uint32_t* __restrict__ dcnt,
                                                              uint32_t* __restrict__ indeg,
                                                              uint32_t* __restrict__ erank) {
    const int lane = threadIdx.x & 31;
    const int g = lane / G, j = lane % G;
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const bool row_ok = i < n;
    uint32_t nb = 0;
    float wt = 0.f;
    bool kept = false;
    if (row_ok && j < k) {
        nb = idx[i * k + j];
        if ((int64_t)nb != i) {
            const float sigma = sigmas[i], rho = rhos[i];
            const float offset = __fsub_rn(dist[i * k + j], rho);
            wt = (offset <= 0.f || sigma == 0.f) ? 1.0f : expf(__fdiv_rn(-offset, sigma));
            kept = wt != 0.f;
        }
    }
    const unsigned long long key = kept ? ((unsigned long long)nb << 32) | (uint32_t)j : ~0ull;
    int rank = 0;
#pragma unroll
    for (int o = 0; o < G; ++o) rank += __shfl_sync(0xffffffffu, key, g * G + o) < key;
    const uint32_t group_bits = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (G * g));
    const int m = __popc(__ballot_sync(0xffffffffu, kept) & group_bits);
    if (!row_ok) return;
    if (j == 0) dcnt[i] = (uint32_t)m;
    if (kept) {
        const int64_t slot = i * k + rank;
        dcol[slot] = nb;
        dw[slot] = wt;
        erank[slot] = atomicAdd(indeg + nb, 1u);
    }
}

// Each kept edge (i -> c, w) into its target row's bucket:
// tval[tstart[c] + rank] = i << 32 | bits(w).
__global__ void bucket_scatter_kernel(const uint32_t* __restrict__ dcol, const float* __restrict__ dw,
                                      const uint32_t* __restrict__ dcnt, const uint32_t* __restrict__ erank,
                                      const uint32_t* __restrict__ tstart, int64_t n, int k,
                                      unsigned long long* __restrict__ tval) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n * k) return;
    const int64_t i = s / k;
    const int t = (int)(s - i * k);
    if (t >= (int)dcnt[i]) return;
    const uint32_t c = dcol[s];
    tval[(int64_t)tstart[c] + erank[s]] = ((unsigned long long)(uint32_t)i << 32) | __float_as_uint(dw[s]);
}

// Ascending sort of one bucket in place by one warp (a bitonic network whose
// merges all run ascending, with positions past `len` read as +infinity, so
// any length works).  Keys are source << 32 | weight bits, sources unique.
__device__ void warp_sort_bucket(unsigned long long* v, uint32_t len) {
    const int lane = threadIdx.x & 31;
    uint32_t p2 = 1;
    while (p2 < len) p2 <<= 1;
    for (uint32_t size = 2; size <= p2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = lane; t < p2 / 2; t += 32) {
                // pair (a, b), a < b: the first stage of a merge compares
                // mirror positions, the later ones positions `stride` apart
                const uint32_t block = t / stride, off = t % stride;
                uint32_t a, b;
                if (stride == (size >> 1)) {
                    const uint32_t base = (t / (size >> 1)) * size;
                    a = base + (t % (size >> 1));
                    b = base + size - 1 - (t % (size >> 1));
                } else {
                    a = block * 2 * stride + off;
                    b = a + stride;
                }
                if (b < len) {
                    const unsigned long long x = v[a], y = v[b];
                    if (y < x) {
                        v[a] = y;
                        v[b] = x;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// The fuzzy union of row i, one warp per row, for graphs with distinct ids
// per row, k <= 32 and n < 2^31.  The row's directed entries (nf, sorted by
// column) and its bucket of incoming edges (nb, sources unique, any order)
// are keyed column << 1 | direction and sorted together across the warp
// (32 or 64 positions, position lane + 32 r in register r), so an edge
// present in both directions becomes a directed entry followed by its
// incoming twin: the pair merges into (w + r) - (w * r), every other entry
// keeps its weight.  The merged row goes, compacted, to the row's scratch run
// at i * k + start[i] (room for k + nb entries) and its length to rowcnt[i];
// merge_place_kernel then copies the runs into the CSR.  Rows with more than
// 64 entries in all sort their bucket in place and place every entry by
// binary search.  Rows [r0, r1) only.
__device__ __forceinline__ uint32_t mask_below(int c) { return c >= 32 ? 0xffffffffu : ((1u << c) - 1u); }

template <int P>
__device__ __forceinline__ int union_sorted_row(const uint32_t* __restrict__ dcol, const float* __restrict__ dw,
                                                const unsigned long long* __restrict__ tval, int64_t i, int k,
                                                int nf, uint32_t b0, int nb, uint32_t* __restrict__ scol,
                                                float* __restrict__ sval) {
    constexpr int R = P / 32;
    const int lane = threadIdx.x & 31;
    uint32_t key[R];
    float w[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int p = lane + 32 * r;
        key[r] = 0xffffffffu;
        w[r] = 0.f;
        if (p < nf) {
            key[r] = dcol[i * k + p] << 1;
            w[r] = dw[i * k + p];
        } else if (p < nf + nb) {
            const unsigned long long e = tval[b0 + (p - nf)];
            key[r] = ((uint32_t)(e >> 32) << 1) | 1u;
            w[r] = __uint_as_float((uint32_t)e);
        }
    }
    // Ascending bitonic sort over the P positions (keys of valid entries are
    // unique; the padding keys are equal and carry nothing).
#pragma unroll
    for (int size = 2; size <= P; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride == 32) {
                if (key[R - 1] < key[0]) {
                    const uint32_t tk = key[0];
                    const float tw = w[0];
                    key[0] = key[R - 1];
                    w[0] = w[R - 1];
                    key[R - 1] = tk;
                    w[R - 1] = tw;
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int p = lane + 32 * r;
                    const uint32_t ok = __shfl_xor_sync(0xffffffffu, key[r], stride);
                    const float ow = __shfl_xor_sync(0xffffffffu, w[r], stride);
                    const bool take_min = ((p & stride) == 0) == ((p & size) == 0);
                    if (ok != key[r] && (ok < key[r]) == take_min) {
                        key[r] = ok;
                        w[r] = ow;
                    }
                }
            }
        }
    }
    // Neighbouring positions: p - 1 and p + 1.
    uint32_t prev[R], next[R];
    float nextw[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t up = __shfl_up_sync(0xffffffffu, key[r], 1);
        const uint32_t dn = __shfl_down_sync(0xffffffffu, key[r], 1);
        const float dnw = __shfl_down_sync(0xffffffffu, w[r], 1);
        const uint32_t wrap_up = r > 0 ? __shfl_sync(0xffffffffu, key[r > 0 ? r - 1 : 0], 31) : 0xffffffffu;
        const uint32_t wrap_dn = r + 1 < R ? __shfl_sync(0xffffffffu, key[r + 1 < R ? r + 1 : r], 0) : 0xffffffffu;
        const float wrap_dnw = r + 1 < R ? __shfl_sync(0xffffffffu, w[r + 1 < R ? r + 1 : r], 0) : 0.f;
        prev[r] = lane == 0 ? wrap_up : up;
        next[r] = lane == 31 ? wrap_dn : dn;
        nextw[r] = lane == 31 ? wrap_dnw : dnw;
    }
    bool keep[R];
    uint32_t ball[R];
    int total = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        // An incoming edge right after its directed twin merged into it.
        keep[r] = key[r] != 0xffffffffu && !((key[r] & 1u) && prev[r] == (key[r] ^ 1u));
        ball[r] = __ballot_sync(0xffffffffu, keep[r]);
        total += __popc(ball[r]);
    }
    int before = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (keep[r]) {
            const int pos = before + __popc(ball[r] & lanemask_lt());
            float v = w[r];
            if (!(key[r] & 1u) && next[r] == (key[r] | 1u)) {
                const float rv = nextw[r];
                v = __fsub_rn(__fadd_rn(w[r], rv), __fmul_rn(w[r], rv));
            }
            scol[pos] = key[r] >> 1;
            sval[pos] = v;
        }
        before += __popc(ball[r]);
    }
    return total;
}

__global__ void __launch_bounds__(256) merge_union_kernel(const uint32_t* __restrict__ dcol,
                                                          const float* __restrict__ dw,
                                                          const uint32_t* __restrict__ dcnt,
                                                          unsigned long long* __restrict__ tval,
                                                          const uint32_t* __restrict__ tstart, int64_t r0, int64_t r1,
                                                          int k, uint32_t* __restrict__ scol, float* __restrict__ sval,
                                                          uint32_t* __restrict__ rowcnt) {
    const int lane = threadIdx.x & 31;
    const int64_t i = r0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (i >= r1) return;
    const int nf = (int)dcnt[i];
    const uint32_t b0 = tstart[i];
    const int nb = (int)(tstart[i + 1] - b0);
    const int64_t run = i * k + b0;
    uint32_t* rc = scol + run;
    float* rv = sval + run;
    int total;
    if (nf + nb <= 32) {
        total = union_sorted_row<32>(dcol, dw, tval, i, k, nf, b0, nb, rc, rv);
    } else if (nf + nb <= 64) {
        total = union_sorted_row<64>(dcol, dw, tval, i, k, nf, b0, nb, rc, rv);
    } else {
        // Many incoming edges: the bucket sorted in place, every directed
        // entry placed by binary search among the sources and every incoming
        // edge by counting the directed columns below it.
        warp_sort_bucket(tval + b0, (uint32_t)nb);
        const uint32_t fcol = lane < nf ? dcol[i * k + lane] : 0xffffffffu;
        const float fw = lane < nf ? dw[i * k + lane] : 0.f;
        int less_b = 0;
        bool dup_f = false;
        float rv_f = 0.f;
        if (lane < nf) {  // lower bound of this lane's column among the sorted sources
            int lo = 0, hi = nb;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if ((uint32_t)(tval[b0 + mid] >> 32) < fcol)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            less_b = lo;
            if (lo < nb) {
                const unsigned long long e = tval[b0 + lo];
                if ((uint32_t)(e >> 32) == fcol) {
                    dup_f = true;
                    rv_f = __uint_as_float((uint32_t)e);
                }
            }
        }
        const uint32_t dupmask = __ballot_sync(0xffffffffu, lane < nf && dup_f);
        for (int base = 0; base < nb; base += 32) {
            const int j = base + lane;
            const unsigned long long e = j < nb ? tval[b0 + j] : ~0ull;
            const uint32_t src = (uint32_t)(e >> 32);
            int lf = 0;
            bool db = false;
            for (int t = 0; t < nf; ++t) {
                const uint32_t c_t = __shfl_sync(0xffffffffu, fcol, t);
                lf += c_t < src;
                db |= c_t == src;
            }
            if (j < nb && !db) {
                const uint32_t q = (uint32_t)(j + lf) - (uint32_t)__popc(dupmask & mask_below(lf));
                rc[q] = src;
                rv[q] = __uint_as_float((uint32_t)e);
            }
        }
        if (lane < nf) {
            const uint32_t q = (uint32_t)(lane + less_b) - (uint32_t)__popc(dupmask & lanemask_lt());
            const float r2 = dup_f ? rv_f : 0.f;
            rc[q] = fcol;
            rv[q] = __fsub_rn(__fadd_rn(fw, r2), __fmul_rn(fw, r2));
        }
        total = nf + nb - __popc(dupmask);
    }
    if (lane == 0) rowcnt[i] = (uint32_t)total;
}

// The writing pass of rows [r0, r1): every merged run into its place in the
// CSR.  `rel` holds the range's row lengths scanned in place (rel[r0] = 0,
// rel[r1] = the range's total); the range starts at *carry_in, the offset
// past the earlier ranges, and the offset past this one goes to *carry_out
// and indptr[r1].
__global__ void __launch_bounds__(256) merge_place_kernel(const uint32_t* __restrict__ scol,
                                                          const float* __restrict__ sval,
                                                          const uint32_t* __restrict__ tstart, int64_t r0, int64_t r1,
                                                          int k, const uint32_t* __restrict__ rel,
                                                          const uint32_t* __restrict__ carry_in,
                                                          uint32_t* __restrict__ carry_out, uint32_t* __restrict__ indptr,
                                                          uint32_t* __restrict__ out_cols, float* __restrict__ out_vals) {
    const int lane = threadIdx.x & 31;
    const int64_t i = r0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (i >= r1) return;
    const uint32_t c0 = *carry_in;
    const int64_t run = i * k + tstart[i];
    const uint32_t base = c0 + rel[i], len = rel[i + 1] - rel[i];
    for (uint32_t j = lane; j < len; j += 32) {
        out_cols[base + j] = scol[run + j];
        out_vals[base + j] = sval[run + j];
    }
    if (lane == 0) {
        indptr[i] = base;
        if (i == r1 - 1) {
            indptr[r1] = c0 + rel[r1];
            *carry_out = c0 + rel[r1];
        }
    }
}

// Bucket starts of the edges sorted by target row: start[j] = the number of
// keys below j, for j in [0, n] (keys are at most n; n marks unused slots).
// Position p writes the starts of the rows in (key[p-1], key[p]]; the last
// position also those above its key.
__global__ void bucket_starts_kernel(const uint32_t* __restrict__ keys, int64_t E, int64_t n,
                                     uint32_t* __restrict__ start) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= E) return;
    const int64_t kp = keys[p];
    const int64_t lo = p == 0 ? 0 : (int64_t)keys[p - 1] + 1;
    for (int64_t j = lo; j <= kp && j <= n; ++j) start[j] = (uint32_t)p;
    if (p == E - 1)
        for (int64_t j = kp + 1; j <= n; ++j) start[j] = (uint32_t)E;
}

// Query rows against a reference: the directed weights of each row
// (directed_kernel's arithmetic, with no self to drop), columns ascending.
__global__ void query_rows_kernel(const uint32_t* __restrict__ idx, const float* __restrict__ dist, int64_t q, int k,
                                  const float* __restrict__ sigmas, const float* __restrict__ rhos,
                                  uint32_t* __restrict__ dcol, float* __restrict__ dw, uint32_t* __restrict__ dcnt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q) return;
    uint32_t* col = dcol + i * k;
    float* w = dw + i * k;
    int m = 0;
    const float sigma = sigmas[i], rho = rhos[i];
    for (int j = 0; j < k; j++) {
        const uint32_t nb = idx[i * k + j];
        const float offset = __fsub_rn(dist[i * k + j], rho);
        const float wt = (offset <= 0.f || sigma == 0.f) ? 1.0f : expf(__fdiv_rn(-offset, sigma));
        if (wt == 0.f) continue;
        int s = m;
        while (s > 0 && col[s - 1] > nb) {
            col[s] = col[s - 1];
            w[s] = w[s - 1];
            s--;
        }
        col[s] = nb;
        w[s] = wt;
        m++;
    }
    dcnt[i] = (uint32_t)m;
}

__global__ void query_csr_kernel(const uint32_t* __restrict__ dcol, const float* __restrict__ dw,
                                 const uint32_t* __restrict__ dcnt, const uint32_t* __restrict__ indptr, int64_t q,
                                 int k, uint32_t* __restrict__ indices, float* __restrict__ values) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q) return;
    const uint32_t o = indptr[i];
    for (uint32_t t = 0; t < dcnt[i]; ++t) {
        indices[o + t] = dcol[i * k + t];
        values[o + t] = dw[i * k + t];
    }
}

// ---- stable LSD radix sort (8-bit digits) ---------------------------------

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;  // 4096

__global__ void rs_hist_kernel(const uint32_t* __restrict__ keys, int64_t total, int shift,
                               uint32_t* __restrict__ block_hist, int nblocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int64_t p = t0 + r * RS_THREADS + threadIdx.x;
        if (p < total) atomicAdd(&h[(keys[p] >> shift) & 255u], 1u);
    }
    __syncthreads();
    block_hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// One tile of RS_TILE pairs per block: each pair's rank among the tile's
// pairs of its digit (warp by warp, in input order: the sort is stable), the
// tile reordered by digit in shared memory, then written out digit run by
// digit run so that neighbouring threads write neighbouring addresses.
constexpr size_t RS_STAGE_BYTES = (size_t)RS_TILE * (sizeof(unsigned long long) + sizeof(uint32_t));
__global__ void __launch_bounds__(RS_THREADS) rs_scatter_kernel(const uint32_t* __restrict__ kin,
                                                                const unsigned long long* __restrict__ vin,
                                                                uint32_t* __restrict__ kout,
                                                                unsigned long long* __restrict__ vout, int64_t total,
                                                                int shift, const uint32_t* __restrict__ offsets,
                                                                int nblocks) {
    extern __shared__ unsigned long long rs_stage[];  // RS_TILE payloads, then RS_TILE keys
    uint32_t* kst = reinterpret_cast<uint32_t*>(rs_stage + RS_TILE);
    __shared__ uint32_t wcnt[RS_WARPS][256];
    __shared__ uint32_t dstart[256], dout[256], wsum[RS_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = lane; d < 256; d += 32) wcnt[warp][d] = 0;
    __syncwarp();
    const int64_t t0 = (int64_t)blockIdx.x * RS_TILE;
    const int64_t base = t0 + (int64_t)warp * (RS_TILE / RS_WARPS);
    uint32_t key[RS_ROUNDS];
    unsigned long long val[RS_ROUNDS];
    uint32_t rank[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int64_t p = base + r * 32 + lane;
        const bool valid = p < total;
        key[r] = valid ? kin[p] : 0xffffffffu;
        val[r] = valid ? vin[p] : 0ull;
        const uint32_t d = valid ? ((key[r] >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = valid ? wcnt[warp][d] : 0u;
        rank[r] = before + __popc(peers & lanemask_lt());
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == lane) wcnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        // Per digit: each warp's offset within the tile's run of that digit,
        // then the run starts (an exclusive scan over the 256 digits).
        const int d = threadIdx.x;  // 256 threads, one digit each
        uint32_t run = 0;
        for (int w = 0; w < RS_WARPS; w++) {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
        uint32_t incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[warp] = incl;
        dout[d] = offsets[(int64_t)d * nblocks + blockIdx.x];
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; w++) before += wsum[w];
        dstart[d] = before + incl - run;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int64_t p = base + r * 32 + lane;
        if (p < total) {
            const uint32_t d = (key[r] >> shift) & 255u;
            const uint32_t lp = dstart[d] + wcnt[warp][d] + rank[r];
            kst[lp] = key[r];
            rs_stage[lp] = val[r];
        }
    }
    __syncthreads();
    const int count = (int)min((int64_t)RS_TILE, total - t0);
    for (int lp = threadIdx.x; lp < count; lp += RS_THREADS) {
        const uint32_t k = kst[lp];
        const uint32_t d = (k >> shift) & 255u;
        const int64_t dst = (int64_t)dout[d] + (lp - (int)dstart[d]);
        kout[dst] = k;
        vout[dst] = rs_stage[lp];
    }
}

// ---- exclusive scan of u32 --------------------------------------------------

constexpr int SC_THREADS = 1024;
constexpr int SC_TILE = 2 * SC_THREADS;

__global__ void scan_tiles_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int64_t n,
                                  uint32_t* __restrict__ sums) {
    __shared__ uint32_t warp_tot[SC_THREADS / 32];
    const int64_t p0 = (int64_t)blockIdx.x * SC_TILE + 2 * threadIdx.x;
    const uint32_t a = p0 < n ? in[p0] : 0u;
    const uint32_t b = p0 + 1 < n ? in[p0 + 1] : 0u;
    const uint32_t t = a + b;
    uint32_t x = t;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = warp_tot[lane];
        uint32_t s = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_tot[lane] = s - v;  // exclusive
        if (lane == 31 && sums) sums[blockIdx.x] = s;
    }
    __syncthreads();
    const uint32_t excl = warp_tot[warp] + x - t;
    if (p0 < n) out[p0] = excl;
    if (p0 + 1 < n) out[p0 + 1] = excl + a;
}

__global__ void scan_add_kernel(uint32_t* __restrict__ out, int64_t n, const uint32_t* __restrict__ sums) {
    const int64_t p0 = (int64_t)blockIdx.x * SC_TILE + 2 * threadIdx.x;
    const uint32_t add = sums[blockIdx.x];
    if (p0 < n) out[p0] += add;
    if (p0 + 1 < n) out[p0 + 1] += add;
}

// ---- symmetrise -------------------------------------------------------------

__global__ void merge_kernel(const uint32_t* __restrict__ dcol, const float* __restrict__ dw,
                             const uint32_t* __restrict__ dcnt, const unsigned long long* __restrict__ tval,
                             const uint32_t* __restrict__ tstart, int64_t n, int k,
                             const uint32_t* __restrict__ indptr, uint32_t* __restrict__ rowcnt,
                             uint32_t* __restrict__ out_cols, float* __restrict__ out_vals) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* fc = dcol + i * k;
    const float* fw = dw + i * k;
    const int nf = (int)dcnt[i];
    const uint32_t b0 = tstart[i], b1 = tstart[i + 1];
    const bool write = indptr != nullptr;
    uint32_t out = write ? indptr[i] : 0u;
    uint32_t count = 0;
    int f = 0;
    uint32_t b = b0;
    while (f < nf || b < b1) {
        const uint32_t fcol = f < nf ? fc[f] : 0xffffffffu;
        const uint32_t bcol = b < b1 ? (uint32_t)(tval[b] >> 32) : 0xffffffffu;
        const uint32_t c = fcol < bcol ? fcol : bcol;
        float wv = 0.f, rv = 0.f;
        if (f < nf && fcol == c) {
            wv = fw[f];
            f++;
        }
        if (b < b1 && bcol == c) {
            rv = __uint_as_float((uint32_t)tval[b]);
            b++;
        }
        if (write) {
            out_cols[out + count] = c;
            out_vals[out + count] = __fsub_rn(__fadd_rn(wv, rv), __fmul_rn(wv, rv));
        }
        count++;
    }
    if (!write) rowcnt[i] = count;
}

}  // namespace

// Exclusive scan of n u32 values (in may equal out).
cudaError_t device_exclusive_scan(scrust_context* ctx, const uint32_t* in, uint32_t* out, int64_t n,
                                  uint32_t* scratch, size_t scratch_elems) {
    const int64_t tiles = (n + SC_TILE - 1) / SC_TILE;
    if (tiles <= 1) {
        scan_tiles_kernel<<<1, SC_THREADS, 0, ctx->stream>>>(in, out, n, nullptr);
        ctx->launches += 1;
        return cudaGetLastError();
    }
    ctx->launches += 2;
    if ((size_t)tiles > scratch_elems) return cudaErrorInvalidValue;
    uint32_t* sums = scratch;
    scan_tiles_kernel<<<(unsigned)tiles, SC_THREADS, 0, ctx->stream>>>(in, out, n, sums);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = device_exclusive_scan(ctx, sums, sums, tiles, scratch + tiles, scratch_elems - (size_t)tiles);
    if (e != cudaSuccess) return e;
    scan_add_kernel<<<(unsigned)tiles, SC_THREADS, 0, ctx->stream>>>(out, n, sums);
    return cudaGetLastError();
}

size_t scan_scratch_elems(int64_t n) {
    size_t total = 0;
    int64_t t = (n + SC_TILE - 1) / SC_TILE;
    while (t > 1) {
        total += (size_t)t;
        t = (t + SC_TILE - 1) / SC_TILE;
    }
    return total + 16;
}

// Stable LSD radix sort of (key, payload) pairs on the low `bits` bits of the
// keys, 8 bits per pass.  Ping-pongs between the A and B buffers; *keys_out
// and *vals_out point at whichever holds the result.  `hist` holds
// 256 * ceil(n / 4096) words and `scan_scratch` scan_scratch_elems(that) words.
cudaError_t radix_sort_pairs(scrust_context* ctx, uint32_t* kA, unsigned long long* vA, uint32_t* kB,
                             unsigned long long* vB, int64_t n, int bits, uint32_t* hist, uint32_t* scan_scratch,
                             size_t scan_elems, uint32_t** keys_out, unsigned long long** vals_out) {
    const int nblocks = (int)((n + RS_TILE - 1) / RS_TILE);
    uint32_t *kin = kA, *kout = kB;
    unsigned long long *vin = vA, *vout = vB;
    cudaError_t e = cudaSuccess;
    for (int shift = 0; shift < bits; shift += 8) {
        rs_hist_kernel<<<nblocks, RS_THREADS, 0, ctx->stream>>>(kin, n, shift, hist, nblocks);
        if ((e = device_exclusive_scan(ctx, hist, hist, (int64_t)256 * nblocks, scan_scratch, scan_elems)) != cudaSuccess)
            return e;
        if ((e = set_smem_limit(ctx, (const void*)rs_scatter_kernel, (int)RS_STAGE_BYTES)) != cudaSuccess) return e;
        rs_scatter_kernel<<<nblocks, RS_THREADS, RS_STAGE_BYTES, ctx->stream>>>(kin, vin, kout, vout, n, shift, hist,
                                                                                nblocks);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ctx->launches += 2;
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    *keys_out = kin;
    *vals_out = vin;
    return cudaSuccess;
}

int radix_blocks(int64_t n) { return (int)((n + RS_TILE - 1) / RS_TILE); }

cudaError_t launch_smooth_knn(scrust_context* ctx, const float* dist, int64_t n, int k, float* sigmas,
                              float* rhos, bool report_sigmas) {
    cudaError_t e = cudaSuccess;
    const int64_t total = n * (int64_t)k;
    float* mean = nullptr;
    if (report_sigmas) {
        mean = (float*)ws_get(ctx, SLOT_MISC, 64, &e);
        if (!mean) return e;
        if ((e = set_smem_limit(ctx, (const void*)unrolled_mean_kernel, (int)FOLD_SMEM_BYTES)) != cudaSuccess)
            return e;
        unrolled_mean_kernel<<<1, FOLD_THREADS, FOLD_SMEM_BYTES, ctx->stream>>>(dist, total, mean);
        ctx->launches += 1;
    }
    const double target = log2((double)(k + 1));
    smooth_knn_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(dist, n, k, target, mean,
                                                                           sigmas, rhos);
    ctx->launches += 1;
    return cudaGetLastError();
}

int32_t run_query_connectivities(scrust_context* ctx, const uint32_t* idx, const float* dist, int64_t q, int k,
                                 CsrBuffers* out, scrust_status* st) {
    cudaError_t e = cudaSuccess;
    cudaStream_t s = ctx->stream;
    const int64_t E = q * (int64_t)k;
    const size_t scan_elems = scan_scratch_elems(q + 1);
    char* a = (char*)ws_get(ctx, SLOT_CONN_A, sizeof(float) * 2 * (size_t)q + sizeof(uint32_t) * (size_t)(q + 1) + 256, &e);
    uint32_t* dcol = (uint32_t*)ws_get(ctx, SLOT_CONN_B, sizeof(uint32_t) * (size_t)E, &e);
    float* dw = (float*)ws_get(ctx, SLOT_CONN_C, sizeof(float) * (size_t)E, &e);
    uint32_t* scan_scratch = (uint32_t*)ws_get(ctx, SLOT_SCAN, sizeof(uint32_t) * scan_elems, &e);
    if (!a || !dcol || !dw || !scan_scratch) return cuda_fail(st, e, "query connectivities: workspace");
    float* sig = (float*)a;
    float* rho = sig + q;
    uint32_t* dcnt = (uint32_t*)(rho + q);  // q + 1
    if ((e = launch_smooth_knn(ctx, dist, q, k, sig, rho, false)) != cudaSuccess) return cuda_fail(st, e, "smooth_knn");
    query_rows_kernel<<<(unsigned)((q + 127) / 128), 128, 0, s>>>(idx, dist, q, k, sig, rho, dcol, dw, dcnt);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "query rows");
    if ((e = cudaMemsetAsync(dcnt + q, 0, sizeof(uint32_t), s)) != cudaSuccess) return cuda_fail(st, e, "memset");
    if ((e = device_exclusive_scan(ctx, dcnt, out->indptr, q + 1, scan_scratch, scan_elems)) != cudaSuccess)
        return cuda_fail(st, e, "query row scan");
    query_csr_kernel<<<(unsigned)((q + 127) / 128), 128, 0, s>>>(dcol, dw, dcnt, out->indptr, q, k, out->indices,
                                                                out->values);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "query csr");
    ctx->launches += 2;
    return ok(st);
}

// The fuzzy union of a graph whose rows hold distinct ids, k <= 32: weights
// with bucket places from one atomic per edge, the in-degree scan, the bucket
// scatter, then per row range a merge with one warp per row into scratch
// runs, the scan of the range's row lengths (in place) and the writing pass,
// each range continuing the last one's offsets.  One range, or with `ranges`
// ctx->csr_stream's kCsrRanges, each range's end recorded (and its end offset
// sent to the host) for a download that overlaps the later ranges.  The CSR
// is bit-identical to the radix-sort path's.
int32_t run_connectivities_distinct(scrust_context* ctx, const uint32_t* idx, const float* dist, int64_t n, int k,
                                    CsrBuffers* out, scrust_status* st, bool ranges) {
    cudaError_t e = cudaSuccess;
    cudaStream_t s = ctx->stream;
    const int64_t E = n * (int64_t)k;
    const size_t scan_elems = scan_scratch_elems(n + 1);
    char* a = (char*)ws_get(ctx, SLOT_CONN_A, sizeof(float) * 2 * (size_t)n + sizeof(uint32_t) * 3 * (size_t)(n + 1) + 256, &e);
    uint32_t* dcol = (uint32_t*)ws_get(ctx, SLOT_CONN_B, sizeof(uint32_t) * (size_t)E, &e);
    float* dw = (float*)ws_get(ctx, SLOT_CONN_C, sizeof(float) * (size_t)E, &e);
    uint32_t* erank = (uint32_t*)ws_get(ctx, SLOT_CONN_D, sizeof(uint32_t) * (size_t)E, &e);
    unsigned long long* tval = (unsigned long long*)ws_get(ctx, SLOT_CONN_E, sizeof(unsigned long long) * (size_t)E, &e);
    // Merged runs: row i's at i * k + start[i], k + in-degree entries each.
    uint32_t* scol = (uint32_t*)ws_get(ctx, SLOT_CONN_H, 2 * sizeof(uint32_t) * 2 * (size_t)E, &e);
    float* sval = scol ? (float*)(scol + 2 * (size_t)E) : nullptr;
    uint32_t* scan_scratch = (uint32_t*)ws_get(ctx, SLOT_SCAN, sizeof(uint32_t) * scan_elems, &e);
    if (!a || !dcol || !dw || !erank || !tval || !scol || !scan_scratch)
        return cuda_fail(st, e, "connectivities: workspace");
    float* sig = (float*)a;
    float* rho = sig + n;
    uint32_t* indeg = (uint32_t*)(rho + n);  // n + 1, then the bucket starts in place
    uint32_t* rowcnt = indeg + (n + 1);      // n + 1: row lengths, scanned range by range in place
    uint32_t* dcnt = rowcnt + (n + 1);       // n (+1 spare)
    uint32_t* carry = dcnt + (n + 1);        // kCsrRanges + 1 offsets, in the 256 spare bytes
    static_assert(sizeof(uint32_t) * (kCsrRanges + 1) <= 256, "range offsets fit the spare bytes");
    const int R = ranges ? kCsrRanges : 1;
    if ((e = cudaMemsetAsync(indeg, 0, sizeof(uint32_t) * (size_t)(n + 1), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(carry, 0, sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(rowcnt + n, 0, sizeof(uint32_t), s)) != cudaSuccess)
        return cuda_fail(st, e, "memset");
    if ((e = launch_smooth_knn(ctx, dist, n, k, sig, rho, false)) != cudaSuccess) return cuda_fail(st, e, "smooth_knn");
    if (k <= 16)
        directed_bucket_kernel<16><<<(unsigned)((n * 16 + 255) / 256), 256, 0, s>>>(idx, dist, n, k, sig, rho, dcol,
                                                                                   dw, dcnt, indeg, erank);
    else
        directed_bucket_kernel<32><<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(idx, dist, n, k, sig, rho, dcol,
                                                                                   dw, dcnt, indeg, erank);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "directed weights");
    if ((e = device_exclusive_scan(ctx, indeg, indeg, n + 1, scan_scratch, scan_elems)) != cudaSuccess)
        return cuda_fail(st, e, "in-degree scan");
    bucket_scatter_kernel<<<(unsigned)((E + 255) / 256), 256, 0, s>>>(dcol, dw, dcnt, erank, indeg, n, k, tval);
    ctx->launches += 2;
    for (int r = 0; r < R; ++r) {
        const int64_t r0 = n * r / R, r1 = n * (r + 1) / R;
        if (r1 > r0) {
            const unsigned blocks = (unsigned)(((r1 - r0) * 32 + 255) / 256);
            merge_union_kernel<<<blocks, 256, 0, s>>>(dcol, dw, dcnt, tval, indeg, r0, r1, k, scol, sval, rowcnt);
            // rowcnt[r1] is the next range's first row (or the zero past the
            // last): it only receives the range's total.
            if ((e = cudaGetLastError()) != cudaSuccess ||
                (e = device_exclusive_scan(ctx, rowcnt + r0, rowcnt + r0, r1 - r0 + 1, scan_scratch, scan_elems)) !=
                    cudaSuccess)
                return cuda_fail(st, e, "row scan");
            merge_place_kernel<<<blocks, 256, 0, s>>>(scol, sval, indeg, r0, r1, k, rowcnt, carry + r, carry + r + 1,
                                                      out->indptr, out->indices, out->values);
            ctx->launches += 2;
        } else if ((e = cudaMemcpyAsync(carry + r + 1, carry + r, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s)) !=
                   cudaSuccess) {
            return cuda_fail(st, e, "merge");
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "merge");
        if (ranges && ((e = cudaMemcpyAsync(ctx->csr_stream.h_bounds + r, carry + r + 1, sizeof(uint32_t),
                                            cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
                       (e = cudaEventRecord(ctx->csr_stream.merged[r], s)) != cudaSuccess))
            return cuda_fail(st, e, "merge");
    }
    if (n == 0 && (e = cudaMemsetAsync(out->indptr, 0, sizeof(uint32_t), s)) != cudaSuccess)
        return cuda_fail(st, e, "memset");
    return ok(st);
}

int32_t run_connectivities(scrust_context* ctx, const uint32_t* idx, const float* dist, int64_t n, int k,
                           bool validate, CsrBuffers* out, scrust_status* st, bool distinct_rows, bool ranges,
                           bool* streamed) {
    const bool distinct = distinct_rows && !validate && k <= 32 && n < ((int64_t)1 << 31);
    if (streamed) *streamed = distinct && ranges;
    if (distinct) return run_connectivities_distinct(ctx, idx, dist, n, k, out, st, ranges);
    cudaError_t e = cudaSuccess;
    cudaStream_t s = ctx->stream;
    const int64_t E = n * (int64_t)k;
    uint64_t scan_launches = 0;
    if (validate) {
        scan_launches += 1;
        check_ids_kernel<<<1024, 256, 0, s>>>(idx, E, n, ctx->d_err);
        int bad = 0;
        if ((e = cudaMemcpyAsync(&bad, ctx->d_err + DERR_BAD_INDEX, sizeof(int), cudaMemcpyDeviceToHost, s)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_fail(st, e, "connectivities: id check");
        if (bad) {
            cudaMemsetAsync(ctx->d_err + DERR_BAD_INDEX, 0, sizeof(int), s);
            return fail(st, SCRUST_SHAPE, "expected neighbour ids below %lld, got an out-of-range neighbour id",
                        (long long)n);
        }
    }
    // Scratch layout.
    const int nblocks = (int)((E + RS_TILE - 1) / RS_TILE);
    const size_t scan_elems = scan_scratch_elems(std::max<int64_t>((int64_t)256 * nblocks, n + 1));
    char* a = (char*)ws_get(ctx, SLOT_CONN_A, sizeof(float) * 2 * (size_t)n + sizeof(uint32_t) * 3 * (size_t)(n + 1) + 256, &e);
    uint32_t* dcol = (uint32_t*)ws_get(ctx, SLOT_CONN_B, sizeof(uint32_t) * (size_t)E, &e);
    float* dw = (float*)ws_get(ctx, SLOT_CONN_C, sizeof(float) * (size_t)E, &e);
    uint32_t* keyA = (uint32_t*)ws_get(ctx, SLOT_CONN_D, sizeof(uint32_t) * 2 * (size_t)E, &e);
    unsigned long long* valA = (unsigned long long*)ws_get(ctx, SLOT_CONN_E, sizeof(unsigned long long) * 2 * (size_t)E, &e);
    uint32_t* hist = (uint32_t*)ws_get(ctx, SLOT_CONN_F, sizeof(uint32_t) * ((size_t)256 * nblocks + 16), &e);
    uint32_t* scan_scratch = (uint32_t*)ws_get(ctx, SLOT_SCAN, sizeof(uint32_t) * scan_elems, &e);
    if (!a || !dcol || !dw || !keyA || !valA || !hist || !scan_scratch) return cuda_fail(st, e, "connectivities: workspace");
    float* sig = (float*)a;
    float* rho = sig + n;
    uint32_t* indeg = (uint32_t*)(rho + n);   // n + 1
    uint32_t* rowcnt = indeg + (n + 1);        // n + 1
    uint32_t* dcnt = rowcnt + (n + 1);         // n (+1 spare)
    uint32_t* keyB = keyA + E;
    unsigned long long* valB = valA + E;

    if ((e = launch_smooth_knn(ctx, dist, n, k, sig, rho, false)) != cudaSuccess) return cuda_fail(st, e, "smooth_knn");
    if (k <= 16)
        directed_group_kernel<16><<<(unsigned)((n * 16 + 255) / 256), 256, 0, s>>>(idx, dist, n, k, sig, rho, dcol,
                                                                                  dw, dcnt, keyA, valA);
    else if (k <= 32)
        directed_group_kernel<32><<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(idx, dist, n, k, sig, rho, dcol,
                                                                                  dw, dcnt, keyA, valA);
    else
        directed_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(idx, dist, n, k, sig, rho, dcol, dw, dcnt, keyA,
                                                                     valA);
    scan_launches += 1 /* directed */ + 2 /* merges */;
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "directed weights");
    // Stable radix sort of the edge slots by target row.
    int bits = 1;
    while (((int64_t)1 << bits) <= n) bits++;
    uint32_t *kin = keyA, *kout = keyB;
    unsigned long long *vin = valA, *vout = valB;
    for (int shift = 0; shift < bits; shift += 8) {
        rs_hist_kernel<<<nblocks, RS_THREADS, 0, s>>>(kin, E, shift, hist, nblocks);
        if ((e = device_exclusive_scan(ctx, hist, hist, (int64_t)256 * nblocks, scan_scratch, scan_elems)) != cudaSuccess)
            return cuda_fail(st, e, "radix scan");
        if ((e = set_smem_limit(ctx, (const void*)rs_scatter_kernel, (int)RS_STAGE_BYTES)) != cudaSuccess)
            return cuda_fail(st, e, "radix scatter");
        rs_scatter_kernel<<<nblocks, RS_THREADS, RS_STAGE_BYTES, s>>>(kin, vin, kout, vout, E, shift, hist, nblocks);
        scan_launches += 2;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "radix scatter");
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    // Transpose bucket starts, from the sorted keys.
    bucket_starts_kernel<<<(unsigned)((E + 255) / 256), 256, 0, s>>>(kin, E, n, indeg);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "bucket starts");
    scan_launches += 1;
    merge_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(dcol, dw, dcnt, vin, indeg, n, k, nullptr, rowcnt,
                                                             nullptr, nullptr);
    if ((e = cudaMemsetAsync(rowcnt + n, 0, sizeof(uint32_t), s)) != cudaSuccess) return cuda_fail(st, e, "memset");
    if ((e = device_exclusive_scan(ctx, rowcnt, out->indptr, n + 1, scan_scratch, scan_elems)) != cudaSuccess)
        return cuda_fail(st, e, "row scan");
    merge_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(dcol, dw, dcnt, vin, indeg, n, k, out->indptr, nullptr,
                                                             out->indices, out->values);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "merge");
    ctx->launches += scan_launches;
    return ok(st);
}

}  // namespace scrust
