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
// Kernel layout (persistent, one CTA per SM, 576 threads):
//   warp 0      TMA producer: A (256 query rows) per work item, B (256
//               reference rows) per tile, 4-stage ring
//   warp 1      TMEM owner and MMA issuer: per B tile, two M=128 x N=256 x
//               K=16 x4 chains into two TMEM accumulators (query halves)
//   warps 2-17  epilogue: 8 warps per half; warp w reads TMEM lanes
//               32*(w%4).. and one 128-column part of its half's
//               accumulator.  Each thread owns one query row and one list per
//               column part; it tests 32 columns at a time against its
//               threshold (3-input min) while the next 32 are loaded from
//               TMEM, appends survivors, and after releasing the accumulator
//               prunes full lists warp-cooperatively.  The two parts of a row
//               share their thresholds through shared memory.
// The two accumulators ping-pong: the epilogue drains half 0 of tile j while
// the tensor core computes half 1 of tile j, so each B tile is read once per
// 256 query rows.  Every wait is bounded (tma.cuh).
//
// The kernel is compiled once per (top-k size, pass kind).  PASS 1 only
// tightens thresholds with a register top-k, PASS 2 only collects ids below
// fixed thresholds, PASS 3 keeps each row's nearest column to within 32 ulp
// of the smallest value (no lists; an ordering needs no more), and
// PASS 0 takes the kind from its arguments.  A specialised pass carries none
// of the others' code, which matters because the epilogue is held to 96
// registers (18 warps on an SM) and its ALU pipe is the bottleneck.
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
constexpr int PARTS = 2;               // column parts of a tile, one epilogue warp each
constexpr int EPI_WARPS = HALVES * PARTS * 4;
constexpr int THREADS = (2 + EPI_WARPS) * 32;
constexpr uint32_t A_BYTES = ROWS * TK * 2;
constexpr uint32_t B_BYTES = TBN * TK * 2;
constexpr uint32_t TMEM_COLS = 512;
constexpr size_t SMEM_BYTES = 2 * A_BYTES + STAGES * B_BYTES + 1024;
constexpr int kPartCols = TBN / PARTS;  // columns one epilogue warp drains per tile

struct TensorArgs {
    Lists lists;
    const float* bA;
    const float* bdelta;
    const float* beps2;
    int64_t nq, nr;
    int k;
    int self;
    int64_t self_offset;  // query row i is column i + self_offset
    int col_tiles;
    int tiles_per_seg;
    int items;
    uint32_t idesc;
    int* err;
    unsigned long long* stats;  // optional counters (TensorStat), null when off
    // Explicit column tiles per work item (one column segment), or null for
    // the outward sweep over the item's whole segment.
    const uint32_t* tl;
    const uint32_t* tl_off;     // per-item offsets into tl, or null: item * tl_stride
    const uint32_t* tl_cnt;
    int tl_stride;
    const uint32_t* tl2;        // a second explicit list per item, visited after the first, or null
    const uint32_t* tl2_cnt;
    int tl2_stride;
    const uint32_t* item_order; // items by decreasing work, dealt out in a snake, or null: round robin
    const uint2* item_range;    // per item its column tiles [x, y) (one column segment), or null
    uint32_t* row_theta;        // per query row the smallest threshold any of its lists reached
                                // (float_key; 0xffffffff = none), shared across column segments; or null
    const uint32_t* row_map;    // per query row its input row, 0xffffffff for padding; null: all rows real
    // k = 1 without lists: per (row, part) the smallest MMA value and its
    // column, packed as float_key << 32 | column; null otherwise.  (The
    // nearest-column pass carries the column in the value's low five bits, so
    // its choice is exact up to values within 32 ulp of each other.)
    unsigned long long* argmin_out;
    int final_cap;              // lists longer than this are pruned once more when an item ends
    int resume;                 // lists and thresholds continue from an earlier pass
    // thr_only: the pass only tightens thresholds (register top-k, theta_io
    // written), no list is touched.  collect: the thresholds are fixed at the
    // smaller of each row's theta_io entries and the pass only appends.
    int thr_only, collect;
    float* theta_io;            // per list: the threshold when the item ends (read when resuming)
    float* topk_out;            // threshold passes: per list, the register top-K when the item ends
                                // (ascending, the first K - k slots -inf; slot t of list l at
                                // t * topk_stride + l, so a warp's stores are contiguous), or null
    int64_t topk_stride;        // lists in all
};

// Counters gathered when statistics are on (summed over all CTAs).
enum TensorStat : int {
    TS_APPENDS = 0,        // candidates appended to lists
    TS_PRUNES = 1,         // warp-cooperative prunes
    TS_OVERFLOWS = 2,      // rows sent to the exact fallback
    TS_EPI_WAIT = 3,       // epilogue cycles waiting for an accumulator (lane 0 of each warp; PASS 0 only)
    // 4: unused (always 0)
    TS_MMA_WAIT_FULL = 5,  // MMA issuer cycles waiting for B tiles
    TS_MMA_WAIT_EMPTY = 6, // MMA issuer cycles waiting for a drained accumulator
    TS_TMA_WAIT = 7,       // producer cycles waiting for a free stage
    TS_TILES = 8,          // (work item, B tile) pairs
    TS_PRUNE_CYCLES = 9,   // epilogue cycles spent in prunes
    // 10, 11: unused (always 0)
    TS_TOPK_ENTER = 12,    // register top-k: 32-column chunks with an entrant in some lane (per warp)
    TS_TOPK_BULK = 13,     // register top-k: chunks sorted and merged in bulk (per warp)
    TS_TOPK_INSERTS = 14,  // register top-k: one-by-one insertion rounds (per warp)
    TS_TOPK_ENTRANTS = 15, // register top-k: entrants (per lane)
    TS_COUNT = 16
};

__device__ __forceinline__ float f_of(uint32_t u) { return __uint_as_float(u); }

// The i-th column tile a work item visits: its home tile first, then tiles at
// growing distance alternately after and before it, within [ct0, ct1).  When
// rows are ordered so that nearby cells sit at nearby positions, the first
// tiles hold most of a row's neighbours and its threshold tightens at once.
__device__ __forceinline__ int sweep_tile(int i, int home, int ct0, int ct1) {
    const int hw = min(max(home, ct0), ct1 - 1);
    if (i == 0) return hw;
    const int L = hw - ct0, R = ct1 - 1 - hw;
    const int m = min(L, R);
    if (i <= 2 * m) {
        const int d = (i + 1) >> 1;
        return (i & 1) ? hw + d : hw - d;
    }
    return R > L ? hw + (i - m) : hw - (i - m);
}

// The column tiles of one work item in visiting order: its explicit list,
// or the outward sweep over [ct0, ct1).  The producer, the MMA issuer and
// the epilogue all derive the same count and sequence from it.
// TWO: the pass may carry a second list (collect passes only), compiled out
// of the others, whose registers are scarce.
template <bool TWO>
struct TileOrder {
    const uint32_t* list;
    const uint32_t* list2;
    int count, count1, home, ct0, ct1;

    __device__ __forceinline__ TileOrder(const TensorArgs& a, int w, int qt, int ct0_, int ct1_)
        : list(nullptr), list2(nullptr), count(ct1_ - ct0_), count1(0), home(qt * ROWS / TBN), ct0(ct0_),
          ct1(ct1_) {
        if (a.tl) {
            // An explicit list holds distinct column tiles from anywhere in
            // the reference (a column segment's list is not confined to the
            // segment's own range).
            list = a.tl + (a.tl_off ? (int64_t)a.tl_off[w] : (int64_t)w * a.tl_stride);
            count = count1 = (int)min(a.tl_cnt[w], (uint32_t)a.col_tiles);
            if (TWO && a.tl2) {
                list2 = a.tl2 + (int64_t)w * a.tl2_stride;
                count += (int)min(a.tl2_cnt[w], (uint32_t)(a.col_tiles - count1));
            }
        }
    }
    __device__ __forceinline__ int next(int it) const {
        if (!list) return sweep_tile(it, home, ct0, ct1);
        if (!TWO) return (int)list[it];
        return it < count1 ? (int)list[it] : (int)list2[it - count1];
    }
};

// The j-th work item of this CTA, or -1.  Round robin over the items; with
// an item order (items by decreasing work) a snake over it: the CTAs take
// the heaviest items first, alternately in forward and reverse CTA order,
// which balances the CTAs' totals.  Every role of the CTA derives the same
// sequence.
__device__ __forceinline__ int item_at(const TensorArgs& a, int j) {
    const int G = gridDim.x, c = blockIdx.x;
    const int64_t pos = (int64_t)j * G + (a.item_order && (j & 1) ? G - 1 - c : c);
    if (pos >= a.items) return -1;
    return a.item_order ? (int)a.item_order[pos] : (int)pos;
}

__device__ __forceinline__ unsigned long long ld_shared_volatile_u64(uint32_t addr) {
    unsigned long long v;
    asm volatile("ld.volatile.shared.u64 %0, [%1];" : "=l"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ void st_shared_volatile_u64(uint32_t addr, unsigned long long v) {
    asm volatile("st.volatile.shared.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

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

// The columns of a 32-column chunk below th, as a mask in an interleaved bit
// order (below_col decodes it).  Each difference v - th is formed on the FMA
// pipe; a byte permute replicates the signs of two differences into bytes,
// and one logic op merges them into the mask: 32 ALU-pipe instructions a
// chunk where a compare and a select per column take 64.  v < th exactly
// when v - th is negative (the difference of two distinct floats is never
// zero).
__device__ __forceinline__ uint32_t below_mask(const uint32_t (&v)[32], float th) {
    uint32_t acc = 0;
#pragma unroll
    for (int p = 0; p < 16; ++p) {
        const uint32_t d0 = __float_as_uint(__fsub_rn(f_of(v[2 * p]), th));
        const uint32_t d1 = __float_as_uint(__fsub_rn(f_of(v[2 * p + 1]), th));
        uint32_t y;  // bytes: sign(d0), sign(d1), sign(d0), sign(d1), each 0x00 or 0xff
        asm("prmt.b32 %0, %1, %2, 0xFBFB;" : "=r"(y) : "r"(d0), "r"(d1));
        acc |= y & ((0x0101u << (p & 7)) << (p >= 8 ? 16 : 0));
    }
    return acc;
}
// The chunk column of bit b of a below_mask: column 2p + i sits in byte
// i + 2 (p / 8), bit p % 8.
__device__ __forceinline__ int below_col(int b) { return 2 * ((b & 7) | ((b >> 4) << 3)) + ((b >> 3) & 1); }

// Appends the columns of one 32-column chunk that pass the row's threshold.
// `valid` masks out columns past the reference rows and the row itself.  The
// survivors' slots come from prefix popcounts of the mask, so the stores are
// independent of one another.
__device__ __forceinline__ void append_chunk(const uint32_t (&v)[32], int64_t colbase, float th, uint32_t valid,
                                             uint32_t* ids, float* vals, uint32_t& cnt) {
    uint32_t mask = 0;
#pragma unroll
    for (int j = 0; j < 32; j++) mask |= (f_of(v[j]) < th) ? (1u << j) : 0u;
    mask &= valid;
#pragma unroll
    for (int j = 0; j < 32; j++) {
        if (mask & (1u << j)) {
            const uint32_t pos = cnt + __popc(mask & ((1u << j) - 1u));
            ids[pos] = (uint32_t)(colbase + j);
            vals[pos] = f_of(v[j]);
        }
    }
    cnt += __popc(mask);
}

// Columns of the chunk starting at colbase that may be appended: below nr and
// not the row itself.
__device__ __forceinline__ uint32_t chunk_valid(int64_t colbase, int64_t nr, bool self, int64_t row) {
    uint32_t m = 0xffffffffu;
    if (colbase + 32 > nr) m = colbase >= nr ? 0u : ((1u << (uint32_t)(nr - colbase)) - 1u);
    if (self && row >= colbase && row < colbase + 32) m &= ~(1u << (uint32_t)(row - colbase));
    return m;
}


// Tests one 32-column chunk against the row's threshold; survivors are rare,
// so the warp branches once and lanes without survivors append an empty mask.
__device__ __forceinline__ void test_chunk(const uint32_t (&v)[32], int64_t colbase, float th, int64_t row,
                                           const TensorArgs& a, uint32_t* ids, float* vals, uint32_t& cnt) {
    const float m = min32(v);
    if (__any_sync(0xffffffffu, m < th))
        append_chunk(v, colbase, th, chunk_valid(colbase, a.nr, a.self != 0, row + a.self_offset), ids, vals, cnt);
}

// The K smallest values a lane has met (k <= K), ascending, in registers.
// With it a lane's threshold follows its k-th smallest value chunk by chunk,
// so its lists only receive columns inside the current bound and a prune is
// a compaction, never a selection.
template <int K>
struct TopK {
    float v[K];
    // The first K - k slots hold -inf, so v[K-1] is always the k-th
    // smallest value met (+inf until k values have been met).
    __device__ __forceinline__ void reset(int k) {
#pragma unroll
        for (int j = 0; j < K; j++) v[j] = j < K - k ? __int_as_float(0xff800000) : __int_as_float(0x7f800000);
    }
    // x below v[K-1]: the larger entries shift up by one.  With v ascending,
    // the new v[j] is min(v[j], max(v[j-1], x)): two independent min/max per
    // slot, no compare-and-select chain.
    __device__ __forceinline__ void insert(float x) {
#pragma unroll
        for (int j = K - 1; j > 0; j--) v[j] = fminf(v[j], fmaxf(v[j - 1], x));
        v[0] = fminf(v[0], x);
    }
    __device__ __forceinline__ float kth() const { return v[K - 1]; }
    // Merges N ascending values in: the K smallest of both, ascending (the
    // N values padded to K with +inf, against the reversed run, then the
    // bitonic clean-up).
    template <int N>
    __device__ __forceinline__ void merge_few(const float (&g)[N]) {
        static_assert(K >= N, "merge_few needs at least N slots");
#pragma unroll
        for (int t = 0; t < N; t++) v[K - N + t] = fminf(v[K - N + t], g[N - 1 - t]);
        clean_up();
    }
    // Bitonic clean-up of v into ascending order.
    __device__ __forceinline__ void clean_up() {
#pragma unroll
        for (int stride = K >> 1; stride > 0; stride >>= 1)
#pragma unroll
            for (int i = 0; i < K; i++) {
                const int j = i ^ stride;
                if (j > i) {
                    const float lo = fminf(v[i], v[j]), hi = fmaxf(v[i], v[j]);
                    v[i] = lo;
                    v[j] = hi;
                }
            }
    }
    // Merges 32 ascending values in (f32 bit patterns): the K smallest of
    // both, ascending (the elementwise minimum against the reversed run is
    // bitonic; a bitonic clean-up sorts it).
    __device__ __forceinline__ void merge_sorted(const uint32_t (&x)[32]) {
        static_assert(K <= 32, "merge_sorted holds at most 32 values");
#pragma unroll
        for (int i = 0; i < K; i++) v[i] = fminf(v[i], __uint_as_float(x[K - 1 - i]));
        clean_up();
    }
};

#define SCRUST_CAS(i, j)                                            \
    {                                                               \
        const float lo_ = fminf(g[i], g[j]), hi_ = fmaxf(g[i], g[j]); \
        g[i] = lo_;                                                 \
        g[j] = hi_;                                                 \
    }
// Ascending sort of eight values in registers (a 19-comparator network).
__device__ __forceinline__ void sort8(float (&g)[8]) {
    SCRUST_CAS(0, 1) SCRUST_CAS(2, 3) SCRUST_CAS(4, 5) SCRUST_CAS(6, 7)
    SCRUST_CAS(0, 2) SCRUST_CAS(1, 3) SCRUST_CAS(4, 6) SCRUST_CAS(5, 7)
    SCRUST_CAS(1, 2) SCRUST_CAS(5, 6) SCRUST_CAS(0, 4) SCRUST_CAS(3, 7)
    SCRUST_CAS(1, 5) SCRUST_CAS(2, 6) SCRUST_CAS(1, 4) SCRUST_CAS(3, 6)
    SCRUST_CAS(2, 4) SCRUST_CAS(3, 5) SCRUST_CAS(3, 4)
}
// Ascending sort of four values (five comparators).
__device__ __forceinline__ void sort4(float (&g)[4]) {
    SCRUST_CAS(0, 1) SCRUST_CAS(2, 3) SCRUST_CAS(0, 2) SCRUST_CAS(1, 3) SCRUST_CAS(1, 2)
}
#undef SCRUST_CAS

// Whether no column of the part's 128 columns from col0 is past the
// reference rows or the row itself, for the whole warp (one vote per tile
// instead of a column mask per chunk).
__device__ __forceinline__ bool tile_clean(int64_t col0, int64_t row, const TensorArgs& a) {
    const int64_t self_col = row + a.self_offset;
    return !__any_sync(0xffffffffu, col0 + kPartCols > a.nr || (a.self && self_col >= col0 && self_col < col0 + kPartCols));
}

// Columns past the reference rows and the row itself become +inf, so that
// no group minimum is taken over them (they occur in at most two chunks of
// a work item: the warp branches once).
__device__ __forceinline__ void mask_chunk(uint32_t (&v)[32], int64_t colbase, int64_t row, const TensorArgs& a) {
    const uint32_t valid = chunk_valid(colbase, a.nr, a.self != 0, row + a.self_offset);
    if (__any_sync(0xffffffffu, valid != 0xffffffffu)) {
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = ((valid >> j) & 1u) ? v[j] : 0x7f800000u;
    }
}

// The minima of a chunk's four 8-column groups.
__device__ __forceinline__ void quarter_mins(uint32_t (&v)[32], int64_t colbase, int64_t row, const TensorArgs& a,
                                             float (&g)[4]) {
    mask_chunk(v, colbase, row, a);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int b = 8 * q;
        g[q] = min3f(min3f(f_of(v[b]), f_of(v[b + 1]), f_of(v[b + 2])),
                     min3f(f_of(v[b + 3]), f_of(v[b + 4]), f_of(v[b + 5])), fminf(f_of(v[b + 6]), f_of(v[b + 7])));
    }
}

// Nearest-group pass: the minimum of each 8-column group of the chunk; the
// lane keeps the smallest group minimum it has met and that group's index
// (column / 8).  The row's nearest column is found among the group's eight
// columns afterwards, which saves carrying a column with every value.
// Columns past the reference rows (and the row itself) become +inf first.
__device__ __forceinline__ void group_argmin_chunk(uint32_t (&v)[32], int64_t colbase, int64_t row,
                                                   const TensorArgs& a, bool clean, float& best_v,
                                                   uint32_t& best_g) {
    if (!clean) mask_chunk(v, colbase, row, a);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int b = 8 * q;
        const float g = min3f(min3f(f_of(v[b]), f_of(v[b + 1]), f_of(v[b + 2])),
                              min3f(f_of(v[b + 3]), f_of(v[b + 4]), f_of(v[b + 5])), fminf(f_of(v[b + 6]), f_of(v[b + 7])));
        if (g < best_v) {
            best_v = g;
            best_g = (uint32_t)(colbase >> 3) + (uint32_t)q;
        }
    }
}

// The minima of a chunk's eight 4-column groups.
__device__ __forceinline__ void eighth_mins(uint32_t (&v)[32], int64_t colbase, int64_t row, const TensorArgs& a,
                                            float (&g)[8]) {
    mask_chunk(v, colbase, row, a);
#pragma unroll
    for (int q = 0; q < 8; q++)
        g[q] = fminf(min3f(f_of(v[4 * q]), f_of(v[4 * q + 1]), f_of(v[4 * q + 2])), f_of(v[4 * q + 3]));
}

// The minima of a chunk's two 16-column halves.
__device__ __forceinline__ void half_mins(uint32_t (&v)[32], int64_t colbase, int64_t row, const TensorArgs& a,
                                          float& lo, float& hi) {
    mask_chunk(v, colbase, row, a);
    float m[12];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int b = 16 * h;
#pragma unroll
        for (int i = 0; i < 5; i++) m[6 * h + i] = min3f(f_of(v[b + 3 * i]), f_of(v[b + 3 * i + 1]), f_of(v[b + 3 * i + 2]));
        m[6 * h + 5] = f_of(v[b + 15]);
    }
    lo = fminf(min3f(m[0], m[1], m[2]), min3f(m[3], m[4], m[5]));
    hi = fminf(min3f(m[6], m[7], m[8]), min3f(m[9], m[10], m[11]));
}

// Ascending bitonic sort of 32 f32 values held as bit patterns in
// registers, in place (fully unrolled, static indices).
__device__ __forceinline__ void sort32(uint32_t (&x)[32]) {
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1)
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1)
#pragma unroll
            for (int i = 0; i < 32; i++) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const float a = __uint_as_float(x[i]), b = __uint_as_float(x[j]);
                    const float lo = fminf(a, b), hi = fmaxf(a, b);
                    x[i] = __float_as_uint(up ? lo : hi);
                    x[j] = __float_as_uint(up ? hi : lo);
                }
            }
}

// v[j] for a lane-varying j, by a five-level select tree (short dependency
// chains; the register array keeps static indices).
__device__ __forceinline__ float pick32(const uint32_t (&v)[32], int j) {
    uint32_t t[16];
#pragma unroll
    for (int q = 0; q < 16; q++) t[q] = (j & 1) ? v[2 * q + 1] : v[2 * q];
#pragma unroll
    for (int q = 0; q < 8; q++) t[q] = (j & 2) ? t[2 * q + 1] : t[2 * q];
#pragma unroll
    for (int q = 0; q < 4; q++) t[q] = (j & 4) ? t[2 * q + 1] : t[2 * q];
#pragma unroll
    for (int q = 0; q < 2; q++) t[q] = (j & 8) ? t[2 * q + 1] : t[2 * q];
    return f_of((j & 16) ? t[1] : t[0]);
}

// A chunk's columns below the lane's K-th smallest so far enter its top-K,
// and the threshold follows the k-th smallest.  Returns the chunk minimum.
// Appending is left to a second look at the tile, once the whole tile has
// tightened the threshold.
template <int K>
__device__ __forceinline__ float topk_chunk(uint32_t (&v)[32], int64_t colbase, float& th, int64_t row,
                                            const TensorArgs& a, TopK<K>& top, const TensorBound& bnd,
                                            uint32_t& best, bool keep_threshold = true) {
    const float m = min32(v);
    if constexpr (K == 1) {
        // The chunk minimum is the only candidate; its column is kept too.
        if (__any_sync(0xffffffffu, m < top.v[0])) {
            const uint32_t valid = chunk_valid(colbase, a.nr, a.self != 0, row + a.self_offset);
            float mv = m;
            if (valid != 0xffffffffu) {
                mv = __int_as_float(0x7f800000);
#pragma unroll
                for (int j = 0; j < 32; j++)
                    if ((valid >> j) & 1u) mv = fminf(mv, f_of(v[j]));
            }
            if (mv < top.v[0]) {
                // The first valid column holding the minimum.
                uint32_t eq = 0;
#pragma unroll
                for (int j = 0; j < 32; j++) eq |= (f_of(v[j]) == mv) ? (1u << j) : 0u;
                const int jj = __ffs(eq & valid) - 1;
                top.v[0] = mv;
                best = (uint32_t)(colbase + jj);
                if (keep_threshold) th = fminf(th, bnd.theta_f32(mv));
            }
        }
        return m;
    }
    // A column at or above the row's current threshold can neither be one of
    // its k nearest nor lower the threshold, so it is not an entrant either.
    if (__any_sync(0xffffffffu, m < fminf(top.kth(), th))) {
        const float lim = fminf(top.kth(), th);
        const uint32_t valid = chunk_valid(colbase, a.nr, a.self != 0, row + a.self_offset);
        uint32_t want = 0;
#pragma unroll
        for (int j = 0; j < 32; j++) want |= (f_of(v[j]) < lim) ? (1u << j) : 0u;
        want &= valid;
        const uint32_t most = __reduce_max_sync(0xffffffffu, (uint32_t)__popc(want));
        if (a.stats) {
            const uint32_t all = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(want));
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(a.stats + TS_TOPK_ENTER, 1ull);
                atomicAdd(a.stats + (most >= 9u ? TS_TOPK_BULK : TS_TOPK_INSERTS),
                          (unsigned long long)(most >= 9u ? 1u : most));
                atomicAdd(a.stats + TS_TOPK_ENTRANTS, (unsigned long long)all);
            }
        }
        // Many entrants in some lane (the first chunks of a row block): sort
        // the chunk and merge it in, with the warp converged; few: insert
        // them one by one.
        if (most >= 9u) {
            // The chunk is not needed after this: sort it in place.
#pragma unroll
            for (int j = 0; j < 32; j++) v[j] = ((want >> j) & 1u) ? v[j] : 0x7f800000u;
            sort32(v);
            top.merge_sorted(v);
        } else if (want) {
            while (want) {
                const int j = __ffs(want) - 1;
                want &= want - 1;
                const float x = pick32(v, j);
                if (x < top.kth()) top.insert(x);
            }
        }
        // (The threshold follows the k-th smallest once per tile, in the
        // caller: its f32 bound costs a directed square root.)
    }
    return m;
}

// Drops, in place, the entries of a lane's list at or above theta; eight
// entries are read before any is written back.
__device__ __forceinline__ uint32_t compact_lane(uint32_t* ids, float* vals, uint32_t cnt, float theta) {
    uint32_t out = 0;
#pragma unroll 1
    for (uint32_t e0 = 0; e0 < cnt; e0 += 8) {
        float x[8];
        uint32_t id[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const bool in = e0 + q < cnt;
            x[q] = in ? vals[e0 + q] : __int_as_float(0x7f800000);
            id[q] = in ? ids[e0 + q] : 0u;
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if (x[q] < theta) {
                ids[out] = id[q];
                vals[out] = x[q];
                out++;
            }
        }
    }
    return out;
}

// Applies a prune result to a lane's registers: a list that keeps `cap` or
// more entries inside its own threshold overflows to the exact fallback.
__device__ __forceinline__ void take_prune(const PruneResult& r, const TensorArgs& a, int64_t row, float& th,
                                           uint32_t& cnt, uint32_t& n_ovf) {
    if ((int)r.cnt >= a.lists.cap) {
        a.lists.overflow[row] = 1u;
        th = __int_as_float(0xff800000);
        cnt = 0;
        n_ovf++;
    } else {
        th = r.theta;
        cnt = r.cnt;
    }
}

// Prunes, with the whole warp, the lists of the lanes set in `need`; each
// lane keeps its own threshold and count in registers.
__device__ __forceinline__ void prune_lanes(uint32_t need, const TensorArgs& a, int seg, int64_t row,
                                            const TensorBound& bnd, float& th, uint32_t& cnt,
                                            uint32_t& n_ovf) {
    const int lane = threadIdx.x & 31;
    const int segs = a.lists.segments;
    while (need) {
        const int l = __ffs(need) - 1;
        need &= need - 1;
        const uint32_t lc = __shfl_sync(0xffffffffu, cnt, l);
        const float lth = __shfl_sync(0xffffffffu, th, l);
        const TensorBound lb{__shfl_sync(0xffffffffu, bnd.A, l), __shfl_sync(0xffffffffu, bnd.delta, l),
                             __shfl_sync(0xffffffffu, bnd.eps2, l)};
        const int64_t lrow = __shfl_sync(0xffffffffu, row, l);
        const int64_t off = (lrow * segs + seg) * (int64_t)a.lists.ctot;  // seg: list slot within the row
        const PruneResult r =
            prune_core(a.lists.ids + off, a.lists.vals + off, min(lc, (uint32_t)a.lists.ctot), a.k, lb, lth);
        if (lane == l) take_prune(r, a, row, th, cnt, n_ovf);
    }
}

// TOPK = K (k <= K, K = 1, 16 or 32): thresholds from a register top-K per
// lane (TopK); TOPK = 0: from warp-cooperative selections over the lists.
template <int TOPK, int PASS>
__global__ void __launch_bounds__(THREADS, 1)
    tensor_candidates_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                             TensorArgs a) {
    // PASS fixes the pass kind at compile time (1: thresholds only, 2:
    // collect for a self solve, 4: collect for query rows, 3: nearest column
    // group only, 0: taken from the arguments), so a
    // specialised pass carries none of the others' code or registers.
    // (A general pass with a register top-16 or top-32 never runs as a
    // threshold or collect pass: those have their own kinds.  Only k = 1 and
    // the top-k-free form take the pass kind from the arguments.)
    const bool thr_only = PASS == 1 || (PASS == 0 && TOPK <= 1 && a.thr_only);
    const bool collect = PASS == 2 || PASS == 4 || (PASS == 0 && TOPK <= 1 && a.collect);
    const bool argmin = PASS == 3 || (PASS == 0 && a.argmin_out != nullptr);
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = base;
    unsigned char* sB = base + 2 * A_BYTES;

    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], afull[2], aempty[2], tfull[HALVES],
        tempty[HALVES];
    __shared__ uint32_t tmem_slot;
    __shared__ unsigned long long theta_s[HALVES][PARTS][TBM];

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int segs = a.lists.segments;        // lists per row
    const int csegs = segs / PARTS;           // column segments

    // No item carries tag 0xffffffff: shared memory left by an earlier kernel
    // must never pass for a partner's threshold.
    for (int i = threadIdx.x; i < HALVES * PARTS * TBM; i += blockDim.x)
        (&theta_s[0][0][0])[i] = 0xffffffff00000000ull | 0x7f800000u;
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
            mbar_init(&tempty[h], EPI_WARPS / HALVES);  // one arrival per epilogue warp
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
            long long w_tma = 0;
            bool ok = true;
            for (int j = 0, w; ok && (w = item_at(a, j)) >= 0; ++j) {
                const int qt = w / csegs, seg = w % csegs;
                const int ct0 = a.item_range ? (int)a.item_range[w].x : seg * a.tiles_per_seg;
                const int ct1 = a.item_range ? (int)a.item_range[w].y : min(a.col_tiles, ct0 + a.tiles_per_seg);
                const TileOrder<PASS == 2 || PASS == 4 || PASS == 0> order(a, w, qt, ct0, ct1);
                if (order.count == 0) continue;
                const uint32_t ab = ac & 1, au = ac >> 1;
                if (!mbar_wait_bounded(&aempty[ab], (au & 1) ^ 1, a.err)) {
                    ok = false;
                    break;
                }
                mbar_arrive_expect_tx(&afull[ab], A_BYTES);
                tma_load_2d(sA + ab * A_BYTES, &ta, 0, qt * ROWS, &afull[ab]);
                ac++;
                for (int it = 0; it < order.count; ++it) {
                    const int ct = order.next(it);
                    const uint32_t st = sc % STAGES, su = sc / STAGES;
                    const long long t0 = a.stats ? clock64() : 0;
                    if (!mbar_wait_bounded(&empty[st], (su & 1) ^ 1, a.err)) {
                        ok = false;
                        break;
                    }
                    if (a.stats) w_tma += clock64() - t0;
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
            if (a.stats) atomicAdd(a.stats + TS_TMA_WAIT, (unsigned long long)w_tma);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t sc = 0, ac = 0, tc = 0;
            long long w_full = 0, w_empty = 0;
            bool ok = true;
            for (int j = 0, w; ok && (w = item_at(a, j)) >= 0; ++j) {
                const int qt = w / csegs, seg = w % csegs;
                const int ct0 = a.item_range ? (int)a.item_range[w].x : seg * a.tiles_per_seg;
                const int ct1 = a.item_range ? (int)a.item_range[w].y : min(a.col_tiles, ct0 + a.tiles_per_seg);
                const TileOrder<PASS == 2 || PASS == 4 || PASS == 0> order(a, w, qt, ct0, ct1);
                if (order.count == 0) continue;
                const uint32_t ab = ac & 1, au = ac >> 1;
                if (!mbar_wait_bounded(&afull[ab], au & 1, a.err)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a_base = smem_addr(sA + ab * A_BYTES);
                for (int it = 0; it < order.count && ok; ++it) {
                    const uint32_t st = sc % STAGES, su = sc / STAGES;
                    long long t0 = a.stats ? clock64() : 0;
                    if (!mbar_wait_bounded(&full[st], su & 1, a.err)) {
                        ok = false;
                        break;
                    }
                    if (a.stats) w_full += clock64() - t0;
                    tc_fence_after();
                    const uint32_t b_base = smem_addr(sB + st * B_BYTES);
                    for (int h = 0; h < HALVES; ++h) {
                        t0 = a.stats ? clock64() : 0;
                        if (!mbar_wait_bounded(&tempty[h], (tc & 1) ^ 1, a.err)) {
                            ok = false;
                            break;
                        }
                        if (a.stats) w_empty += clock64() - t0;
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
            if (a.stats) {
                atomicAdd(a.stats + TS_MMA_WAIT_FULL, (unsigned long long)w_full);
                atomicAdd(a.stats + TS_MMA_WAIT_EMPTY, (unsigned long long)w_empty);
                atomicAdd(a.stats + TS_TILES, (unsigned long long)tc);
            }
        }
    } else {
        // ---------------- epilogue ----------------
        const int e = warp - 2;
        const int h = e / (EPI_WARPS / HALVES);
        const int part = (e / 4) % PARTS;
        const int quarter = warp & 3;
        const int r_local = quarter * 32 + lane;
        const int cap = a.lists.cap;
        const int col_segs = csegs;
        // Shared-window addresses (32-bit) of this lane's and its partner's slot.
        const uint32_t my_th = smem_addr(&theta_s[h][part][r_local]);
        const uint32_t other_th = smem_addr(&theta_s[h][part ^ 1][r_local]);
        uint32_t tc = 0;
        uint32_t n_app = 0, n_prune = 0, n_ovf = 0;
        long long c_prune = 0, c_wait = 0;
        bool ok = true;
        for (int j = 0, w; ok && (w = item_at(a, j)) >= 0; ++j) {
            const int qt = w / col_segs, seg = w % col_segs;
            const int ct0 = a.item_range ? (int)a.item_range[w].x : seg * a.tiles_per_seg;
            const int ct1 = a.item_range ? (int)a.item_range[w].y : min(a.col_tiles, ct0 + a.tiles_per_seg);
            const TileOrder<PASS == 2 || PASS == 4 || PASS == 0> order(a, w, qt, ct0, ct1);
            if (order.count == 0) continue;
            const int64_t row = (int64_t)qt * ROWS + h * TBM + r_local;
            const bool valid = row < a.nq && (!a.row_map || a.row_map[row] != 0xffffffffu);
            float th = valid ? __int_as_float(0x7f800000) : __int_as_float(0xff800000);
            uint32_t cnt = 0;
            TensorBound bnd{0.f, 0.f, 0.f};
            if (valid) bnd = TensorBound{a.bA[row], a.bdelta[row], a.beps2[row]};
            const int64_t lslot = (row * col_segs + seg) * PARTS + part;
            if (valid && collect) {
                // The row's lists in this column segment are lslot and
                // lslot ^ 1; other segments' thresholds arrive through
                // row_theta below.
                th = fminf(a.theta_io[lslot], a.theta_io[lslot ^ 1]);
                if (a.resume) cnt = min(a.lists.cnt[lslot], (uint32_t)cap);
            } else if (valid && a.resume) {
                if (!thr_only) cnt = min(a.lists.cnt[lslot], (uint32_t)cap);  // below cap when an item ends
                th = a.theta_io[lslot];
            }
            uint32_t* ids = a.lists.ids + lslot * (int64_t)a.lists.ctot;
            float* vals = a.lists.vals + lslot * (int64_t)a.lists.ctot;
            const uint64_t tag = (uint64_t)(uint32_t)w << 32;
            st_shared_volatile_u64(my_th, tag | __float_as_uint(th));
            TopK<(TOPK > 0 ? TOPK : 1)> top;
            if constexpr (TOPK > 0) top.reset(TOPK == 1 ? 1 : a.k);
            uint32_t best = 0xffffffffu;
            for (int it = 0; it < order.count; ++it) {
                const int ct = order.next(it);
                // (Wait cycles are counted in the unspecialised passes only:
                // their registers are scarce in the threshold pass.)
                const long long w0 = (PASS == 0 && a.stats) ? clock64() : 0;
                if (!mbar_wait_bounded(&tfull[h], tc & 1, a.err)) {
                    ok = false;
                    break;
                }
                if (PASS == 0 && a.stats) c_wait += clock64() - w0;
                tc_fence_after();
                // The partner part's threshold bounds this row just as well,
                // and so does any other column segment's (through HBM).
                const unsigned long long o = ld_shared_volatile_u64(other_th);
                if ((o & 0xffffffff00000000ull) == tag) th = fminf(th, __uint_as_float((uint32_t)o));
                if (a.row_theta && valid) th = fminf(th, key_float(a.row_theta[row]));
                const int64_t col0 = (int64_t)ct * TBN + part * kPartCols;
                const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(h * TBN + part * kPartCols);
                const uint32_t before = cnt;
                const float th_before = th;
                if constexpr (TOPK > 0) {
                    // First look: the tile's columns update the top-K and the
                    // threshold.  Second look: chunks holding columns below
                    // the tightened threshold are read again and appended.
                    uint32_t va[32];
                    float cm[4];
                    if (collect) {
                        // At the final thresholds every column that passes is a
                        // candidate: only its id is kept (the rerank measures it
                        // again), and each lane loops over its own passes.
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            tmem_ld32(tbase + 32 * c, va);
                            tmem_ld_wait(va);
                            // A self solve's rows collect among their own
                            // cells, nearly every chunk holding some row's
                            // candidate: the mask is formed at once (PASS 2).
                            // Query rows meet many chunks with none: a
                            // minimum tree and a vote skip those (PASS 4).
                            if (PASS == 2 || __any_sync(0xffffffffu, min32(va) < th)) {
                                uint32_t mask = below_mask(va, th);
                                const int64_t cb = col0 + 32 * c;
                                while (mask) {
                                    const int64_t col = cb + below_col(__ffs(mask) - 1);
                                    mask &= mask - 1;
                                    // Not past the reference rows, not the row itself.
                                    if (col < a.nr && !(a.self && col == row + a.self_offset))
                                        ids[cnt++] = (uint32_t)col;  // ids only: no values
                                }
                            }
                        }
                    } else if constexpr (PASS == 3) {
                        const bool clean = tile_clean(col0, row, a);
                        uint32_t vb[32];
                        tmem_ld32(tbase, va);
                        tmem_ld_wait(va);
                        tmem_ld32(tbase + 32, vb);
                        group_argmin_chunk(va, col0, row, a, clean, top.v[0], best);
                        tmem_ld_wait(vb);
                        tmem_ld32(tbase + 64, va);
                        group_argmin_chunk(vb, col0 + 32, row, a, clean, top.v[0], best);
                        tmem_ld_wait(va);
                        tmem_ld32(tbase + 96, vb);
                        group_argmin_chunk(va, col0 + 64, row, a, clean, top.v[0], best);
                        tmem_ld_wait(vb);
                        group_argmin_chunk(vb, col0 + 96, row, a, clean, top.v[0], best);
                    } else if constexpr (TOPK == 16 && PASS == 1) {
                        // Threshold pass: each group of columns offers only
                        // its minimum.  The top-K then holds values of
                        // distinct columns, so its K-th is still an upper
                        // bound of the row's k-th smallest (slightly above it
                        // when two of the nearest share a group), and a tile
                        // costs a sort of its group minima and a merge instead
                        // of an insertion per entrant.  Groups of 8 on an
                        // item's first tile (16 minima per lane: the K-th is
                        // finite after one tile), of 16 after it.
                        const float kth0 = top.kth();
                        uint32_t vb[32];
                        if (it == 0) {
#pragma unroll 1
                            for (int c = 0; c < 4; ++c) {
                                float q[4];
                                tmem_ld32(tbase + 32 * c, va);
                                tmem_ld_wait(va);
                                quarter_mins(va, col0 + 32 * c, row, a, q);
                                cm[c] = fminf(fminf(q[0], q[1]), fminf(q[2], q[3]));
                                if (__any_sync(0xffffffffu, cm[c] < fminf(top.kth(), th))) {
                                    sort4(q);
                                    top.merge_few(q);
                                }
                            }
                            th = fminf(th, bnd.theta_f32(top.kth()));
                        } else {
                            float g[8];
                            tmem_ld32(tbase, va);
                            tmem_ld_wait(va);
                            tmem_ld32(tbase + 32, vb);
                            half_mins(va, col0, row, a, g[0], g[1]);
                            tmem_ld_wait(vb);
                            tmem_ld32(tbase + 64, va);
                            half_mins(vb, col0 + 32, row, a, g[2], g[3]);
                            tmem_ld_wait(va);
                            tmem_ld32(tbase + 96, vb);
                            half_mins(va, col0 + 64, row, a, g[4], g[5]);
                            tmem_ld_wait(vb);
                            half_mins(vb, col0 + 96, row, a, g[6], g[7]);
#pragma unroll
                            for (int c = 0; c < 4; ++c) cm[c] = fminf(g[2 * c], g[2 * c + 1]);
                            const float lim = fminf(top.kth(), th);
                            const float tmin = fminf(fminf(cm[0], cm[1]), fminf(cm[2], cm[3]));
                            if (__any_sync(0xffffffffu, tmin < lim)) {
                                if (a.stats) {
                                    uint32_t in = 0;
#pragma unroll
                                    for (int t = 0; t < 8; t++) in += g[t] < lim ? 1u : 0u;
                                    const uint32_t all = __reduce_add_sync(0xffffffffu, in);
                                    if (lane == 0) {
                                        atomicAdd(a.stats + TS_TOPK_ENTER, 1ull);
                                        atomicAdd(a.stats + TS_TOPK_BULK, 1ull);
                                        atomicAdd(a.stats + TS_TOPK_ENTRANTS, (unsigned long long)all);
                                    }
                                }
                                sort8(g);
                                top.merge_few(g);
                            }
                            if (top.kth() < kth0) th = fminf(th, bnd.theta_f32(top.kth()));
                        }
                    } else if constexpr (TOPK == 32 && PASS == 1) {
                        // The same for a top-32: groups of 4 on an item's
                        // first tile (32 minima per lane), of 16 after it; one
                        // chunk in flight (a top-32 leaves no registers for
                        // two).
                        const float kth0 = top.kth();
                        if (it == 0) {
#pragma unroll 1
                            for (int c = 0; c < 4; ++c) {
                                float q[8];
                                tmem_ld32(tbase + 32 * c, va);
                                tmem_ld_wait(va);
                                eighth_mins(va, col0 + 32 * c, row, a, q);
                                cm[c] = fminf(fminf(fminf(q[0], q[1]), fminf(q[2], q[3])),
                                              fminf(fminf(q[4], q[5]), fminf(q[6], q[7])));
                                if (__any_sync(0xffffffffu, cm[c] < fminf(top.kth(), th))) {
                                    sort8(q);
                                    top.merge_few(q);
                                }
                            }
                            th = fminf(th, bnd.theta_f32(top.kth()));
                        } else {
                            float g[8];
#pragma unroll
                            for (int c = 0; c < 4; ++c) {
                                tmem_ld32(tbase + 32 * c, va);
                                tmem_ld_wait(va);
                                half_mins(va, col0 + 32 * c, row, a, g[2 * c], g[2 * c + 1]);
                                cm[c] = fminf(g[2 * c], g[2 * c + 1]);
                            }
                            const float tmin = fminf(fminf(cm[0], cm[1]), fminf(cm[2], cm[3]));
                            if (__any_sync(0xffffffffu, tmin < fminf(top.kth(), th))) {
                                sort8(g);
                                top.merge_few(g);
                            }
                            if (top.kth() < kth0) th = fminf(th, bnd.theta_f32(top.kth()));
                        }
                    } else if constexpr (TOPK <= 16) {
                        const float kth0 = top.kth();
                        uint32_t vb[32];
                        tmem_ld32(tbase, va);
                        tmem_ld_wait(va);
                        tmem_ld32(tbase + 32, vb);
                        cm[0] = topk_chunk(va, col0, th, row, a, top, bnd, best, !argmin);
                        tmem_ld_wait(vb);
                        tmem_ld32(tbase + 64, va);
                        cm[1] = topk_chunk(vb, col0 + 32, th, row, a, top, bnd, best, !argmin);
                        tmem_ld_wait(va);
                        tmem_ld32(tbase + 96, vb);
                        cm[2] = topk_chunk(va, col0 + 64, th, row, a, top, bnd, best, !argmin);
                        tmem_ld_wait(vb);
                        cm[3] = topk_chunk(vb, col0 + 96, th, row, a, top, bnd, best, !argmin);
                        if (TOPK > 1 && top.kth() < kth0) th = fminf(th, bnd.theta_f32(top.kth()));
                    } else {
                        // A top-32 leaves no registers for a second chunk in flight.
                        const float kth0 = top.kth();
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            tmem_ld32(tbase + 32 * c, va);
                            tmem_ld_wait(va);
                            cm[c] = topk_chunk(va, col0 + 32 * c, th, row, a, top, bnd, best, !argmin);
                        }
                        if (top.kth() < kth0) th = fminf(th, bnd.theta_f32(top.kth()));
                    }
                    const unsigned long long o2 = ld_shared_volatile_u64(other_th);
                    if ((o2 & 0xffffffff00000000ull) == tag) th = fminf(th, __uint_as_float((uint32_t)o2));
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        if (!collect && !thr_only && !argmin && __any_sync(0xffffffffu, cm[c] < th)) {
                            tmem_ld32(tbase + 32 * c, va);
                            tmem_ld_wait(va);
                            append_chunk(va, col0 + 32 * c, th,
                                         chunk_valid(col0 + 32 * c, a.nr, a.self != 0, row + a.self_offset), ids, vals, cnt);
                        }
                    }
                } else {
                    // Four 32-column chunks; each TMEM load overlaps the
                    // previous chunk's threshold test.
                    uint32_t va[32], vb[32];
                    tmem_ld32(tbase, va);
                    tmem_ld_wait(va);
                    tmem_ld32(tbase + 32, vb);
                    test_chunk(va, col0, th, row, a, ids, vals, cnt);
                    tmem_ld_wait(vb);
                    tmem_ld32(tbase + 64, va);
                    test_chunk(vb, col0 + 32, th, row, a, ids, vals, cnt);
                    tmem_ld_wait(va);
                    tmem_ld32(tbase + 96, vb);
                    test_chunk(va, col0 + 64, th, row, a, ids, vals, cnt);
                    tmem_ld_wait(vb);
                    test_chunk(vb, col0 + 96, th, row, a, ids, vals, cnt);
                }
                // Release the accumulator before any prune, so the tensor
                // core refills it while this warp prunes.
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty[h]);
                n_app += cnt - before;
                const uint32_t need = __ballot_sync(0xffffffffu, cnt >= (uint32_t)cap);
                if (need) {
                    const long long p0 = a.stats ? clock64() : 0;
                    n_prune += __popc(need);
                    if constexpr (TOPK > 0) {
                        // A collected list holds only columns below its fixed
                        // threshold (and no values): nothing to compact.
                        if (cnt >= (uint32_t)cap)
                            take_prune(PruneResult{th, collect ? min(cnt, (uint32_t)a.lists.ctot)
                                                               : compact_lane(ids, vals, min(cnt, (uint32_t)a.lists.ctot), th)},
                                       a, row, th, cnt, n_ovf);
                        __syncwarp();
                    } else {
                        prune_lanes(need, a, seg * PARTS + part, row, bnd, th, cnt, n_ovf);
                    }
                    if (a.stats) c_prune += clock64() - p0;
                }
                if (__any_sync(0xffffffffu, th != th_before)) {
                    st_shared_volatile_u64(my_th, tag | __float_as_uint(th));
                    if (a.row_theta && valid && th < th_before) atomicMin(a.row_theta + row, float_key(th));
                }
                tc++;
            }
            // A last prune keeps every finished list short enough for the
            // union of a row's lists to fit the rerank.
            if (ok) {
                const uint32_t need = __ballot_sync(0xffffffffu, cnt > (uint32_t)a.final_cap);
                if (need) {
                    const long long p0 = a.stats ? clock64() : 0;
                    n_prune += __popc(need);
                    if constexpr (TOPK > 0) {
                        if (cnt > (uint32_t)a.final_cap)
                            take_prune(PruneResult{th, collect ? min(cnt, (uint32_t)a.lists.ctot)
                                                               : compact_lane(ids, vals, min(cnt, (uint32_t)a.lists.ctot), th)},
                                       a, row, th, cnt, n_ovf);
                        __syncwarp();
                    } else {
                        prune_lanes(need, a, seg * PARTS + part, row, bnd, th, cnt, n_ovf);
                    }
                    if (a.stats) c_prune += clock64() - p0;
                }
            }
            if (argmin) {
                if (valid && ok)
                    a.argmin_out[row * PARTS + part] =
                        ((unsigned long long)float_key(top.v[0]) << 32) | (unsigned long long)best;
                continue;
            }
            if (valid && ok) {
                if (!thr_only) a.lists.cnt[lslot] = min(cnt, (uint32_t)a.lists.ctot);
                if (a.theta_io && !collect) a.theta_io[lslot] = th;
                if constexpr (TOPK > 1) {
                    if (thr_only && a.topk_out) {
#pragma unroll
                        for (int t = 0; t < TOPK; ++t) a.topk_out[t * a.topk_stride + lslot] = top.v[t];
                    }
                }
            }
        }
        if (a.stats) {
            unsigned long long s_app = n_app, s_ovf = n_ovf;
            for (int o = 16; o > 0; o >>= 1) {
                s_app += __shfl_xor_sync(0xffffffffu, s_app, o);
                s_ovf += __shfl_xor_sync(0xffffffffu, s_ovf, o);
            }
            if (lane == 0) {
                atomicAdd(a.stats + TS_APPENDS, s_app);
                atomicAdd(a.stats + TS_OVERFLOWS, s_ovf);
                atomicAdd(a.stats + TS_PRUNES, (unsigned long long)n_prune);
                atomicAdd(a.stats + TS_PRUNE_CYCLES, (unsigned long long)c_prune);
                atomicAdd(a.stats + TS_EPI_WAIT, (unsigned long long)c_wait);
            }
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
__device__ __forceinline__ float f32_of(__half v) { return __half2float(v); }
__device__ __forceinline__ float f32_of(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ uint32_t bits16(__half v) { return (uint32_t)__half_as_ushort(v); }
__device__ __forceinline__ uint32_t bits16(__nv_bfloat16 v) { return (uint32_t)__bfloat16_as_ushort(v); }

// One thread per padded row: writes A_i and B_i of input row perm[i] (a
// padding row where perm[i] is 0xffffffff or i >= n) (64 16-bit values each), the
// quantised squared norm A = |a_hat|^2, the per-row error radius
// eps = |a_hat - scale*c| + scale*u*|c| (+ scale*u for normalised rows), and
// the running maxima of eps and |b_hat|.
//
// All in f32.  Rows are centred on the f32-rounded column means (the same
// centre for every row and query, so no distance depends on it).  A square
// of a 16-bit value is exact in f32, and |a_hat|^2 is summed as an
// unevaluated pair (two-sum), so its three-part split is as close as an f64
// sum's.  Sums of rounded non-negative terms are scaled up past their
// rounding and every step of a bound is rounded upwards.
template <class T>
__global__ void __launch_bounds__(128) tensor_operands_kernel(const float* __restrict__ x, int64_t n, int64_t n_pad, int d,
                                       const double* __restrict__ means, const uint32_t* __restrict__ max_norm_bits,
                                       int cosine, const uint32_t* __restrict__ perm, T* __restrict__ A16,
                                       T* __restrict__ B16,
                                       float* __restrict__ bA, float* __restrict__ eps,
                                       uint32_t* __restrict__ max_eps_bits, uint32_t* __restrict__ max_bhat_bits) {
    __shared__ float mean32[TK];
    for (int t = threadIdx.x; t < d; t += blockDim.x) mean32[t] = __double2float_rn(means[t]);
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    const float M = __uint_as_float(*max_norm_bits);
    // Power-of-two scale so every |scale * c| <= 64 (and |b_hat|^2 < 65504).
    int sexp = M > 0.f ? (int)floorf(log2f(64.0f / M)) : 0;
    sexp = max(-100, min(100, sexp));
    const float scale = ldexpf(1.0f, sexp);
    // Rows are built as packed 16-bit pairs in registers (static indices
    // only): aw[w] holds columns 2w and 2w + 1.
    uint32_t aw[TK / 2], bw[TK / 2];
    const bool real = i < n && (!perm || perm[i] != 0xffffffffu);
    const uint32_t one = bits16(to16<T>(1.0f));
    if (real) {
        const int64_t src = perm ? (int64_t)perm[i] : i;
        const float* xr = x + src * d;
        float hs = 0.f, hl = 0.f, e2 = 0.f, c2 = 0.f;
#pragma unroll
        for (int w = 0; w < TK / 2; w++) {
            uint32_t pa = 0u, pb = 0u;
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int t = 2 * w + hh;
                if (t < d) {
                    const float c = __fsub_rn(__ldg(xr + t), mean32[t]);
                    const float y = c * scale;
                    const T q = to16<T>(y);
                    const float qf = f32_of(q);
                    pa |= bits16(q) << (16 * hh);
                    pb |= bits16(to16<T>(-2.0f * qf)) << (16 * hh);
                    const float sq = __fmul_rn(qf, qf);  // exact: at most 22 significant bits
                    const float sum = __fadd_rn(hs, sq), bv = __fsub_rn(sum, hs);
                    hl = __fadd_rn(hl, __fadd_rn(__fsub_rn(hs, __fsub_rn(sum, bv)), __fsub_rn(sq, bv)));
                    hs = sum;
                    const float err = __fsub_rn(qf, y);  // exact: q is y rounded
                    e2 = __fmaf_rn(err, err, e2);
                    c2 = __fmaf_rn(c, c, c2);
                }
            }
            aw[w] = pa;
            bw[w] = pb;
        }
        // |a_hat|^2 = h + hlo, then n1 + n2 + n3 (each difference below is
        // exact: a value less its own 16-bit rounding).
        const float h = __fadd_rn(hs, hl), hlo = __fsub_rn(hl, __fsub_rn(h, hs));
        const T n1 = to16<T>(h);
        const float r1 = __fadd_rn(__fsub_rn(h, f32_of(n1)), hlo);
        const T n2 = to16<T>(r1);
        const float r2 = __fsub_rn(r1, f32_of(n2));
        const T n3 = to16<T>(r2);
        // Columns d .. d + 2: ones in A, the split norm in B.
#pragma unroll
        for (int w = 0; w < TK / 2; w++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int t = 2 * w + hh;
                const int k3 = t - d;
                if (k3 >= 0 && k3 < 3) {
                    const uint32_t nb = bits16(k3 == 0 ? n1 : (k3 == 1 ? n2 : n3));
                    aw[w] |= one << (16 * hh);
                    bw[w] |= nb << (16 * hh);
                }
            }
        bA[i] = h;
        const float grow = 1.0f + (float)(d + 4) * 1.1920929e-07f;
        const float ku = __fmul_ru(__fmul_ru(1.01f, scale), 5.9604645e-08f);
        float ep = __fadd_ru(__fsqrt_ru(__fmul_ru(e2, grow)), __fmul_ru(ku, __fsqrt_ru(__fmul_ru(c2, grow))));
        if (cosine) ep = __fadd_ru(ep, ku);
        ep = __fadd_ru(ep, 1e-30f);
        eps[i] = ep;
        atomicMax(max_eps_bits, __float_as_uint(ep));
        atomicMax(max_bhat_bits, __float_as_uint(__fmul_ru(__fsqrt_ru(__fadd_ru(hs, hl)), 1.0f + 1e-6f)));
    } else {
        // Padding: a reference row whose value against any query is +inf,
        // so it can never become a candidate (and a query row with the same
        // ones as a real row, so that no product is 0 * inf).
        const uint32_t inf = bits16(to16<T>(__int_as_float(0x7f800000)));
#pragma unroll
        for (int w = 0; w < TK / 2; w++) {
            uint32_t pa = 0u, pb = 0u;
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int k3 = 2 * w + hh - d;
                if (k3 >= 0 && k3 < 3) pa |= one << (16 * hh);
                if (k3 == 0) pb |= inf << (16 * hh);
            }
            aw[w] = pa;
            bw[w] = pb;
        }
        bA[i] = 0.f;
        eps[i] = 0.f;
    }
    uint4* ad = reinterpret_cast<uint4*>(A16 + i * TK);
    uint4* bd = reinterpret_cast<uint4*>(B16 + i * TK);
#pragma unroll
    for (int q = 0; q < TK / 8; q++) {
        ad[q] = make_uint4(aw[4 * q], aw[4 * q + 1], aw[4 * q + 2], aw[4 * q + 3]);
        bd[q] = make_uint4(bw[4 * q], bw[4 * q + 1], bw[4 * q + 2], bw[4 * q + 3]);
    }
}

// delta: bound on the FP32 accumulation error of the 64-term MMA chain,
// 8 * 64 * 2^-24 * (2 |a_hat| Mb + Mb^2 + 3), plus the rounding of A to f32
// and the residual of the three-part 16-bit split of |b_hat|^2 (at most
// 2^-24 |b_hat|^2 for bf16 parts, far less for fp16); eps2 = 2 (eps_i + E).
// Every step rounded upwards.
__global__ void tensor_bounds_kernel(int64_t n, const float* __restrict__ bA, const float* __restrict__ eps,
                                     const uint32_t* __restrict__ max_eps_bits,
                                     const uint32_t* __restrict__ max_bhat_bits, float* __restrict__ bdelta,
                                     float* __restrict__ beps2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float Mb = __uint_as_float(*max_bhat_bits);
    const float E = __uint_as_float(*max_eps_bits);
    const float A = bA[i];
    const float a = __fsqrt_ru(A);
    const float mb2 = __fmul_ru(Mb, Mb);
    const float chain = __fadd_ru(__fadd_ru(__fmul_ru(__fmul_ru(2.0f, a), Mb), mb2), 3.0f);
    float delta = __fmul_ru(3.0517578125e-05f, chain);           // 8 * 64 * 2^-24
    delta = __fadd_ru(delta, __fmul_ru(1.1920928955078125e-07f, A));  // 2 * 2^-24
    delta = __fadd_ru(delta, __fmul_ru(2.384185791015625e-07f, mb2)); // 4 * 2^-24
    bdelta[i] = __fadd_ru(delta, 1e-7f);
    beps2[i] = __fmul_ru(2.0f, __fadd_ru(eps[i], E));
}

}  // namespace

size_t tensor_smem_bytes() { return SMEM_BYTES; }

cudaError_t launch_tensor_operands(const float* x, int64_t n, int64_t n_pad, int d, const double* means,
                                   const uint32_t* max_norm_bits, bool cosine, bool bf16, const uint32_t* perm,
                                   void* A16, void* B16, float* bA, float* eps, uint32_t* max_eps_bits,
                                   uint32_t* max_bhat_bits, cudaStream_t s) {
    const unsigned blocks = (unsigned)((n_pad + 127) / 128);
    if (bf16)
        tensor_operands_kernel<__nv_bfloat16><<<blocks, 128, 0, s>>>(
            x, n, n_pad, d, means, max_norm_bits, cosine ? 1 : 0, perm, (__nv_bfloat16*)A16, (__nv_bfloat16*)B16,
            bA, eps, max_eps_bits, max_bhat_bits);
    else
        tensor_operands_kernel<__half><<<blocks, 128, 0, s>>>(x, n, n_pad, d, means, max_norm_bits,
                                                              cosine ? 1 : 0, perm, (__half*)A16, (__half*)B16, bA,
                                                              eps, max_eps_bits, max_bhat_bits);
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
                                     const float* beps2, const Lists& lists, bool bf16, const TileLists* tiles,
                                     bool resume, float* theta_io, int* grid_out, unsigned long long* stats,
                                     unsigned long long* argmin_out, int pass_mode, float* topk_out) {
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
    a.self_offset = plan.self_offset;
    a.col_tiles = (int)(nr_pad / TBN);
    const int col_segs = lists.segments / PARTS;
    a.tiles_per_seg = (a.col_tiles + col_segs - 1) / col_segs;
    if ((a.col_tiles + a.tiles_per_seg - 1) / a.tiles_per_seg != col_segs) return cudaErrorInvalidValue;
    if (lists.ctot < lists.cap + kPartCols || lists.ctot > 32 * kListMaxEntriesPerLane) return cudaErrorInvalidValue;
    // The rerank takes the union of a row's lists: up to kRerankUnion keys.
    a.final_cap = std::max(kListFinalMin, kRerankUnion / lists.segments);
    if (lists.segments % PARTS) return cudaErrorInvalidValue;
    a.items = (int)(nq_pad / ROWS) * (lists.segments / PARTS);
    a.idesc = umma_idesc_f16(TBM, TBN, bf16);
    a.err = ctx->d_err;
    a.stats = stats;
    a.tl = nullptr;
    a.tl_off = nullptr;
    a.tl_cnt = nullptr;
    a.tl_stride = 0;
    a.tl2 = nullptr;
    a.tl2_cnt = nullptr;
    a.tl2_stride = 0;
    a.item_order = nullptr;
    a.item_range = tiles ? tiles->range : nullptr;
    a.row_map = tiles ? tiles->row_map : nullptr;
    a.row_theta = tiles ? tiles->row_theta : nullptr;
    if (tiles && !tiles->tiles) a.item_order = tiles->order;
    if (a.item_range && lists.segments != PARTS) return cudaErrorInvalidValue;
    if (tiles && tiles->tiles) {
        // Explicit tile lists are per work item (row block and column
        // segment); several segments of a row block must share its threshold
        // through row_theta.
        if ((col_segs != 1 && !tiles->row_theta) || !tiles->count) return cudaErrorInvalidValue;
        a.tl = tiles->tiles;
        a.tl_off = tiles->offset;
        a.tl_cnt = tiles->count;
        a.tl_stride = tiles->stride;
        a.item_order = tiles->order;
        if (tiles->tiles2) {
            if (tiles->offset || !tiles->count2) return cudaErrorInvalidValue;
            a.tl2 = tiles->tiles2;
            a.tl2_cnt = tiles->count2;
            a.tl2_stride = tiles->stride2;
        }
    }
    a.resume = resume ? 1 : 0;
    a.theta_io = theta_io;
    a.thr_only = pass_mode == kPassThresholds ? 1 : 0;
    a.collect = pass_mode == kPassCollect ? 1 : 0;
    // Threshold and collect passes keep one column segment per row, or share
    // the row's threshold between its segments through row_theta.
    if ((a.thr_only || a.collect) && (!theta_io || plan.k > 32 || (lists.segments != PARTS && !a.row_theta)))
        return cudaErrorInvalidValue;
    a.argmin_out = argmin_out;
    a.topk_out = topk_out;
    a.topk_stride = nq_pad * lists.segments;
    // (The top-K is written by the top-16 and top-32 threshold passes: k >= 2.)
    if (topk_out && (!a.thr_only || lists.segments != PARTS || plan.k < 2)) return cudaErrorInvalidValue;
    if (argmin_out && (plan.k != 1 || resume)) return cudaErrorInvalidValue;
    if (a.tl2 && !a.collect) return cudaErrorInvalidValue;  // a second list is read by collect passes only
    if (resume && !theta_io) return cudaErrorInvalidValue;
    // Register top-k width of a general pass (threshold and collect passes
    // keep the width that holds k).
    int width = a.k == 1 ? 1 : a.k <= 16 ? 16 : a.k <= 32 ? 32 : 0;
    if (!a.thr_only && !a.collect && a.k > 1) {
        if (plan.topk_width < 0) width = 0;
        else if (plan.topk_width == 32 && a.k <= 32) width = 32;
        else if (plan.topk_width != 0 && plan.topk_width != 16 && plan.topk_width != 32) return cudaErrorInvalidValue;
    }
    auto kern = width == 1    ? (argmin_out ? tensor_candidates_kernel<1, 3> : tensor_candidates_kernel<1, 0>)
                : width == 16 ? (a.thr_only ? tensor_candidates_kernel<16, 1>
                                 : a.collect ? (a.self ? tensor_candidates_kernel<16, 2> : tensor_candidates_kernel<16, 4>)
                                             : tensor_candidates_kernel<16, 0>)
                : width == 32 ? (a.thr_only ? tensor_candidates_kernel<32, 1>
                                 : a.collect ? (a.self ? tensor_candidates_kernel<32, 2> : tensor_candidates_kernel<32, 4>)
                                             : tensor_candidates_kernel<32, 0>)
                              : tensor_candidates_kernel<0, 0>;
    cudaError_t e = set_smem_limit(ctx, (const void*)kern, (int)SMEM_BYTES);
    if (e != cudaSuccess) return e;
    const int grid = std::min(a.items, plan.max_ctas > 0 ? std::min(plan.max_ctas, ctx->sm_count) : ctx->sm_count);
    if (grid_out) *grid_out = grid;
    kern<<<grid, THREADS, SMEM_BYTES, ctx->stream>>>(ta, tb, a);
    return cudaGetLastError();
}

// The threshold of each row from both column parts' register top-K of a
// threshold pass (k <= K; each list ascending with its first K - k slots
// -inf): the k-th smallest of the two lists' union, which lies at or below
// each part's own k-th (a row's nearest columns fall in both halves of a
// tile, so each part alone sees only some of them), bounded as the sweep
// bounds a k-th, and never above either part's threshold.  Both of the
// row's theta slots receive it.
template <int K>
__global__ void merge_part_thresholds_kernel(const float* __restrict__ topk, int64_t stride, int64_t n, int k,
                                             const float* __restrict__ bA, const float* __restrict__ bdelta,
                                             const float* __restrict__ beps2, float* __restrict__ theta) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p0 = topk + (int64_t)(K - k) * stride + i * PARTS;
    const float* p1 = p0 + 1;
    int u = 0, v = 0;
    float kth = __int_as_float(0x7f800000);
    for (int t = 0; t < k; ++t) {
        const float x = u < k ? p0[u * stride] : __int_as_float(0x7f800000);
        const float y = v < k ? p1[v * stride] : __int_as_float(0x7f800000);
        if (x <= y) {
            kth = x;
            ++u;
        } else {
            kth = y;
            ++v;
        }
    }
    const float t0 = theta[i * PARTS], t1 = theta[i * PARTS + 1];
    const float th = fminf(fminf(t0, t1), TensorBound{bA[i], bdelta[i], beps2[i]}.theta_f32(kth));
    theta[i * PARTS] = th;
    theta[i * PARTS + 1] = th;
}

cudaError_t launch_merge_part_thresholds(const float* topk, int width, int64_t n, int64_t n_pad, int k,
                                         const float* bA, const float* bdelta, const float* beps2, float* theta,
                                         cudaStream_t s) {
    if (k < 1 || k > width || (width != 16 && width != 32)) return cudaErrorInvalidValue;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    const int64_t stride = n_pad * PARTS;  // one column segment: PARTS lists a row
    if (width == 16)
        merge_part_thresholds_kernel<16><<<blocks, 256, 0, s>>>(topk, stride, n, k, bA, bdelta, beps2, theta);
    else
        merge_part_thresholds_kernel<32><<<blocks, 256, 0, s>>>(topk, stride, n, k, bA, bdelta, beps2, theta);
    return cudaGetLastError();
}

}  // namespace scrust
