// rerank.cu -- exact finish of every row: candidates from the lists are
// pruned to the final threshold, re-measured in the FP32 difference form on
// the caller's coordinates, sorted by (distance, id), and any group of
// candidates whose FP32 gap is inside the difference form's error bound and
// that reaches the first k positions is adjudicated in FP64.
//
// This is what makes the neighbour lists equal to the FP64 exact kNN with
// lowest-index tie-break (tests/test_neighbors_audit.py:52-61) whatever form
// produced the candidates.  In reference-snap mode the value is instead the
// reference Metal kernel's (crates/scrust-gpu/src/kernels/knn.rs:223-244) and
// the order its (d^2, id) order (knn.rs:179-182), with no adjudication.
//
// One warp per row in the common case; rows whose lists overflowed, or whose
// union exceeds the warp's capacity, go to a block-per-row fallback that
// re-measures the whole row.
#include "common.cuh"
#include "internal.h"
#include "lists.cuh"

namespace scrust {

namespace {

constexpr int RR_WARPS = 4;
constexpr int RC = kRerankUnion;  // keys per warp
constexpr int FB_CAP = 4096;  // keys per fallback block
constexpr int FB_THREADS = 256;
constexpr int FB_BLOCKS = 32;

struct RerankArgs {
    const float* qx;
    const float* rx;
    const float* qn2;
    const float* rn2;
    const double* qn64;
    const double* rn64;
    const float* qraw;
    const float* rraw;
    RowBounds bounds;
    Lists lists;
    const uint32_t* perm;  // list entry (candidate id) -> input reference row, or null
    const uint32_t* qperm; // list row -> input query row, or null (a self solve: perm)
    const float* xs;       // working rows in list order (ordered solves), or null
    const float* xr_list;  // reference rows indexed by list entry (xs for a self solve)
    int ids_only;          // the lists hold ids only (collected below their thresholds): keep every entry
    int xs_stride;         // floats per row of xs and xr_list
    int xs_v8;             // rows padded with zeros to a multiple of 8 floats, 32-byte aligned
    const uint32_t* row_lo;  // per input row: first row of its solve (a batch of solves), or null
    const uint32_t* row_hi;  // per input row: end of its solve
    const float* theta;    // per list: its threshold when the candidate pass ended, or null
    int64_t nq, nr;
    int d, k, mode, metric, self;
    int64_t self_offset;  // query row q is reference row q + self_offset
    float gamma;
    uint32_t* out_idx;
    float* out_dist;
    uint32_t* fb_rows;
    uint32_t* fb_count;
    uint32_t* fb_next;
    uint32_t* big_rows;   // rows with many survivors, for the second sorted pass
    uint32_t* big_count;
    uint32_t* big_next;
    float* fb_scratch;
    int* err;
};

__device__ __forceinline__ float compute_r(const RerankArgs& a, int64_t q, uint32_t j) {
    if (a.mode == SCRUST_MODE_REFERENCE_SNAP)
        return dist2_reference_snap(a.qx + q * a.d, a.rx + (int64_t)j * a.d, a.d, a.qn2[q], a.rn2[j]);
    return dist2_f32(a.qx + q * a.d, a.rx + (int64_t)j * a.d, a.d);
}

// Two sorted FP32 values that the difference form cannot order reliably.
__device__ __forceinline__ bool tied(const RerankArgs& a, float r1, float r2) {
    if (a.mode == SCRUST_MODE_REFERENCE_SNAP) return false;
    float tol = a.gamma * (r1 + r2) + kTieAbs;
    if (a.metric == SCRUST_METRIC_COSINE)
        tol += 2.384185791015625e-07f * (sqrtf(r1) + sqrtf(r2)) + 1e-14f;
    return (r2 - r1) <= tol;
}

__device__ __forceinline__ double adjudicate(const RerankArgs& a, int64_t q, uint32_t j) {
    if (a.metric == SCRUST_METRIC_COSINE)
        return cosine_f64(a.qraw + q * a.d, a.rraw + (int64_t)j * a.d, a.d, a.qn64[q], a.rn64[j]);
    return sqrt(dist2_f64(a.qraw + q * a.d, a.rraw + (int64_t)j * a.d, a.d));
}

__device__ __forceinline__ float key_r(unsigned long long key) { return key_float((uint32_t)(key >> 32)); }
__device__ __forceinline__ uint32_t key_id(unsigned long long key) { return (uint32_t)key; }

// Rows of the reference with the same bits in every coordinate.
__device__ __forceinline__ bool rows_equal(const float* __restrict__ u, const float* __restrict__ v, int d) {
    const uint32_t* x = reinterpret_cast<const uint32_t*>(u);
    const uint32_t* y = reinterpret_cast<const uint32_t*>(v);
    for (int t0 = 0; t0 < d; t0 += 8) {
        bool eq = true;
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (t0 + t < d) eq &= __ldg(x + t0 + t) == __ldg(y + t0 + t);
        if (!eq) return false;
    }
    return true;
}

// Tie groups are runs of consecutive sorted candidates whose FP32 values the
// difference form cannot order.  A group that reaches the first k positions
// is ordered by FP64 (distance, id), and its members take FP64 distances --
// unless every member's row has the same bits as the first member's row
// (duplicated cells): the FP32 values are then equal, the order by id that
// the sort left is already the FP64 order, and the FP32 value is the
// distance.  Cosine rows always take FP64 values.
enum : uint8_t { TIE_NONE = 0, TIE_SAME = 1, TIE_DIFF = 2 };

// Writes the first k of the sorted candidates keys[0..m), resolving tie
// groups as above; dbl and flags hold m entries of scratch.
template <class Team>
__device__ void finalize_row(const Team& team, const RerankArgs& a, int64_t q,
                             const unsigned long long* keys, int m, double* dbl, uint8_t* flags) {
    const int k = a.k;
    const bool cosine = a.metric == SCRUST_METRIC_COSINE;
    for (int p = team.rank; p < m; p += team.size()) {
        int gs = p;
        while (gs > 0 && tied(a, key_r(keys[gs - 1]), key_r(keys[gs]))) gs--;
        if (gs >= k) continue;
        int ge = p;
        while (ge + 1 < m && tied(a, key_r(keys[ge]), key_r(keys[ge + 1]))) ge++;
        uint8_t f = TIE_NONE;
        if (ge > gs && !cosine)
            f = (p == gs || rows_equal(a.rraw + (int64_t)key_id(keys[gs]) * a.d,
                                       a.rraw + (int64_t)key_id(keys[p]) * a.d, a.d))
                    ? TIE_SAME
                    : TIE_DIFF;
        flags[p] = f;
    }
    team.sync();
    for (int p = team.rank; p < m; p += team.size()) {
        int gs = p;
        while (gs > 0 && tied(a, key_r(keys[gs - 1]), key_r(keys[gs]))) gs--;
        if (gs >= k) continue;
        int ge = p;
        while (ge + 1 < m && tied(a, key_r(keys[ge]), key_r(keys[ge + 1]))) ge++;
        bool fp64 = cosine;
        if (ge > gs && !cosine)
            for (int o = gs; o <= ge; ++o) fp64 |= flags[o] == TIE_DIFF;
        if (fp64) dbl[p] = adjudicate(a, q, key_id(keys[p]));
    }
    team.sync();
    for (int p = team.rank; p < m; p += team.size()) {
        int gs = p;
        while (gs > 0 && tied(a, key_r(keys[gs - 1]), key_r(keys[gs]))) gs--;
        if (gs >= k) continue;
        int ge = p;
        while (ge + 1 < m && tied(a, key_r(keys[ge]), key_r(keys[ge + 1]))) ge++;
        bool fp64 = cosine;
        if (ge > gs && !cosine)
            for (int o = gs; o <= ge; ++o) fp64 |= flags[o] == TIE_DIFF;
        const uint32_t id = key_id(keys[p]);
        int pos = p;
        if (fp64 && ge > gs) {
            const double dv = dbl[p];
            int rank = 0;
            for (int o = gs; o <= ge; ++o) {
                const double dq = dbl[o];
                const uint32_t io = key_id(keys[o]);
                rank += (dq < dv) || (dq == dv && io < id);
            }
            pos = gs + rank;
        }
        if (pos < k) {
            const float dist = fp64 ? __double2float_rn(dbl[p]) : sqrtf(key_r(keys[p]));
            a.out_idx[q * k + pos] = a.row_lo ? id - a.row_lo[q] : id;
            a.out_dist[q * k + pos] = dist;
        }
    }
    team.sync();
}

__device__ void push_fallback(const RerankArgs& a, int64_t slot) {
    uint32_t pos = atomicAdd(a.fb_count, 1u);
    a.fb_rows[pos] = (uint32_t)slot;
}

__device__ __forceinline__ int64_t input_row(const RerankArgs& a, int64_t s) {
    return a.perm ? (int64_t)a.perm[s] : s;
}
// The input query row of list row `slot`.
__device__ __forceinline__ int64_t query_row(const RerankArgs& a, int64_t slot) {
    return a.qperm ? (int64_t)a.qperm[slot] : slot;
}

__global__ void __launch_bounds__(RR_WARPS * 32) rerank_warp_kernel(RerankArgs a) {
    extern __shared__ unsigned long long rr_smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    unsigned long long* A = rr_smem + (size_t)warp * 2 * RC;
    unsigned long long* B = A + RC;
    uint8_t* flags = reinterpret_cast<uint8_t*>(rr_smem + (size_t)RR_WARPS * 2 * RC) + (size_t)warp * RC;
    const int64_t slot = (int64_t)blockIdx.x * RR_WARPS + warp;  // list row
    if (slot >= a.nq || (a.qperm && a.qperm[slot] == 0xffffffffu)) return;
    WarpTeam team;
    if (a.lists.overflow[slot]) {
        if (lane == 0) push_fallback(a, slot);
        return;
    }
    const int64_t q = query_row(a, slot);
    const int segs = a.lists.segments;
    int m0 = 0;
    for (int s = 0; s < segs; ++s) m0 += (int)min(a.lists.cnt[slot * segs + s], (uint32_t)a.lists.ctot);
    if (m0 > RC || m0 < a.k) {
        if (lane == 0) push_fallback(a, slot);
        return;
    }
    int off = 0;
    for (int s = 0; s < segs; ++s) {
        const int c = (int)min(a.lists.cnt[slot * segs + s], (uint32_t)a.lists.ctot);
        const int64_t base = (slot * segs + s) * (int64_t)a.lists.ctot;
        for (int p = lane; p < c; p += 32) {
            uint32_t id = a.lists.ids[base + p];
            float v = a.lists.vals[base + p];
            if ((int64_t)id >= a.nr) {  // never written by a candidate kernel: refuse to read it
                atomicExch(a.err + DERR_CANDIDATES, 1);
                id = 0;
                v = __int_as_float(0x7f800000);
            }
            if (a.perm) id = a.perm[id];
            A[off + p] = ((unsigned long long)float_key(v) << 32) | id;
        }
        off += c;
    }
    __syncwarp();
    const uint32_t kth = team_select_hi(team, A, m0, a.k);
    const float theta = a.bounds.margin ? PlainBound{a.bounds.margin[slot]}.theta(key_float(kth))
                                        : TensorBound{a.bounds.A[slot], a.bounds.delta[slot], a.bounds.eps2[slot]}.theta(
                                              key_float(kth));
    int m = 0;
    for (int b0 = 0; b0 < m0; b0 += 32) {
        const int p = b0 + lane;
        bool keep = false;
        uint32_t id = 0;
        if (p < m0) {
            const unsigned long long kk = A[p];
            keep = key_r(kk) < theta;
            id = key_id(kk);
        }
        const uint32_t ballot = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const float r = compute_r(a, q, id);
            B[m + __popc(ballot & lanemask_lt())] = ((unsigned long long)float_key(r) << 32) | id;
        }
        m += __popc(ballot);
    }
    __syncwarp();
    const int P = next_pow2(m);
    for (int p = m + lane; p < P; p += 32) B[p] = ~0ull;
    __syncwarp();
    team_bitonic_sort(team, B, P);
    finalize_row(team, a, q, B, m, reinterpret_cast<double*>(A), flags);
}

// Tensor-form solves: the candidate pass left every list with a threshold no
// smaller than the final one, so the rerank needs no selection.  A warp per
// list row keeps the entries below the smaller of its lists' thresholds,
// measures them on the working rows laid out in list order (for an ordered
// solve neighbouring rows share candidates, which stay in cache), and
// finishes as above with input ids.  A row with more than RS_KEYS survivors
// (many cells inside the bound of the k-th, as for queries off the data's
// manifold in high dimension) is finished by a second pass with room for
// RS_BIG_KEYS; beyond that, by the fallback.
constexpr int RS_WARPS = 8;
constexpr int RS_KEYS = 128;
constexpr int RS_BIG_WARPS = 4;
constexpr int RS_BIG_KEYS = 2048;

// 0: done; 1: more than `cap` survivors; 2: needs the fallback.
template <int CAP>
__device__ int sorted_row(const RerankArgs& a, int64_t slot, unsigned long long* keys, double* dbl, uint8_t* flags) {
    const int lane = threadIdx.x & 31;
    WarpTeam team;
    if (a.lists.overflow[slot]) return 2;
    const int segs = a.lists.segments;
    float theta = __int_as_float(0x7f800000);
    for (int l = 0; l < segs; ++l) theta = fminf(theta, a.theta[slot * segs + l]);
    const float* xq = a.xs + slot * a.xs_stride;
    int m = 0;
    for (int l = 0; l < segs; ++l) {
        const int c = (int)min(a.lists.cnt[slot * segs + l], (uint32_t)a.lists.ctot);
        const int64_t base = (slot * segs + l) * (int64_t)a.lists.ctot;
        for (int b0 = 0; b0 < c; b0 += 32) {
            const int p = b0 + lane;
            bool keep = false;
            uint32_t id = 0;
            if (p < c) {
                id = a.lists.ids[base + p];
                if ((int64_t)id >= a.nr) {  // never written by a candidate kernel: refuse to read it
                    atomicExch(a.err + DERR_CANDIDATES, 1);
                } else {
                    keep = a.ids_only || a.lists.vals[base + p] < theta;
                }
            }
            const uint32_t ballot = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int pos = m + __popc(ballot & lanemask_lt());
                if (pos < CAP) {
                    const float* xr = a.xr_list + (int64_t)id * a.xs_stride;
                    const float r = a.xs_v8 ? dist2_f32_v8(xq, xr, a.xs_stride / 8) : dist2_f32(xq, xr, a.d);
                    keys[pos] = ((unsigned long long)float_key(r) << 32) | (uint32_t)input_row(a, id);
                }
            }
            m += __popc(ballot);
        }
    }
    if (m < a.k) return 2;
    if (m > CAP) return 1;
    __syncwarp();
    const int P = next_pow2(m);
    for (int p = m + lane; p < P; p += 32) keys[p] = ~0ull;
    __syncwarp();
    team_bitonic_sort(team, keys, P);
    finalize_row(team, a, query_row(a, slot), keys, m, dbl, flags);
    return 0;
}

__device__ __forceinline__ unsigned long long min_u64(unsigned long long x, unsigned long long y) {
    return x < y ? x : y;
}
__device__ __forceinline__ unsigned long long max_u64(unsigned long long x, unsigned long long y) {
    return x < y ? y : x;
}

// Ascending bitonic sort across the warp of P = 32 or 64 keys, position
// lane + 32 r in key[r] (key[1] unused when P = 32); fully unrolled.
template <int P>
__device__ __forceinline__ void warp_sort_keys(unsigned long long (&key)[2]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int size = 2; size <= P; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride == 32) {
                const unsigned long long lo = min_u64(key[0], key[1]), hi = max_u64(key[0], key[1]);
                key[0] = lo;
                key[1] = hi;
            } else {
#pragma unroll
                for (int r = 0; r < P / 32; ++r) {
                    const int i = lane + 32 * r;
                    const unsigned long long o = __shfl_xor_sync(0xffffffffu, key[r], stride);
                    const bool take_min = ((i & stride) == 0) == ((i & size) == 0);
                    key[r] = ((key[r] < o) == take_min) ? key[r] : o;
                }
            }
        }
    }
}

// Rows whose lists hold at most 64 entries in all (nearly every row): the
// entries are read two per lane, the survivors measured, and the (distance,
// id) keys sorted in registers across the warp (bitonic over 64 positions,
// position lane + 32 r in key[r]); tie groups are then found from a ballot of
// the positions that start one.  The result is finalize_row's.  Returns 0
// when done, 2 for the fallback, 3 when the lists hold more than 64 entries.
__device__ int sorted_row_regs(const RerankArgs& a, int64_t slot, unsigned long long* keys_s, double* dbl) {
    const int lane = threadIdx.x & 31;
    const int segs = a.lists.segments;
    if (segs > 32) return 3;
    // The row's header, its own coordinates and -- with two lists, the
    // common case -- the first 32 slots of both lists are read at once (the
    // lists hold at least 64 slots each); only then is anything tested.
    // Slots 32..63 of a list are read only when it holds more than 32.
    const uint32_t ovf = a.lists.overflow[slot];
    const int cl = lane < segs ? (int)min(a.lists.cnt[slot * segs + lane], (uint32_t)a.lists.ctot) : 0;
    const float tl = lane < segs ? a.theta[slot * segs + lane] : __int_as_float(0x7f800000);
    const int64_t base0 = slot * segs * (int64_t)a.lists.ctot;
    uint32_t sid[2][2] = {{0u, 0u}, {0u, 0u}};
    float sval[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    if (segs == 2) {
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            sid[l][0] = a.lists.ids[base0 + l * (int64_t)a.lists.ctot + lane];
            sval[l][0] = a.ids_only ? __int_as_float(0xff800000) : a.lists.vals[base0 + l * (int64_t)a.lists.ctot + lane];
        }
    }
    if (ovf) return 2;
    float theta = tl;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) theta = fminf(theta, __shfl_xor_sync(0xffffffffu, theta, o));
    int m0 = 0;
    uint32_t eid[2] = {0u, 0u};
    float eval[2] = {0.f, 0.f};
    bool have[2] = {false, false};
    if (segs == 2) {
        const int c0 = __shfl_sync(0xffffffffu, cl, 0), c1 = __shfl_sync(0xffffffffu, cl, 1);
        m0 = c0 + c1;
        if (m0 > 64) return 3;
#pragma unroll
        for (int l = 0; l < 2; ++l)
            if ((l == 0 ? c0 : c1) > 32) {
                sid[l][1] = a.lists.ids[base0 + l * (int64_t)a.lists.ctot + lane + 32];
                sval[l][1] = a.ids_only ? __int_as_float(0xff800000)
                                        : a.lists.vals[base0 + l * (int64_t)a.lists.ctot + lane + 32];
            }
        // Position e = lane + 32 r: list 0 slot e below c0, else list 1 slot e - c0.
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int e = lane + 32 * r;
            const int p1 = max(e - c0, 0);
            const uint32_t i10 = __shfl_sync(0xffffffffu, sid[1][0], p1 & 31);
            const uint32_t i11 = __shfl_sync(0xffffffffu, sid[1][1], p1 & 31);
            const float v10 = __shfl_sync(0xffffffffu, sval[1][0], p1 & 31);
            const float v11 = __shfl_sync(0xffffffffu, sval[1][1], p1 & 31);
            have[r] = e < m0;
            eid[r] = e < c0 ? sid[0][r] : (p1 < 32 ? i10 : i11);
            eval[r] = e < c0 ? sval[0][r] : (p1 < 32 ? v10 : v11);
        }
    } else {
        // Entry e of the row's lists (in list order) -> list and position.
        int list[2] = {-1, -1}, pos[2] = {0, 0};
        for (int l = 0; l < segs; ++l) {
            const int c = __shfl_sync(0xffffffffu, cl, l);
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int e = lane + 32 * r;
                if (list[r] < 0 && e < m0 + c) {
                    list[r] = l;
                    pos[r] = e - m0;
                }
            }
            m0 += c;
        }
        if (m0 > 64) return 3;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            if (list[r] >= 0) {
                const int64_t at = base0 + list[r] * (int64_t)a.lists.ctot + pos[r];
                have[r] = true;
                eid[r] = a.lists.ids[at];
                eval[r] = a.ids_only ? __int_as_float(0xff800000) : a.lists.vals[at];
            }
        }
    }
    const float* xq = a.xs + slot * a.xs_stride;
    unsigned long long key[2] = {~0ull, ~0ull};
    int m = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        bool keep = false;
        const uint32_t id = eid[r];
        if (have[r]) {
            if ((int64_t)id >= a.nr) {  // never written by a candidate kernel: refuse to read it
                atomicExch(a.err + DERR_CANDIDATES, 1);
            } else {
                keep = eval[r] < theta;
            }
        }
        if (keep) {
            const float* xr = a.xr_list + (int64_t)id * a.xs_stride;
            const float d2 = a.xs_v8 ? dist2_f32_v8(xq, xr, a.xs_stride / 8) : dist2_f32(xq, xr, a.d);
            key[r] = ((unsigned long long)float_key(d2) << 32) | (uint32_t)input_row(a, id);
        }
        m += __popc(__ballot_sync(0xffffffffu, keep));
    }
    if (m < a.k) return 2;
    // Bitonic sort of the 64 positions (32 when the second half is empty).
    if (m0 > 32)
        warp_sort_keys<64>(key);
    else
        warp_sort_keys<32>(key);
    // Positions that start a tie group (runs of consecutive tied values).
    const unsigned long long up0 = __shfl_up_sync(0xffffffffu, key[0], 1);
    const unsigned long long up1 = __shfl_up_sync(0xffffffffu, key[1], 1);
    const unsigned long long last0 = __shfl_sync(0xffffffffu, key[0], 31);
    bool start[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int p = lane + 32 * r;
        const unsigned long long prev = r == 0 ? up0 : (lane == 0 ? last0 : up1);
        start[r] = p == 0 || p >= m || !tied(a, key_r(prev), key_r(key[r]));
    }
    const unsigned long long S =
        (unsigned long long)__ballot_sync(0xffffffffu, start[0]) |
        ((unsigned long long)__ballot_sync(0xffffffffu, start[1]) << 32);
    const int k = a.k;
    const bool cosine = a.metric == SCRUST_METRIC_COSINE;
    const int64_t q = query_row(a, slot);
    // The common case: positions 0..k all start a group, so the first k are
    // singletons and the sort's order and FP32 values are final.
    if (!cosine && k < 63 && (S & ((2ull << k) - 1)) == ((2ull << k) - 1)) {
        if (lane < k) {
            const uint32_t id = key_id(key[0]);
            a.out_idx[q * k + lane] = a.row_lo ? id - a.row_lo[q] : id;
            a.out_dist[q * k + lane] = sqrtf(key_r(key[0]));
        }
        if (lane + 32 < k) {
            const uint32_t id = key_id(key[1]);
            a.out_idx[q * k + lane + 32] = a.row_lo ? id - a.row_lo[q] : id;
            a.out_dist[q * k + lane + 32] = sqrtf(key_r(key[1]));
        }
        return 0;
    }
    int gs[2], ge[2];
    bool grouped[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int p = lane + 32 * r;
        const unsigned long long upto = p == 63 ? ~0ull : (2ull << p) - 1;  // positions 0..p
        gs[r] = 63 - __clzll(S & upto);
        const unsigned long long after = S & ~upto;
        ge[r] = min(after ? __ffsll(after) - 2 : 63, m - 1);
        grouped[r] = p < m && gs[r] < k && ge[r] > gs[r];
    }
    // Members whose row differs from their group's first member's row.
    unsigned long long D = 0;
    if (!cosine && __any_sync(0xffffffffu, grouped[0] || grouped[1])) {
        bool differs[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int p = lane + 32 * r;
            const uint32_t f0 = __shfl_sync(0xffffffffu, key_id(key[0]), gs[r] & 31);
            const uint32_t f1 = __shfl_sync(0xffffffffu, key_id(key[1]), gs[r] & 31);
            const uint32_t first = gs[r] < 32 ? f0 : f1;
            differs[r] = grouped[r] && p != gs[r] &&
                         !rows_equal(a.rraw + (int64_t)first * a.d, a.rraw + (int64_t)key_id(key[r]) * a.d, a.d);
        }
        D = (unsigned long long)__ballot_sync(0xffffffffu, differs[0]) |
            ((unsigned long long)__ballot_sync(0xffffffffu, differs[1]) << 32);
    }
    bool need[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int p = lane + 32 * r;
        const unsigned long long span =
            (ge[r] == 63 ? ~0ull : (2ull << ge[r]) - 1) & ~((1ull << gs[r]) - 1);  // positions gs..ge
        need[r] = p < m && gs[r] < k && (cosine || (grouped[r] && (D & span) != 0));
    }
    const bool any_group = __any_sync(0xffffffffu, need[0] || need[1]);
    if (any_group) {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int p = lane + 32 * r;
            if (p < m) keys_s[p] = key[r];
            if (need[r]) dbl[p] = adjudicate(a, q, key_id(key[r]));
        }
        __syncwarp();
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int p = lane + 32 * r;
        if (p >= m || gs[r] >= k) continue;
        const uint32_t id = key_id(key[r]);
        int at = p;
        if (need[r] && ge[r] > gs[r]) {
            const double dv = dbl[p];
            int rank = 0;
            for (int o = gs[r]; o <= ge[r]; ++o) {
                const double dq = dbl[o];
                const uint32_t io = key_id(keys_s[o]);
                rank += (dq < dv) || (dq == dv && io < id);
            }
            at = gs[r] + rank;
        }
        if (at < k) {
            const float dist = need[r] ? __double2float_rn(dbl[p]) : sqrtf(key_r(key[r]));
            a.out_idx[q * k + at] = a.row_lo ? id - a.row_lo[q] : id;
            a.out_dist[q * k + at] = dist;
        }
    }
    __syncwarp();
    return 0;
}

// Each block walks its own contiguous range of list rows, its warps on
// consecutive rows: the rows an SM holds at once come from a few ranges, and
// neighbouring rows' candidate rows (mostly the same cells) stay in its L1.
__global__ void __launch_bounds__(RS_WARPS * 32, 6) rerank_sorted_kernel(RerankArgs a, int64_t span) {
    extern __shared__ unsigned long long rs_smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    unsigned long long* keys = rs_smem + (size_t)warp * 2 * RS_KEYS;
    double* dbl = reinterpret_cast<double*>(keys + RS_KEYS);
    uint8_t* flags = reinterpret_cast<uint8_t*>(rs_smem + (size_t)RS_WARPS * 2 * RS_KEYS) + (size_t)warp * RS_KEYS;
    const int64_t lo = (int64_t)blockIdx.x * span, hi = min(a.nq, lo + span);
    for (int64_t slot = lo + warp; slot < hi; slot += RS_WARPS) {
        if (a.qperm && a.qperm[slot] == 0xffffffffu) continue;  // padding of a batch layout
        int r = sorted_row_regs(a, slot, keys, dbl);
        if (r == 3) r = sorted_row<RS_KEYS>(a, slot, keys, dbl, flags);
        if (r && lane == 0) {
            if (r == 1) {
                a.big_rows[atomicAdd(a.big_count, 1u)] = (uint32_t)slot;
            } else {
                push_fallback(a, slot);
            }
        }
        __syncwarp();
    }
}

// The rows with more survivors than the first pass holds: warps take them
// from a queue.
__global__ void __launch_bounds__(RS_BIG_WARPS * 32) rerank_sorted_big_kernel(RerankArgs a) {
    extern __shared__ unsigned long long rb_smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    unsigned long long* keys = rb_smem + (size_t)warp * 2 * RS_BIG_KEYS;
    double* dbl = reinterpret_cast<double*>(keys + RS_BIG_KEYS);
    uint8_t* flags =
        reinterpret_cast<uint8_t*>(rb_smem + (size_t)RS_BIG_WARPS * 2 * RS_BIG_KEYS) + (size_t)warp * RS_BIG_KEYS;
    for (;;) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(a.big_next, 1u);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= *a.big_count) break;
        const int64_t slot = a.big_rows[i];
        const int r = sorted_row<RS_BIG_KEYS>(a, slot, keys, dbl, flags);
        if (r && lane == 0) push_fallback(a, slot);
        __syncwarp();
    }
}

// One block per row, over every reference row: used for rows whose
// candidate lists overflowed (many cells within the margin, e.g. duplicates).
__global__ void __launch_bounds__(FB_THREADS) rerank_fallback_kernel(RerankArgs a) {
    extern __shared__ unsigned long long fb_smem[];
    unsigned long long* keys = fb_smem;
    double* dbl = reinterpret_cast<double*>(fb_smem + FB_CAP);
    uint8_t* flags = reinterpret_cast<uint8_t*>(fb_smem + 2 * FB_CAP);
    __shared__ int scratch;
    __shared__ uint32_t row_s;
    __shared__ uint32_t hist[256];
    __shared__ uint32_t sel_prefix;
    __shared__ int sel_rank;
    __shared__ int cnt_s;
    BlockTeam team(&scratch);
    const int tid = threadIdx.x;
    float* sc = a.fb_scratch + (int64_t)blockIdx.x * a.nr;
    for (;;) {
        if (tid == 0) {
            const uint32_t i = atomicAdd(a.fb_next, 1u);
            row_s = i < *a.fb_count ? a.fb_rows[i] : 0xffffffffu;
        }
        __syncthreads();
        const uint32_t row = row_s;
        __syncthreads();
        if (row == 0xffffffffu) break;
        const int64_t q = query_row(a, row);
        // The columns of the row's own solve: [lo, hi) of the input rows.
        const int64_t lo = a.row_lo ? (int64_t)a.row_lo[q] : 0, hi = a.row_lo ? (int64_t)a.row_hi[q] : a.nr;
        for (int64_t j = tid; j < a.nr; j += blockDim.x)
            sc[j] = (a.self && j == q + a.self_offset) || j < lo || j >= hi ? __int_as_float(0x7f800000) : compute_r(a, q, (uint32_t)j);
        __syncthreads();
        // k-th smallest of the row: four 8-bit radix passes.
        if (tid == 0) {
            sel_prefix = 0;
            sel_rank = a.k;
        }
        uint32_t mask = 0;
        for (int pass = 0; pass < 4; ++pass) {
            const int shift = 24 - 8 * pass;
            hist[tid] = 0;
            __syncthreads();
            const uint32_t prefix = sel_prefix;
            for (int64_t j = tid; j < a.nr; j += blockDim.x) {
                const uint32_t key = float_key(sc[j]);
                if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
            }
            __syncthreads();
            if (tid == 0) {
                int rank = sel_rank;
                uint32_t b = 0;
                for (; b < 256; ++b) {
                    if ((int)hist[b] >= rank) break;
                    rank -= (int)hist[b];
                }
                sel_rank = rank;
                sel_prefix = prefix | (b << shift);
            }
            mask |= 255u << shift;
            __syncthreads();
        }
        const float vk = key_float(sel_prefix);
        float T = vk;
        if (a.mode != SCRUST_MODE_REFERENCE_SNAP) T = vk + 4.0f * (a.gamma * 2.0f * vk + kTieAbs) +
                                                      (a.metric == SCRUST_METRIC_COSINE ? 1e-6f : 0.0f);
        int m = 0;
        for (int attempt = 0; attempt < 8; ++attempt) {
            if (tid == 0) cnt_s = 0;
            __syncthreads();
            for (int64_t j = tid; j < a.nr; j += blockDim.x) {
                const float r = sc[j];
                if (r <= T) {
                    const int pos = atomicAdd(&cnt_s, 1);
                    if (pos < FB_CAP) keys[pos] = ((unsigned long long)float_key(r) << 32) | (uint32_t)j;
                }
            }
            __syncthreads();
            m = cnt_s;
            if (m > FB_CAP) break;
            const int P = next_pow2(m);
            for (int p = m + tid; p < P; p += blockDim.x) keys[p] = ~0ull;
            __syncthreads();
            team_bitonic_sort(team, keys, P);
            if (a.mode == SCRUST_MODE_REFERENCE_SNAP) break;
            // If the tie group holding the last collected candidate reaches
            // position k-1, make sure nothing just outside T could join it.
            const float rl = key_r(keys[m - 1]);
            int gs = m - 1;
            while (gs > 0 && tied(a, key_r(keys[gs - 1]), key_r(keys[gs]))) gs--;
            if (gs >= a.k) break;
            const float T2 = rl + 2.0f * (a.gamma * 2.0f * rl + kTieAbs) +
                             (a.metric == SCRUST_METRIC_COSINE ? 1e-6f : 0.0f);
            int outside = 0;
            for (int64_t j = tid; j < a.nr; j += blockDim.x) outside += (sc[j] > T && sc[j] <= T2);
            if (team.sum(outside) == 0) break;
            T = T2;
        }
        if (m > FB_CAP || m < a.k) {
            if (tid == 0) atomicExch(a.err + (m > FB_CAP ? DERR_TIE_OVERFLOW : DERR_CANDIDATES), 1);
            __syncthreads();
            continue;
        }
        finalize_row(team, a, q, keys, m, dbl, flags);
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_rerank(scrust_context* ctx, const KnnPlan& plan, const float* qx,
                          const float* rx, const float* qnorm2, const float* rnorm2,
                          const double* qn64, const double* rn64, const float* qraw,
                          const float* rraw, const RowBounds& bounds, const Lists& lists,
                          const uint32_t* perm, const float* xs, const float* theta, uint32_t* out_idx,
                          float* out_dist, const uint32_t* row_lo, const uint32_t* row_hi, const float* xr_list,
                          int xs_stride, bool ids_only, const uint32_t* qperm) {
    cudaError_t e;
    uint32_t* fb_rows = (uint32_t*)ws_get(ctx, SLOT_FALLBACK_ROWS, sizeof(uint32_t) * (size_t)plan.nq, &e);
    if (!fb_rows) return e;
    float* fb_scratch =
        (float*)ws_get(ctx, SLOT_FALLBACK_SCRATCH, sizeof(float) * (size_t)plan.nr * FB_BLOCKS, &e);
    if (!fb_scratch) return e;
    RerankArgs a;
    a.qx = qx;
    a.rx = rx;
    a.qn2 = qnorm2;
    a.rn2 = rnorm2;
    a.qn64 = qn64;
    a.rn64 = rn64;
    a.qraw = qraw;
    a.rraw = rraw;
    a.bounds = bounds;
    a.lists = lists;
    a.perm = perm;
    a.qperm = qperm ? qperm : perm;
    a.xs = xs;
    a.xr_list = xr_list ? xr_list : xs;
    a.xs_stride = xs_stride > 0 ? xs_stride : plan.d;
    a.ids_only = ids_only ? 1 : 0;
    // 32-byte loads need rows padded to 8 floats on both sides: the lists'
    // query rows and the reference rows the candidate ids index.
    a.xs_v8 = xs && a.xs_stride % 8 == 0 && ((uintptr_t)xs & 31) == 0 && ((uintptr_t)a.xr_list & 31) == 0 &&
              (!xr_list || a.xs_stride == padded_row_floats(plan.d));
    a.theta = theta;
    a.row_lo = row_lo;
    a.row_hi = row_hi;
    a.nq = plan.nq;
    a.nr = plan.nr;
    a.d = plan.d;
    a.k = plan.k;
    a.mode = plan.mode;
    a.metric = plan.metric;
    a.self = plan.self ? 1 : 0;
    a.self_offset = plan.self_offset;
    a.gamma = dist2_f32_gamma(plan.d);
    a.out_idx = out_idx;
    a.out_dist = out_dist;
    a.fb_rows = fb_rows;
    a.fb_count = ctx->d_counter;
    a.fb_next = ctx->d_counter + 1;
    a.big_count = ctx->d_counter + 2;
    a.big_next = ctx->d_counter + 3;
    a.big_rows = nullptr;
    if (xs && theta) {
        a.big_rows = (uint32_t*)ws_get(ctx, SLOT_RERANK_BIG, sizeof(uint32_t) * (size_t)plan.nq, &e);
        if (!a.big_rows) return e;
    }
    a.fb_scratch = fb_scratch;
    a.err = ctx->d_err;
    e = cudaMemsetAsync(ctx->d_counter, 0, 4 * sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) return e;
    if (xs && theta) {
        const size_t smem_s = (size_t)RS_WARPS * (2 * RS_KEYS * sizeof(unsigned long long) + RS_KEYS);
        // As many blocks as stay resident (6 an SM), each over a contiguous
        // range of rows.
        const int64_t groups = (plan.nq + RS_WARPS - 1) / RS_WARPS;
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(groups, 6 * (int64_t)ctx->sm_count));
        const int64_t span = (groups + blocks - 1) / blocks * RS_WARPS;
        // Most rows need no shared memory (the register path): leave the rest
        // of the SM's unified memory to L1, which caches the candidate rows
        // that neighbouring rows share.
        static_assert(RS_WARPS * (2 * RS_KEYS * 8 + RS_KEYS) <= 24 * 1024, "rerank block smem");
        if ((e = set_smem_carveout(ctx, (const void*)rerank_sorted_kernel, 50)) != cudaSuccess) return e;
        rerank_sorted_kernel<<<(unsigned)((plan.nq + span - 1) / span), RS_WARPS * 32, smem_s, ctx->stream>>>(a, span);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        const size_t smem_b = (size_t)RS_BIG_WARPS * (2 * RS_BIG_KEYS * sizeof(unsigned long long) + RS_BIG_KEYS);
        if ((e = set_smem_limit(ctx, (const void*)rerank_sorted_big_kernel, (int)smem_b)) != cudaSuccess) return e;
        rerank_sorted_big_kernel<<<2 * ctx->sm_count, RS_BIG_WARPS * 32, smem_b, ctx->stream>>>(a);
        ctx->launches += 2;
    } else {
        const size_t smem_w = (size_t)RR_WARPS * (2 * RC * sizeof(unsigned long long) + RC);
        e = set_smem_limit(ctx, (const void*)rerank_warp_kernel, (int)smem_w);
        if (e != cudaSuccess) return e;
        const unsigned blocks = (unsigned)((plan.nq + RR_WARPS - 1) / RR_WARPS);
        rerank_warp_kernel<<<blocks, RR_WARPS * 32, smem_w, ctx->stream>>>(a);
        ctx->launches += 1;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const size_t smem_f = (size_t)FB_CAP * (sizeof(unsigned long long) + sizeof(double) + 1);
    e = set_smem_limit(ctx, (const void*)rerank_fallback_kernel, (int)smem_f);
    if (e != cudaSuccess) return e;
    rerank_fallback_kernel<<<FB_BLOCKS, FB_THREADS, smem_f, ctx->stream>>>(a);
    ctx->launches += 1;
    return cudaGetLastError();
}

}  // namespace scrust
