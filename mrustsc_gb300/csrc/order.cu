// order.cu -- a spatial ordering of the rows for the tensor sweep.
//
// Exactness never depends on the order in which a row meets its columns, but
// speed does: a row's threshold only tightens once it has seen columns near
// it, and until then every column it meets is appended to its list.  So
// before the sweep the rows are grouped into cells around anchors (every
// n/m-th row), the cells are laid out consecutively, and every 256-row work
// item gets a short list of priority tiles: the tiles holding its own cells
// and the cells of the anchors nearest to them.  The sweep visits those
// first (knn_tensor.cu).  Nearest anchors come from the tensor candidate lists
// of a points x anchors pass with k = 1 (an approximate assignment is enough
// for an ordering); anchor neighbourhoods from an FP32 anchors x anchors kNN.
//
// The sweep then runs in two passes.  The first visits only the priority
// tiles and leaves every list with a threshold.  Between the passes each
// column tile gets a bounding ball of its quantised rows (centre c_T, radius
// R_T) and each row block the largest distance U_I that can still matter:
// the MMA value of a pair is at least |a_i - b_j|^2 - A_i - delta_i, so a
// column j can join row i's list only while |a_i - b_j| < sqrt(theta_i + A_i
// + delta_i).  A tile with |c_I - c_T| - R_I - R_T >= U_I cannot add to any
// row of block I and is left out of the second pass, which visits the rest.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

// Anchor c is input row floor(c * n / m); its coordinates are copied out
// for the anchor neighbourhoods.
__global__ void anchors_kernel(const float* __restrict__ x, int d, int64_t n, int64_t m, uint32_t* __restrict__ src,
                               float* __restrict__ out) {
    const int64_t c = blockIdx.x;
    if (c >= m) return;
    const int64_t r = (c * n) / m;
    if (threadIdx.x == 0) src[c] = (uint32_t)r;
    for (int t = threadIdx.x; t < d; t += blockDim.x) out[c * d + t] = x[r * d + t];
}

// Squared FP32 distances between all anchors (a sequential fma chain over
// the dimensions per pair), 64 x 64 per block and 4 x 4 per thread; the
// diagonal is +inf.
__global__ void __launch_bounds__(256) anchor_dist_kernel(const float* __restrict__ anc, int m, int d,
                                                          float* __restrict__ dist) {
    __shared__ __align__(16) float As[64][64 + 4];  // padded as in segment_pairs_kernel
    __shared__ __align__(16) float Bs[64][64 + 4];
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
    float acc[4][4] = {};
    for (int t0 = 0; t0 < d; t0 += 64) {  // 64 dimensions at a time
        const int dc = min(64, d - t0);
        __syncthreads();
        for (int p = threadIdx.x; p < 64 * 64; p += blockDim.x) {
            const int r = p / 64, t = p % 64;
            As[t][r] = (i0 + r < m && t < dc) ? anc[(int64_t)(i0 + r) * d + t0 + t] : 0.f;
            Bs[t][r] = (j0 + r < m && t < dc) ? anc[(int64_t)(j0 + r) * d + t0 + t] : 0.f;
        }
        __syncthreads();
        for (int t = 0; t < dc; ++t) {
            const float4 a4 = *reinterpret_cast<const float4*>(&As[t][ty * 4]);
            const float4 b4 = *reinterpret_cast<const float4*>(&Bs[t][tx * 4]);
            const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float df = av[p] - bv[q];
                    acc[p][q] = fmaf(df, df, acc[p][q]);
                }
        }
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const int i = i0 + ty * 4 + p;
        if (i >= m) continue;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = j0 + tx * 4 + q;
            if (j < m) dist[(int64_t)i * m + j] = i == j ? __int_as_float(0x7f800000) : acc[p][q];
        }
    }
}

// One warp per anchor: its kAnchorNeighbours nearest other anchors, nearest
// first, ties to the smaller id; 0xffffffff past the last.  Each lane keeps a
// sorted top-k of its columns, then the lanes' heads are merged.
__global__ void __launch_bounds__(128) anchor_top_kernel(const float* __restrict__ dist, int m,
                                                         uint32_t* __restrict__ nb) {
    const int lane = threadIdx.x & 31;
    const int64_t c = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    if (c >= m) return;
    constexpr int K = kAnchorNeighbours;
    unsigned long long top[K];
#pragma unroll
    for (int r = 0; r < K; ++r) top[r] = ~0ull;
    for (int j = lane; j < m; j += 32) {
        unsigned long long key = ((unsigned long long)float_key(dist[c * m + j]) << 32) | (uint32_t)j;
        if (key < top[K - 1]) {
#pragma unroll
            for (int r = 0; r < K; ++r) {
                const unsigned long long lo = key < top[r] ? key : top[r];
                key = key < top[r] ? top[r] : key;
                top[r] = lo;
            }
        }
    }
    for (int r = 0; r < K; ++r) {
        unsigned long long best = top[0];
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
            best = other < best ? other : best;
        }
        if (top[0] == best) {  // the owning lane pops its head (keys are distinct)
#pragma unroll
            for (int q = 0; q < K - 1; ++q) top[q] = top[q + 1];
            top[K - 1] = ~0ull;
        }
        if (lane == 0) {
            const bool found = (uint32_t)(best >> 32) < float_key(__int_as_float(0x7f800000));
            nb[c * K + r] = found ? (uint32_t)best : 0xffffffffu;
        }
    }
}

// Cells are laid out in the order of a walk over the anchors: from each
// anchor to its nearest unvisited neighbouring anchor, or, when all of them
// have been visited, to the lowest unvisited anchor.  Consecutive cells are
// then mostly neighbours, so a 256-row block rarely mixes far-apart cells.
// The block stages the first kChainNb neighbours of every anchor (16-bit
// ids) in shared memory, many loads in flight; then one thread walks, since
// every step depends on the one before.  A step is kept short: the
// neighbour ids and their visited bytes are independent shared loads issued
// together, the first unvisited one is found from a mask of the twelve tests
// (no chain of selects), and marking an anchor visited is a single byte
// store.  rank[a] is anchor a's place.
constexpr int kChainNb = 12;
constexpr int kChainThreads = 1024;
__global__ void __launch_bounds__(kChainThreads) anchor_chain_kernel(const uint32_t* __restrict__ nb, int m,
                                                                     uint32_t* __restrict__ rank) {
    extern __shared__ uint32_t ch_smem[];
    const int words = (m + 3) / 4 + 1;                      // visited bytes, then one full word past them
    uint8_t* vis = reinterpret_cast<uint8_t*>(ch_smem);     // m bytes (+ padding), 1 = visited
    uint16_t* nbs = reinterpret_cast<uint16_t*>(ch_smem + (words + 1) / 2 * 2);  // m * kChainNb, 8-byte aligned
    for (int i = threadIdx.x; i < words; i += blockDim.x) ch_smem[i] = 0u;
    __syncthreads();
    // Bytes past m read as visited, so neither the tests nor the scan for
    // the lowest unvisited anchor ever pick one.
    for (int i = m + threadIdx.x; i < 4 * words; i += blockDim.x) vis[i] = 1;
    for (int a = threadIdx.x; a < m; a += blockDim.x) {
        const uint4* src = reinterpret_cast<const uint4*>(nb + (int64_t)a * kAnchorNeighbours);
        uint32_t c[kChainNb];
#pragma unroll
        for (int q = 0; q < kChainNb / 4; ++q) {
            const uint4 w = src[q];
            c[4 * q] = w.x;
            c[4 * q + 1] = w.y;
            c[4 * q + 2] = w.z;
            c[4 * q + 3] = w.w;
        }
        // Missing neighbours point past m (a visited byte).
#pragma unroll
        for (int j = 0; j < kChainNb; ++j)
            nbs[(int64_t)a * kChainNb + j] = c[j] < (uint32_t)m ? (uint16_t)c[j] : (uint16_t)m;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    vis[0] = 1;
    rank[0] = 0;
    const uint32_t* vis4 = ch_smem;
    int cur = 0, scan = 0, pos = 1;
    for (; pos < m; ++pos) {
        // The 12 neighbour ids of cur as six 32-bit words (two ids each).
        const uint2* row = reinterpret_cast<const uint2*>(nbs + (size_t)cur * kChainNb);
        const uint2 r0 = row[0], r1 = row[1], r2 = row[2];
        const uint32_t w[6] = {r0.x, r0.y, r1.x, r1.y, r2.x, r2.y};
        uint32_t free = 0;
#pragma unroll
        for (int j = 0; j < kChainNb; ++j) {
            const uint32_t c = (w[j >> 1] >> (16 * (j & 1))) & 0xffffu;
            free |= vis[c] ? 0u : (1u << j);
        }
        int next;
        if (free) {
            const int j = __ffs(free) - 1;
            const uint32_t wj = (j >> 2) == 0 ? ((j & 2) ? w[1] : w[0]) : (j >> 2) == 1 ? ((j & 2) ? w[3] : w[2])
                                                                                       : ((j & 2) ? w[5] : w[4]);
            next = (int)((wj >> (16 * (j & 1))) & 0xffffu);
        } else {
            // The lowest unvisited anchor (words below `scan` are all visited).
            while (scan < words && vis4[scan] == 0x01010101u) ++scan;
            if (scan >= words) break;  // cannot happen: an unvisited anchor exists while pos < m
            const uint32_t v = vis4[scan];
            int b = 0;
            while (b < 3 && ((v >> (8 * b)) & 0xffu)) ++b;
            next = 4 * scan + b;
            if (next >= m) break;      // cannot happen: bytes past m are marked visited
        }
        vis[next] = 1;
        rank[next] = (uint32_t)pos;
        cur = next;
    }
    // Every anchor gets a rank whatever happened above.
    for (int a = 0; a < m && pos < m; ++a)
        if (!vis[a]) {
            vis[a] = 1;
            rank[a] = (uint32_t)pos++;
        }
}

// Anchor neighbourhoods renamed into walk order: row rank[a] of out holds
// the ranks of a's neighbours.
__global__ void relabel_neighbours_kernel(const uint32_t* __restrict__ nb, const uint32_t* __restrict__ rank, int m,
                                          uint32_t* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)m * kAnchorNeighbours) return;
    const int64_t a = i / kAnchorNeighbours, j = i % kAnchorNeighbours;
    const uint32_t c = nb[i];
    out[(int64_t)rank[a] * kAnchorNeighbours + j] = c < (uint32_t)m ? rank[c] : 0xffffffffu;
}

// Each row's nearest anchor from the nearest-group pass: the better of its
// two parts' groups, then the group's eight anchors measured on the same
// 16-bit operands (a row's [a, 1, 1, 1] times an anchor's [-2b, three norm
// parts], summed in f32 over the `words` 16-byte words that hold them) and
// the smallest taken (ties to the lower anchor): an approximately nearest
// anchor, which is all an ordering needs.  Eight lanes per row, lane l
// holding word l of the row and of each of the eight anchors, so that every
// load of an anchor row is one contiguous line for the eight lanes; the
// partial sums meet by shuffles.  keys[i] receives the anchor
// (anchor_rank_kernel turns it into the sort key once the walk is done),
// vals[i] the row.
template <class T>
__device__ __forceinline__ float dot_word(uint4 x, uint4 y) {
    const uint32_t xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
    float acc = 0.f;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        float2 p, q;
        if constexpr (std::is_same<T, __nv_bfloat16>::value) {
            p = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&xs[h]));
            q = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&ys[h]));
        } else {
            p = __half22float2(*reinterpret_cast<const __half2*>(&xs[h]));
            q = __half22float2(*reinterpret_cast<const __half2*>(&ys[h]));
        }
        acc = fmaf(p.x, q.x, acc);
        acc = fmaf(p.y, q.y, acc);
    }
    return acc;
}

template <class T>
__global__ void nearest_anchor_kernel(const unsigned long long* __restrict__ best, int64_t n, int64_t m,
                                      const T* __restrict__ A, const T* __restrict__ B, int words,
                                      uint32_t* __restrict__ keys, unsigned long long* __restrict__ vals) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t i = t >> 3;
    const int l = (int)(t & 7);
    const bool row_ok = i < n;
    const uint32_t g = row_ok ? (uint32_t)min(best[2 * i], best[2 * i + 1]) : 0u;
    const int64_t c0 = (int64_t)g * 8;
    float part[8];
    const bool lane_ok = row_ok && l < words;
    const uint4 x = lane_ok ? __ldg(reinterpret_cast<const uint4*>(A + i * 64) + l) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        part[a] = 0.f;
        if (lane_ok && c0 + a < m) part[a] = dot_word<T>(x, __ldg(reinterpret_cast<const uint4*>(B + (c0 + a) * 64) + l));
    }
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) part[a] += __shfl_xor_sync(0xffffffffu, part[a], o);
    if (row_ok && l == 0) {
        int arg = 0;
        float bv = c0 < m ? part[0] : __int_as_float(0x7f800000);
#pragma unroll
        for (int a = 1; a < 8; ++a)
            if (c0 + a < m && part[a] < bv) {
                bv = part[a];
                arg = a;
            }
        const int64_t col = c0 + arg;
        keys[i] = (uint32_t)(col < m ? col : m - 1);
        vals[i] = (unsigned long long)i;
    }
}

// keys[i] = rank[keys[i]]: each row's anchor becomes the anchor's walk rank.
__global__ void anchor_rank_kernel(uint32_t* __restrict__ keys, int64_t n, const uint32_t* __restrict__ rank) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = rank[keys[i]];
}

__global__ void unpack_perm_kernel(const uint32_t* __restrict__ skeys, const unsigned long long* __restrict__ svals,
                                   int64_t n, uint32_t* __restrict__ perm, uint32_t* __restrict__ cell_of_pos,
                                   uint32_t* __restrict__ cell_count) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    perm[s] = (uint32_t)svals[s];
    cell_of_pos[s] = skeys[s];
    atomicAdd(cell_count + skeys[s], 1u);
}

// One warp per 256-row work item: the column tiles holding the item's own
// cells, then those holding the cells of their nearest anchors, nearest
// anchors first; distinct, at most kPrioMax.  In a self solve the item's own
// tile always comes first, so no list is empty.
constexpr int kHomeMax = 8;
__global__ void prio_tiles_kernel(const uint32_t* __restrict__ cell_of_pos, int64_t n,
                                  const uint32_t* __restrict__ cell_start, int m,
                                  const uint32_t* __restrict__ anchor_nb, int ka, int items, int col_tiles,
                                  uint32_t* __restrict__ prio, uint32_t* __restrict__ prio_cnt, int self_tile = 1) {
    __shared__ uint32_t outs[4][kPrioMax];
    __shared__ uint32_t homes[4][kHomeMax];
    __shared__ int nhome[4];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int item = blockIdx.x * 4 + wi;
    if (item >= items) return;
    uint32_t* out = outs[wi];
    const int64_t s0 = (int64_t)item * 256, s1 = min(n, s0 + 256);
    if (lane == 0) nhome[wi] = 0;
    __syncwarp();
    for (int64_t b = s0; b < s1; b += 32) {
        const int64_t sp = b + lane;
        const bool head = sp < s1 && (sp == s0 || cell_of_pos[sp] != cell_of_pos[sp - 1]);
        const uint32_t bal = __ballot_sync(0xffffffffu, head);
        if (head) {
            const int pos = nhome[wi] + __popc(bal & lanemask_lt());
            if (pos < kHomeMax) homes[wi][pos] = cell_of_pos[sp];
        }
        __syncwarp();
        if (lane == 0) nhome[wi] = min(kHomeMax, nhome[wi] + __popc(bal));
        __syncwarp();
    }
    const int nh = nhome[wi];
    int cnt = 0;
    // Appends tile t unless present (every lane tracks cnt).
    auto add = [&](uint32_t t) {
        if (cnt >= kPrioMax || t >= (uint32_t)col_tiles) return;
        const bool dup = (lane < cnt && out[lane] == t) || (lane + 32 < cnt && out[lane + 32] == t);
        if (__any_sync(0xffffffffu, dup)) return;
        if (lane == 0) out[cnt] = t;
        cnt++;
        __syncwarp();
    };
    if (self_tile) add((uint32_t)item);  // a self solve's own tile (query solves have none)
    const int kk = min(ka, kAnchorNeighbours);
    for (int j = -1; j < kk && cnt < kPrioMax; ++j) {
        for (int hh = 0; hh < nh && cnt < kPrioMax; ++hh) {
            const uint32_t h = homes[wi][hh];
            const uint32_t c = j < 0 ? h : anchor_nb[(int64_t)h * ka + j];
            if (c >= (uint32_t)m) continue;
            const uint32_t a = cell_start[c], b = cell_start[c + 1];
            if (b <= a) continue;
            for (uint32_t t = a / 256; t <= (b - 1) / 256 && cnt < kPrioMax; ++t) add(t);
        }
    }
    __syncwarp();
    for (int t = lane; t < cnt; t += 32) prio[(int64_t)item * kPrioMax + t] = out[t];
    if (lane == 0) prio_cnt[item] = (uint32_t)cnt;
}


__device__ __forceinline__ float op_float(__half v) { return __half2float(v); }
__device__ __forceinline__ float op_float(__nv_bfloat16 v) { return __bfloat162float(v); }
// A 16-bit operand value from the low half of a word.
template <class T>
__device__ __forceinline__ float op_bits(uint32_t w);
template <>
__device__ __forceinline__ float op_bits<__half>(uint32_t w) {
    return __half2float(__ushort_as_half((unsigned short)(w & 0xffffu)));
}
template <>
__device__ __forceinline__ float op_bits<__nv_bfloat16>(uint32_t w) {
    return __bfloat162float(__ushort_as_bfloat16((unsigned short)(w & 0xffffu)));
}

// Balls of one tile: the whole tile and each of its cell segments (runs of
// rows of one cell; a cell lies in one region of the data, while a tile
// may straddle two far-apart cells).  Segments past kSegMax merge into the
// last.  Centres are stored dimension-major for coalesced pair tests.
constexpr int kSegMax = 8;
struct TileBalls {
    float* centre;      // [d][tiles]
    float* radius;      // [tiles]
    float* reach;       // [tiles]
    float* seg_centre;  // [kSegMax][d][tiles]
    float* seg_radius;  // [kSegMax][tiles]
    float* seg_reach;   // [kSegMax][tiles]
    uint32_t* nseg;     // [tiles]
};

// One block of 256 threads per column tile (= row block, the solve being a
// self-kNN): centres (means) and radii of the tile's quantised rows, and the
// reach U = max over the rows of sqrt(theta + A + delta), theta being the
// smaller of the row's two list thresholds.
template <class T>
__global__ void __launch_bounds__(256) tile_balls_kernel(const T* __restrict__ ops, int64_t n, int d, int tiles,
                                                         const uint32_t* __restrict__ cell_of_pos,
                                                         const float* __restrict__ theta, const float* __restrict__ bA,
                                                         const float* __restrict__ bdelta, TileBalls b) {
    __shared__ float part[8][64];
    __shared__ float centre[64];
    __shared__ float scentre[kSegMax][64];
    __shared__ int sstart[kSegMax + 1];
    __shared__ int wheads[8];
    __shared__ uint32_t rmax_all, rmax_seg[kSegMax];
    __shared__ uint32_t umax_all, umax_seg[kSegMax];
    const int tile = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t j = (int64_t)tile * 256 + threadIdx.x;
    const bool valid = j < n;
    const int rows = (int)min((int64_t)256, n - (int64_t)tile * 256);
    const T* row = ops + j * 64;
    // The row's 64 16-bit values, read once as eight 16-byte words.
    uint32_t rw[32];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint4 u = valid ? reinterpret_cast<const uint4*>(row)[q] : make_uint4(0u, 0u, 0u, 0u);
        rw[4 * q] = u.x;
        rw[4 * q + 1] = u.y;
        rw[4 * q + 2] = u.z;
        rw[4 * q + 3] = u.w;
    }
    // Segment of each row: the number of run heads at or before it, less one.
    const bool head = valid && (threadIdx.x == 0 || cell_of_pos[j] != cell_of_pos[j - 1]);
    const uint32_t hb = __ballot_sync(0xffffffffu, head);
    if (lane == 0) wheads[w] = __popc(hb);
    if (threadIdx.x == 0) {
        rmax_all = 0u;
        umax_all = 0u;
    }
    if (threadIdx.x < kSegMax) {
        rmax_seg[threadIdx.x] = 0u;
        umax_seg[threadIdx.x] = 0u;
    }
    __syncthreads();
    int before = 0, nheads = 0;
    for (int q = 0; q < 8; ++q) {
        before += q < w ? wheads[q] : 0;
        nheads += wheads[q];
    }
    const int nseg = min(nheads, kSegMax);
    const int seg = min(before + __popc(hb & lanemask_lt()) + (head ? 1 : 0) - 1, kSegMax - 1);
    if (head && seg == before + __popc(hb & lanemask_lt())) sstart[seg] = threadIdx.x;
    if (threadIdx.x == 0) sstart[nseg] = rows;
#pragma unroll
    for (int t = 0; t < 64; ++t) {
        if (t < d) {
            float v = valid ? op_bits<T>(rw[t >> 1] >> (16 * (t & 1))) : 0.f;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) part[w][t] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < d) {
        float sum = 0.f;
        for (int q = 0; q < 8; ++q) sum += part[q][threadIdx.x];
        centre[threadIdx.x] = sum / (float)rows;
        b.centre[(int64_t)threadIdx.x * tiles + tile] = centre[threadIdx.x];
    }
    for (int p = threadIdx.x; p < nseg * d; p += blockDim.x) {
        const int sg = p / d, t = p % d;
        float sum = 0.f;
        for (int r = sstart[sg]; r < sstart[sg + 1]; ++r) sum += op_float(ops[((int64_t)tile * 256 + r) * 64 + t]);
        const float c = sum / (float)(sstart[sg + 1] - sstart[sg]);
        scentre[sg][t] = c;
        b.seg_centre[((int64_t)sg * d + t) * tiles + tile] = c;
    }
    __syncthreads();
    if (valid) {
        // Squared distances to both centres in f32: a sum of d non-negative
        // rounded squares of rounded differences is at most (d + 2) units of
        // the last place below the exact value, so scaling by
        // 1 + (d + 4) 2^-23 (rounded up) bounds it from above.
        float r2 = 0.f, s2 = 0.f;
#pragma unroll
        for (int t = 0; t < 64; ++t) {
            if (t < d) {
                const float v = op_bits<T>(rw[t >> 1] >> (16 * (t & 1)));
                const float df = v - centre[t], ds = v - scentre[seg][t];
                r2 = fmaf(df, df, r2);
                s2 = fmaf(ds, ds, s2);
            }
        }
        const float grow = 1.0f + (float)(d + 4) * 1.1920929e-07f;
        r2 = __fmul_ru(r2, grow);
        s2 = __fmul_ru(s2, grow);
        const float th = fminf(theta[2 * j], theta[2 * j + 1]);
        // The reach sqrt(theta + A + delta), every step rounded up.
        const float v = __fadd_ru(__fadd_ru(th, bA[j]), bdelta[j]);
        const float u = isinf(th) && th > 0.f ? th : (v > 0.f ? __fsqrt_ru(v) : 0.f);
        // Non-negative floats order like their bit patterns.
        atomicMax(&rmax_all, __float_as_uint(r2));
        atomicMax(&rmax_seg[seg], __float_as_uint(s2));
        atomicMax(&umax_all, __float_as_uint(u));
        atomicMax(&umax_seg[seg], __float_as_uint(u));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        b.radius[tile] = __fmul_ru(__fsqrt_ru(__uint_as_float(rmax_all)), 1.0f + 1e-6f);
        b.reach[tile] = __uint_as_float(umax_all);
        b.nseg[tile] = (uint32_t)nseg;
    }
    if (threadIdx.x < nseg) {
        const int sg = threadIdx.x;
        b.seg_radius[(int64_t)sg * tiles + tile] = __fmul_ru(__fsqrt_ru(__uint_as_float(rmax_seg[sg])), 1.0f + 1e-6f);
        b.seg_reach[(int64_t)sg * tiles + tile] = __uint_as_float(umax_seg[sg]);
    }
}

// Whether a ball of reach u around centre I may hold a point within u of a
// point of ball T (conservatively true).  The f32 centre distance is within
// 1e-5 relative plus 3e-5 absolute (centre coordinates are at most 64 in
// magnitude); the slack covers both.  The test is made on squares in f32,
// each side moved past its own rounding (a few units of 2^-24 relative), so
// it never drops a tile the exact test keeps; a NaN keeps the tile.
__device__ __forceinline__ bool tile_needed(float dc2, float rI, float rT, float uI) {
    const float reach = (rI + rT + uI * (1.0f + 1e-5f) + 1e-4f) * (1.0f + 1e-6f);
    const float lhs = dc2 * ((1.0f - 1e-5f) * (1.0f - 1e-5f) * (1.0f - 1e-6f));
    return !(lhs >= reach * reach * (1.0f + 1e-6f));
}

// The cell-segment balls of all tiles, one row each (centres padded to 64
// dimensions with zeros), in tile order.
__global__ void flatten_segments_kernel(TileBalls b, int d, int tiles, const uint32_t* __restrict__ seg_off,
                                        float* __restrict__ fc, float* __restrict__ fr, float* __restrict__ fu,
                                        uint32_t* __restrict__ fo) {
    const int T = blockIdx.x;
    const int ns = (int)min(b.nseg[T], (uint32_t)kSegMax);
    const uint32_t o = seg_off[T];
    for (int p = threadIdx.x; p < ns * 64; p += blockDim.x) {
        const int sg = p / 64, t = p % 64;
        fc[(int64_t)(o + sg) * 64 + t] = t < d ? b.seg_centre[((int64_t)sg * d + t) * tiles + T] : 0.f;
    }
    if (threadIdx.x < ns) {
        fr[o + threadIdx.x] = b.seg_radius[(int64_t)threadIdx.x * tiles + T];
        fu[o + threadIdx.x] = b.seg_reach[(int64_t)threadIdx.x * tiles + T];
        fo[o + threadIdx.x] = (uint32_t)T;
    }
}

// All pairs of segment balls, 64 x 64 per block step, 4 x 4 per thread:
// when segment i (of row block owner[i]) may reach segment j (of tile
// owner[j]), bit (owner[i], owner[j]) of the reach bitmap is set.  The
// segment count S is read on the device; blocks stride over the block pairs
// of the upper triangle, and each centre distance serves both directions.
constexpr int SP = 64;
__global__ void __launch_bounds__(256) segment_pairs_kernel(const float* __restrict__ fc, const float* __restrict__ fr,
                                                            const float* __restrict__ fu,
                                                            const uint32_t* __restrict__ fo,
                                                            const uint32_t* __restrict__ S_ptr, int d, int words,
                                                            uint32_t* __restrict__ bitmap) {
    // Rows padded by 4 floats: the transposing stores (consecutive t, same
    // r) then spread over 8 banks instead of one; float4 reads stay aligned.
    __shared__ __align__(16) float As[64][SP + 4];
    __shared__ __align__(16) float Bs[64][SP + 4];
    const int S = (int)*S_ptr;
    const int nb = (S + SP - 1) / SP;
    const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
    for (int64_t bp = blockIdx.x; bp < (int64_t)nb * nb; bp += gridDim.x) {
        const int bi = (int)(bp / nb), bj = (int)(bp % nb);
        if (bi > bj) continue;
        const int i0 = bi * SP, j0 = bj * SP;
        __syncthreads();
        for (int p = threadIdx.x; p < SP * 64; p += blockDim.x) {
            const int r = p / 64, t = p % 64;
            As[t][r] = i0 + r < S ? fc[(int64_t)(i0 + r) * 64 + t] : 0.f;
            Bs[t][r] = j0 + r < S ? fc[(int64_t)(j0 + r) * 64 + t] : 0.f;
        }
        __syncthreads();
        float acc[4][4] = {};
        for (int t = 0; t < d; ++t) {
            const float4 a4 = *reinterpret_cast<const float4*>(&As[t][ty * 4]);
            const float4 b4 = *reinterpret_cast<const float4*>(&Bs[t][tx * 4]);
            const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float df = av[p] - bv[q];
                    acc[p][q] = fmaf(df, df, acc[p][q]);
                }
        }
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int i = i0 + ty * 4 + p;
            if (i >= S) continue;
            const float ri = fr[i], ui = fu[i];
            const uint32_t oi = fo[i];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = j0 + tx * 4 + q;
                if (j >= S) continue;
                const float rj = fr[j];
                const uint32_t oj = fo[j];
                if (tile_needed(acc[p][q], ri, rj, ui))
                    atomicOr(bitmap + (int64_t)oi * words + (oj >> 5), 1u << (oj & 31));
                // Off the diagonal block, the same distance for j reaching i.
                if (bi != bj && tile_needed(acc[p][q], rj, ri, fu[j]))
                    atomicOr(bitmap + (int64_t)oj * words + (oi >> 5), 1u << (oi & 31));
            }
        }
    }
}

// One block per row block I: the tiles of its reach bitmap row that are not
// in its priority list, ascending, at entries[I * tiles ...].
__global__ void __launch_bounds__(256) tile_lists_kernel(const uint32_t* __restrict__ bitmap, int words, int tiles,
                                                         const uint32_t* __restrict__ prio,
                                                         const uint32_t* __restrict__ prio_cnt,
                                                         uint32_t* __restrict__ counts, uint32_t* __restrict__ entries,
                                                         int prio_stride = kPrioMax) {
    extern __shared__ uint32_t in_prio[];  // words
    __shared__ int wsum[8];
    const int I = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int pc = (int)min(prio_cnt[I], (uint32_t)min(prio_stride, (int)blockDim.x));
    for (int i = threadIdx.x; i < words; i += blockDim.x) in_prio[i] = 0u;
    __syncthreads();
    if (threadIdx.x < pc) {
        const uint32_t t = prio[(int64_t)I * prio_stride + threadIdx.x];
        if (t < (uint32_t)tiles) atomicOr(&in_prio[t >> 5], 1u << (t & 31));
    }
    __syncthreads();
    const uint32_t* row = bitmap + (int64_t)I * words;
    uint32_t* out = entries + (int64_t)I * tiles;
    int base = 0;
    for (int w0 = 0; w0 < words; w0 += 256) {
        const int wd = w0 + threadIdx.x;
        uint32_t bits = wd < words ? row[wd] & ~in_prio[wd] : 0u;
        int c = __popc(bits);
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        int before = 0, total = 0;
        for (int q = 0; q < 8; ++q) {
            before += q < w ? wsum[q] : 0;
            total += wsum[q];
        }
        int pos = base + before + incl - c;
        while (bits) {
            const int bt = __ffs(bits) - 1;
            bits &= bits - 1;
            out[pos++] = (uint32_t)(wd * 32 + bt);
        }
        base += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) counts[I] = (uint32_t)base;
}

// Operand rows (128 bytes each) and their per-row terms moved into list
// order; padding rows are zero like the operand kernel writes them.
// Eight lanes per row: lane q of a row copies the row's q-th 16-byte word of
// A and B (a warp writes four whole 128-byte rows at a time).
__global__ void gather_operands_kernel(const uint4* __restrict__ A0, const uint4* __restrict__ B0,
                                       const float* __restrict__ bA0, const float* __restrict__ eps0,
                                       const uint32_t* __restrict__ perm, int64_t n, int64_t n_pad,
                                       uint4* __restrict__ A16, uint4* __restrict__ B16, float* __restrict__ bA,
                                       float* __restrict__ eps) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = t >> 3;
    const int q = (int)(t & 7);
    if (s >= n_pad) return;
    if (s < n) {
        const int64_t r = perm[s];
        A16[s * 8 + q] = A0[r * 8 + q];
        B16[s * 8 + q] = B0[r * 8 + q];
        if (q == 0) {
            bA[s] = bA0[r];
            eps[s] = eps0[r];
        }
    } else {
        const uint4 z = make_uint4(0u, 0u, 0u, 0u);
        A16[s * 8 + q] = z;
        B16[s * 8 + q] = z;
        if (q == 0) {
            bA[s] = 0.f;
            eps[s] = 0.f;
        }
    }
}

// Keys that sort row blocks by decreasing count (stable, so ties keep
// block order).
__global__ void work_keys_kernel(const uint32_t* __restrict__ counts, int items, uint32_t* __restrict__ keys,
                                 unsigned long long* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= items) return;
    keys[i] = 0xffffu - min(counts[i], 0xffffu);
    vals[i] = (unsigned long long)i;
}

__global__ void narrow_kernel(const unsigned long long* __restrict__ vals, int items, uint32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < items) out[i] = (uint32_t)vals[i];
}

// One thread per 4-float group of an output row (stride is a multiple of 4
// for the padded layout; otherwise one float per thread).
// Segment centres transposed to [64][segs], so that threads reading one
// dimension of consecutive segments read consecutive words.
__global__ void transpose_centres_kernel(const float* __restrict__ fc, int64_t segs, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= segs * 64) return;
    out[(i % 64) * segs + i / 64] = fc[i];
}

// Query blocks against atlas tiles: for every (query segment, atlas segment)
// pair, the atlas tile may hold a candidate of the query block while
// tile_needed holds (the same test as a self solve's, with the query
// segment's reach).  One block per query segment at a time, its centre in
// shared memory; threads over the atlas segments.
__global__ void __launch_bounds__(256) cross_segment_pairs_kernel(
    const float* __restrict__ qc, const float* __restrict__ qr, const float* __restrict__ qu,
    const uint32_t* __restrict__ qo, const uint32_t* __restrict__ q_count, const float* __restrict__ act,
    const float* __restrict__ ar, const uint32_t* __restrict__ ao, int64_t asegs, int d, int words,
    uint32_t* __restrict__ bitmap) {
    __shared__ float c[64];
    const uint32_t sq = *q_count;
    for (uint32_t a = blockIdx.x; a < sq; a += gridDim.x) {
        __syncthreads();
        if (threadIdx.x < 64) c[threadIdx.x] = qc[(int64_t)a * 64 + threadIdx.x];
        __syncthreads();
        const float ra = qr[a], ua = qu[a];
        const uint32_t item = qo[a];
        for (int64_t b = threadIdx.x; b < asegs; b += blockDim.x) {
            float acc = 0.f;
            for (int t = 0; t < d; ++t) {
                const float df = c[t] - act[(int64_t)t * asegs + b];
                acc = fmaf(df, df, acc);
            }
            if (tile_needed(acc, ra, ar[b], ua)) {
                const uint32_t tb = ao[b];
                atomicOr(bitmap + (int64_t)item * words + (tb >> 5), 1u << (tb & 31));
            }
        }
    }
}

// Priority tiles of a block of routed queries.  A block of 256 queries sorted
// by cell may span many cells (queries are few per cell), so every cell of
// its rows counts: the tiles holding those cells, lowest first, then the
// tiles of their eight nearest neighbouring cells, at most kQueryPrio in all.
// One block of 256 threads per query block; two tile bitmaps in shared memory.
constexpr int kQueryPrio = 256;
constexpr int kQueryPrioNb = 8;
__global__ void __launch_bounds__(256) query_prio_kernel(const uint32_t* __restrict__ cell_of_pos, int64_t n,
                                                         const uint32_t* __restrict__ cell_start, int m,
                                                         const uint32_t* __restrict__ cell_nb, int col_tiles,
                                                         uint32_t* __restrict__ prio, uint32_t* __restrict__ prio_cnt) {
    extern __shared__ uint32_t qp_bm[];
    const int words = (col_tiles + 31) / 32;
    uint32_t* home = qp_bm;
    uint32_t* near = qp_bm + words;
    const int I = blockIdx.x;
    for (int i = threadIdx.x; i < 2 * words; i += blockDim.x) qp_bm[i] = 0u;
    __syncthreads();
    const int64_t p = (int64_t)I * 256 + threadIdx.x;
    auto mark = [&](uint32_t* bm, uint32_t c) {
        if (c >= (uint32_t)m) return;
        const uint32_t a = cell_start[c], b = cell_start[c + 1];
        if (b <= a) return;
        for (uint32_t t = a / 256; t <= (b - 1) / 256 && t < (uint32_t)col_tiles; ++t)
            atomicOr(&bm[t >> 5], 1u << (t & 31));
    };
    if (p < n) {
        const uint32_t c = cell_of_pos[p];
        // Rows of one cell come together: the first of each run marks for all.
        if (p == (int64_t)I * 256 || cell_of_pos[p - 1] != c) {
            mark(home, c);
            if (c < (uint32_t)m)
                for (int j = 0; j < kQueryPrioNb; ++j) mark(near, cell_nb[(int64_t)c * kAnchorNeighbours + j]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t* out = prio + (int64_t)I * kQueryPrio;
        int cnt = 0;
        for (int w = 0; w < words && cnt < kQueryPrio; ++w) {
            uint32_t bits = home[w];
            while (bits && cnt < kQueryPrio) {
                out[cnt++] = (uint32_t)(w * 32 + __ffs(bits) - 1);
                bits &= bits - 1;
            }
        }
        for (int w = 0; w < words && cnt < kQueryPrio; ++w) {
            uint32_t bits = near[w] & ~home[w];
            while (bits && cnt < kQueryPrio) {
                out[cnt++] = (uint32_t)(w * 32 + __ffs(bits) - 1);
                bits &= bits - 1;
            }
        }
        prio_cnt[I] = (uint32_t)cnt;
    }
}

// A row block's tile list cut into `segs` contiguous chunks of equal size,
// one per column segment, so that each segment of a row block is its own
// work item: dst row (block * segs + segment), `dst_stride` entries apart.
// Contiguous, not dealt round robin: the list starts with the tiles nearest
// the block, and one segment that sees them all finds a threshold near the
// rows' k-th distance, which the others then share; tiles dealt out one by
// one would leave every segment's own k-th smallest far out.  One block per
// row block.
__global__ void split_lists_kernel(const uint32_t* __restrict__ src, int src_stride, const uint32_t* __restrict__ cnt,
                                   int segs, uint32_t* __restrict__ dst, int dst_stride,
                                   uint32_t* __restrict__ dst_cnt) {
    const int I = blockIdx.x;
    const int c = (int)min(cnt[I], (uint32_t)src_stride);
    const int chunk = (c + segs - 1) / segs;  // <= dst_stride = ceil(src_stride / segs)
    for (int t = threadIdx.x; t < c; t += blockDim.x)
        dst[((int64_t)I * segs + t / chunk) * dst_stride + t % chunk] = src[(int64_t)I * src_stride + t];
    if (threadIdx.x < segs)
        dst_cnt[(int64_t)I * segs + threadIdx.x] = (uint32_t)max(0, min(chunk, c - (int)threadIdx.x * chunk));
}

// Per row, its shared threshold as both part thresholds (the layout the
// tile balls read).
__global__ void row_theta_pairs_kernel(const uint32_t* __restrict__ row_theta, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = row_theta[i];
    const float t = k == 0xffffffffu ? __int_as_float(0x7f800000) : key_float(k);  // none yet: reach everything
    out[2 * i] = t;
    out[2 * i + 1] = t;
}

__global__ void gather_rows_kernel(const float* __restrict__ x, const uint32_t* __restrict__ perm, int64_t n, int d,
                                   int stride, float* __restrict__ xs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if ((stride & 3) == 0) {
        const int groups = stride >> 2;
        if (i >= n * groups) return;
        const int64_t s = i / groups;
        const int t0 = (int)(i - s * groups) * 4;
        const uint32_t r = perm[s];
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = (r == 0xffffffffu || t0 + e >= d) ? 0.f : x[(int64_t)r * d + t0 + e];
        reinterpret_cast<float4*>(xs + s * stride)[t0 >> 2] = make_float4(v[0], v[1], v[2], v[3]);
        return;
    }
    if (i >= n * stride) return;
    const int64_t s = i / stride, t = i % stride;
    const uint32_t r = perm[s];
    xs[i] = (r == 0xffffffffu || t >= d) ? 0.f : x[(int64_t)r * d + t];
}

}  // namespace

// Row blocks sorted by decreasing count into `order`; scratch holds
// work_order_scratch(items) bytes.
size_t work_order_scratch(int items) {
    const int nb = radix_blocks(items);
    return align_up(4 * (size_t)items) * 2 + align_up(8 * (size_t)items) * 2 + align_up(4 * ((size_t)256 * nb + 16)) +
           align_up(4 * scan_scratch_elems((int64_t)256 * nb));
}

cudaError_t sort_by_work(scrust_context* ctx, const uint32_t* counts, int items, char* scratch, uint32_t* order) {
    const int nb = radix_blocks(items);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = scratch + off;
        off += align_up(bytes);
        return p;
    };
    uint32_t* kA = (uint32_t*)take(4 * (size_t)items);
    uint32_t* kB = (uint32_t*)take(4 * (size_t)items);
    unsigned long long* vA = (unsigned long long*)take(8 * (size_t)items);
    unsigned long long* vB = (unsigned long long*)take(8 * (size_t)items);
    uint32_t* hist = (uint32_t*)take(4 * ((size_t)256 * nb + 16));
    const size_t scan_elems = scan_scratch_elems((int64_t)256 * nb);
    uint32_t* scan = (uint32_t*)take(4 * scan_elems);
    work_keys_kernel<<<(items + 255) / 256, 256, 0, ctx->stream>>>(counts, items, kA, vA);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint32_t* ks = nullptr;
    unsigned long long* vs = nullptr;
    if ((e = radix_sort_pairs(ctx, kA, vA, kB, vB, items, 16, hist, scan, scan_elems, &ks, &vs)) != cudaSuccess)
        return e;
    narrow_kernel<<<(items + 255) / 256, 256, 0, ctx->stream>>>(vs, items, order);
    ctx->launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_gather_rows(const float* x, const uint32_t* perm, int64_t n, int d, int stride, float* xs,
                               cudaStream_t s) {
    const int64_t threads = (stride & 3) == 0 ? n * (stride >> 2) : n * stride;
    gather_rows_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(x, perm, n, d, stride, xs);
    return cudaGetLastError();
}


int32_t build_row_order(scrust_context* ctx, const float* x, int64_t n, int d, const double* means,
                        uint32_t* max_bits, bool cosine, bool bf16, void* A16, void* B16, float* bA, float* beps,
                        float* bdelta, float* beps2, RowOrder* out, scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int64_t n_pad = (n + 255) / 256 * 256;
    const int items = (int)(n_pad / 256);
    const int64_t m = std::min<int64_t>(std::max<int64_t>(n / 256, 2), kMaxAnchors);
    const int64_t m_pad = (m + 255) / 256 * 256;
    const int nblocks = radix_blocks(n);
    const size_t scan_elems = scan_scratch_elems(std::max<int64_t>((int64_t)256 * nblocks, m + 1));

    // Carve the ordering slot.
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes);
        return o;
    };
    const size_t o_src = take(4 * (size_t)m), o_anc = take(4 * (size_t)m * d), o_aA = take(128 * (size_t)m_pad),
                 o_aB = take(128 * (size_t)m_pad), o_arb = take(8 * (size_t)m_pad), o_kA = take(4 * (size_t)n),
                 o_kB = take(4 * (size_t)n), o_vA = take(8 * (size_t)n), o_vB = take(8 * (size_t)n),
                 o_perm = take(4 * (size_t)n), o_cell = take(4 * (size_t)n), o_ccnt = take(4 * (size_t)(m + 1)),
                 o_cst = take(4 * (size_t)(m + 1)), o_nb = take(4 * (size_t)m * kAnchorNeighbours),
                 o_nb2 = take(4 * (size_t)m * kAnchorNeighbours), o_rank = take(4 * (size_t)m),
                 o_adist = take(4 * (size_t)m * (size_t)m),
                 o_prio = take(4 * (size_t)items * kPrioMax), o_pc = take(4 * (size_t)items),
                 o_theta = take(8 * (size_t)n_pad), o_po = take(4 * (size_t)items),
                 o_best = take(16 * (size_t)n_pad), o_A0 = take(128 * (size_t)n_pad),
                 o_B0 = take(128 * (size_t)n_pad), o_bA0 = take(4 * (size_t)n_pad), o_eps0 = take(4 * (size_t)n_pad),
                 o_ws = take(work_order_scratch(items)),
                 o_hist = take(4 * ((size_t)256 * nblocks + 16)), o_scan = take(4 * scan_elems);
    char* base = (char*)ws_get(ctx, SLOT_ORDER, off, &e);
    if (!base) return cuda_fail(st, e, "ordering: workspace");
    uint32_t* src = (uint32_t*)(base + o_src);
    float* anc = (float*)(base + o_anc);
    uint32_t *keysA = (uint32_t*)(base + o_kA), *keysB = (uint32_t*)(base + o_kB);
    unsigned long long *valsA = (unsigned long long*)(base + o_vA), *valsB = (unsigned long long*)(base + o_vB);
    uint32_t* perm = (uint32_t*)(base + o_perm);
    uint32_t* cell_of_pos = (uint32_t*)(base + o_cell);
    uint32_t* cell_count = (uint32_t*)(base + o_ccnt);
    uint32_t* cell_start = (uint32_t*)(base + o_cst);
    uint32_t* anchor_nb = (uint32_t*)(base + o_nb);
    uint32_t* cell_nb = (uint32_t*)(base + o_nb2);
    uint32_t* rank = (uint32_t*)(base + o_rank);
    uint32_t* prio = (uint32_t*)(base + o_prio);
    uint32_t* prio_cnt = (uint32_t*)(base + o_pc);
    float* arb = (float*)(base + o_arb);

    // Anchors, and both operand sets in the input order.
    anchors_kernel<<<(unsigned)m, 64, 0, s>>>(x, d, n, m, src, anc);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "ordering: anchors");
    // The anchor neighbourhoods and the walk that orders the cells run on the
    // copy stream beside the operands and the rows x anchors pass below; the
    // main stream waits for them before the cells are formed.
    const size_t chain_smem = 4 * (size_t)((((m + 3) / 4 + 1) + 1) / 2 * 2) + 2 * (size_t)m * kChainNb;
    if ((e = set_smem_limit(ctx, (const void*)anchor_chain_kernel, (int)chain_smem)) != cudaSuccess ||
        (e = cudaEventRecord(ctx->copy_ev, s)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev, 0)) != cudaSuccess)
        return cuda_fail(st, e, "ordering: anchor walk");
    {
        float* adist = (float*)(base + o_adist);
        const dim3 grid((unsigned)((m + 63) / 64), (unsigned)((m + 63) / 64));
        anchor_dist_kernel<<<grid, 256, 0, ctx->copy_stream>>>(anc, (int)m, d, adist);
        anchor_top_kernel<<<(unsigned)((m + 3) / 4), 128, 0, ctx->copy_stream>>>(adist, (int)m, anchor_nb);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "ordering: anchor neighbours");
        ctx->launches += 2;
    }
    anchor_chain_kernel<<<1, kChainThreads, chain_smem, ctx->copy_stream>>>(anchor_nb, (int)m, rank);
    relabel_neighbours_kernel<<<(unsigned)((m * kAnchorNeighbours + 255) / 256), 256, 0, ctx->copy_stream>>>(
        anchor_nb, rank, (int)m, cell_nb);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaEventRecord(ctx->copy_ev, ctx->copy_stream)) != cudaSuccess)
        return cuda_fail(st, e, "ordering: anchor walk");
    ctx->launches += 2;

    void* A0 = base + o_A0;
    void* B0 = base + o_B0;
    float* bA0 = (float*)(base + o_bA0);
    float* eps0 = (float*)(base + o_eps0);
    if ((e = launch_tensor_operands(x, n, n_pad, d, means, max_bits, cosine, bf16, nullptr, A0, B0, bA0, eps0,
                                    max_bits + 1, max_bits + 2, s)) != cudaSuccess ||
        (e = launch_tensor_bounds(n, bA0, eps0, max_bits + 1, max_bits + 2, bdelta, beps2, s)) != cudaSuccess ||
        (e = launch_tensor_operands(x, m, m_pad, d, means, max_bits, cosine, bf16, src, base + o_aA, base + o_aB, arb,
                                    arb + m_pad, max_bits + 1, max_bits + 2, s)) != cudaSuccess)
        return cuda_fail(st, e, "ordering: operands");
    ctx->launches += 4;

    // Rows x anchors with k = 1 on the tensor cores, keeping only each row's
    // nearest anchor.
    KnnPlan px;
    px.nq = n;
    px.nr = m;
    px.d = d;
    px.k = 1;
    px.self = false;
    px.form = SCRUST_FORM_TENSOR;
    Lists lx;  // no storage: the pass keeps no lists
    lx.cap = 64;
    lx.ctot = 64 + 128;
    lx.segments = 2;
    px.cap = lx.cap;
    px.ctot = lx.ctot;
    px.segments = lx.segments;
    px.max_ctas = ctx->sm_count - 1;
    unsigned long long* best = (unsigned long long*)(base + o_best);
    if ((e = launch_tensor_candidates(ctx, px, A0, n_pad, base + o_aB, m_pad, bA0, bdelta, beps2, lx, bf16, nullptr,
                                      false, nullptr, nullptr, nullptr, best)) != cudaSuccess)
        return cuda_fail(st, e, "ordering: anchor candidates");
    const int op_words = (d + 3 + 7) / 8;  // 16-byte words of an operand row holding values
    if (bf16)
        nearest_anchor_kernel<__nv_bfloat16><<<(unsigned)((n * 8 + 255) / 256), 256, 0, s>>>(
            best, n, m, (const __nv_bfloat16*)A0, (const __nv_bfloat16*)(base + o_aB), op_words, keysA, valsA);
    else
        nearest_anchor_kernel<__half><<<(unsigned)((n * 8 + 255) / 256), 256, 0, s>>>(
            best, n, m, (const __half*)A0, (const __half*)(base + o_aB), op_words, keysA, valsA);
    // The walk ranks (copy stream) are needed from here on.
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamWaitEvent(s, ctx->copy_ev, 0)) != cudaSuccess)
        return cuda_fail(st, e, "ordering: nearest anchor");
    anchor_rank_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(keysA, n, rank);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "ordering: nearest anchor");
    ctx->launches += 3;

    // Stable sort of the rows by anchor: the permutation and the cells.
    int bits = 1;
    while (((int64_t)1 << bits) < m) bits++;
    uint32_t* skeys = nullptr;
    unsigned long long* svals = nullptr;
    if ((e = radix_sort_pairs(ctx, keysA, valsA, keysB, valsB, n, bits, (uint32_t*)(base + o_hist),
                              (uint32_t*)(base + o_scan), scan_elems, &skeys, &svals)) != cudaSuccess)
        return cuda_fail(st, e, "ordering: sort");
    if ((e = cudaMemsetAsync(cell_count, 0, 4 * (size_t)(m + 1), s)) != cudaSuccess)
        return cuda_fail(st, e, "ordering: memset");
    unpack_perm_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(skeys, svals, n, perm, cell_of_pos, cell_count);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "ordering: permutation");
    if ((e = device_exclusive_scan(ctx, cell_count, cell_start, m + 1, (uint32_t*)(base + o_scan), scan_elems)) !=
        cudaSuccess)
        return cuda_fail(st, e, "ordering: cell scan");

    // The priority tiles of every work item.
    prio_tiles_kernel<<<(unsigned)((items + 3) / 4), 128, 0, s>>>(cell_of_pos, n, cell_start, (int)m, cell_nb,
                                                                  kAnchorNeighbours, items, items, prio, prio_cnt);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "ordering: priority tiles");
    ctx->launches += 2;
    if ((e = sort_by_work(ctx, prio_cnt, items, base + o_ws, (uint32_t*)(base + o_po))) != cudaSuccess)
        return cuda_fail(st, e, "ordering: work order");
    // The operands in list order (bounds follow in the caller).
    gather_operands_kernel<<<(unsigned)((n_pad * 8 + 255) / 256), 256, 0, s>>>(
        (const uint4*)A0, (const uint4*)B0, bA0, eps0, perm, n, n_pad, (uint4*)A16, (uint4*)B16, bA, beps);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "ordering: operands");
    ctx->launches += 1;
    out->perm = perm;
    out->prio = prio;
    out->prio_cnt = prio_cnt;
    out->prio_order = (const uint32_t*)(base + o_po);
    out->theta = (float*)(base + o_theta);
    out->cell_of_pos = cell_of_pos;
    out->anchors = m;
    out->anchors_pad = m_pad;
    out->anchor_B16 = base + o_aB;
    out->anchor_rank = rank;
    out->cell_start = cell_start;
    out->cell_nb = cell_nb;
    return SCRUST_OK;
}

int32_t build_second_pass(scrust_context* ctx, const void* A16, bool bf16, int64_t n, int d, const RowOrder& order,
                          const float* bA, const float* bdelta, TileLists* out, scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int tiles = (int)((n + 255) / 256);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes);
        return o;
    };
    const int words = (tiles + 31) / 32;
    const int64_t smax = (int64_t)tiles * kSegMax;
    const size_t scan_elems = scan_scratch_elems((int64_t)tiles + 1);
    const size_t o_c = take(4 * (size_t)d * tiles), o_r = take(4 * (size_t)tiles), o_u = take(4 * (size_t)tiles),
                 o_sc = take(4 * (size_t)kSegMax * d * tiles), o_sr = take(4 * (size_t)kSegMax * tiles),
                 o_su = take(4 * (size_t)kSegMax * tiles), o_ns = take(4 * ((size_t)tiles + 1)),
                 o_so = take(4 * ((size_t)tiles + 1)), o_fc = take(4 * 64 * (size_t)smax), o_fr = take(4 * (size_t)smax),
                 o_fu = take(4 * (size_t)smax), o_fo = take(4 * (size_t)smax), o_scan = take(4 * scan_elems),
                 o_bm = take(4 * (size_t)tiles * words), o_cnt = take(4 * ((size_t)tiles + 1)),
                 o_wo = take(4 * (size_t)tiles), o_ws = take(work_order_scratch(tiles)),
                 o_ent = take(4 * (size_t)tiles * (size_t)tiles);
    char* base = (char*)ws_get(ctx, SLOT_PRUNE, off, &e);
    if (!base) return cuda_fail(st, e, "pruning: workspace");
    TileBalls balls;
    balls.centre = (float*)(base + o_c);
    balls.radius = (float*)(base + o_r);
    balls.reach = (float*)(base + o_u);
    balls.seg_centre = (float*)(base + o_sc);
    balls.seg_radius = (float*)(base + o_sr);
    balls.seg_reach = (float*)(base + o_su);
    balls.nseg = (uint32_t*)(base + o_ns);
    uint32_t* seg_off = (uint32_t*)(base + o_so);
    float* fc = (float*)(base + o_fc);
    float* fr = (float*)(base + o_fr);
    float* fu = (float*)(base + o_fu);
    uint32_t* fo = (uint32_t*)(base + o_fo);
    uint32_t* bitmap = (uint32_t*)(base + o_bm);
    uint32_t* counts = (uint32_t*)(base + o_cnt);
    uint32_t* entries = (uint32_t*)(base + o_ent);
    if ((e = cudaMemsetAsync(balls.nseg + tiles, 0, sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(bitmap, 0, 4 * (size_t)tiles * words, s)) != cudaSuccess)
        return cuda_fail(st, e, "pruning: memset");
    if (bf16)
        tile_balls_kernel<__nv_bfloat16><<<tiles, 256, 0, s>>>((const __nv_bfloat16*)A16, n, d, tiles,
                                                               order.cell_of_pos, order.theta, bA, bdelta, balls);
    else
        tile_balls_kernel<__half><<<tiles, 256, 0, s>>>((const __half*)A16, n, d, tiles, order.cell_of_pos,
                                                        order.theta, bA, bdelta, balls);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "pruning: tile balls");
    if ((e = device_exclusive_scan(ctx, balls.nseg, seg_off, (int64_t)tiles + 1, (uint32_t*)(base + o_scan),
                                   scan_elems)) != cudaSuccess)
        return cuda_fail(st, e, "pruning: segment scan");
    flatten_segments_kernel<<<tiles, 64, 0, s>>>(balls, d, tiles, seg_off, fc, fr, fu, fo);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "pruning: segments");
    segment_pairs_kernel<<<8 * ctx->sm_count, 256, 0, s>>>(fc, fr, fu, fo, seg_off + tiles, d, words, bitmap);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "pruning: segment pairs");
    const size_t lists_smem = 4 * (size_t)words;
    if ((e = set_smem_limit(ctx, (const void*)tile_lists_kernel, (int)lists_smem)) !=
        cudaSuccess)
        return cuda_fail(st, e, "pruning: tile lists");
    tile_lists_kernel<<<tiles, 256, lists_smem, s>>>(bitmap, words, tiles, order.prio, order.prio_cnt, counts, entries);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "pruning: tile lists");
    ctx->launches += 3;
    if ((e = sort_by_work(ctx, counts, tiles, base + o_ws, (uint32_t*)(base + o_wo))) != cudaSuccess)
        return cuda_fail(st, e, "pruning: work order");
    out->tiles = entries;
    out->offset = nullptr;
    out->count = counts;
    out->stride = tiles;
    out->order = (const uint32_t*)(base + o_wo);
    return SCRUST_OK;
}

// ---- query solves against an ordered atlas -------------------------------------

namespace {

void launch_tile_balls(bool bf16, const void* ops, int64_t n, int d, int tiles, const uint32_t* cell_of_pos,
                       const float* theta, const float* bA, const float* bdelta, const TileBalls& b, cudaStream_t s) {
    if (bf16)
        tile_balls_kernel<__nv_bfloat16><<<tiles, 256, 0, s>>>((const __nv_bfloat16*)ops, n, d, tiles, cell_of_pos,
                                                               theta, bA, bdelta, b);
    else
        tile_balls_kernel<__half><<<tiles, 256, 0, s>>>((const __half*)ops, n, d, tiles, cell_of_pos, theta, bA,
                                                        bdelta, b);
}

// The per-tile ball arrays of `tiles` tiles, laid out from byte `at` of
// `base`; returns the end of the layout.
size_t carve_balls(char* base, size_t at, int tiles, int d, TileBalls* b) {
    auto take = [&](size_t bytes) {
        const size_t a = at;
        at = align_up(at + bytes);
        return base + a;
    };
    b->centre = (float*)take(4 * (size_t)d * tiles);
    b->radius = (float*)take(4 * (size_t)tiles);
    b->reach = (float*)take(4 * (size_t)tiles);
    b->seg_centre = (float*)take(4 * (size_t)kSegMax * d * tiles);
    b->seg_radius = (float*)take(4 * (size_t)kSegMax * tiles);
    b->seg_reach = (float*)take(4 * (size_t)kSegMax * tiles);
    b->nseg = (uint32_t*)take(4 * ((size_t)tiles + 1));
    return at;
}

}  // namespace

void atlas_order_free(AtlasOrder* o) {
    if (!o) return;
    void* ptrs[] = {o->B16, o->perm, o->rows, o->anchor_B16, o->anchor_rank, o->cell_start,
                    o->cell_nb, o->seg_centre_t, o->seg_radius, o->seg_tile};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    *o = AtlasOrder{};
}

int32_t atlas_order_build(scrust_context* ctx, const float* atlas, int64_t m, int d, const double* means,
                          uint32_t* words, bool bf16, AtlasOrder* out, scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    AtlasOrder o;
    o.m = m;
    o.m_pad = (m + 255) / 256 * 256;
    o.d = d;
    o.bf16 = bf16;
    const int tiles = (int)(o.m_pad / 256);
    const int P = padded_row_floats(d);
    // Scratch of the build: operands and row terms in list order, the tile
    // balls and their flattened segments.
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off = align_up(off + bytes);
        return at;
    };
    const int64_t smax = (int64_t)tiles * kSegMax;
    const size_t scan_elems = scan_scratch_elems((int64_t)tiles + 1);
    const size_t o_A = take(128 * (size_t)o.m_pad), o_t = take(4 * 4 * (size_t)o.m_pad),
                 o_th = take(4 * 2 * (size_t)o.m_pad), o_so = take(4 * ((size_t)tiles + 1)),
                 o_fc = take(4 * 64 * (size_t)smax), o_fr = take(4 * (size_t)smax), o_fu = take(4 * (size_t)smax),
                 o_fo = take(4 * (size_t)smax), o_scan = take(4 * scan_elems);
    TileBalls balls;
    const size_t total = carve_balls(nullptr, off, tiles, d, &balls);
    char* base = nullptr;
    if ((e = cudaMalloc(&base, total)) != cudaSuccess || (e = cudaMalloc(&o.B16, 128 * (size_t)o.m_pad)) != cudaSuccess) {
        cudaFree(base);
        atlas_order_free(&o);
        cudaGetLastError();
        return cuda_fail(st, e, "atlas ordering: allocation");
    }
    carve_balls(base, off, tiles, d, &balls);
    float* terms = (float*)(base + o_t);
    float *bA = terms, *beps = terms + o.m_pad, *bdelta = terms + 2 * o.m_pad, *beps2 = terms + 3 * o.m_pad;
    RowOrder ord;
    int32_t rc = build_row_order(ctx, atlas, m, d, means, words, false, bf16, base + o_A, o.B16, bA, beps, bdelta,
                                 beps2, &ord, st);
    auto bail = [&](int32_t code) {
        cudaStreamSynchronize(s);
        cudaFree(base);
        atlas_order_free(&o);
        cudaGetLastError();
        return code;
    };
    if (rc) return bail(rc);
    o.anchors = ord.anchors;
    o.anchors_pad = ord.anchors_pad;
    const size_t na = (size_t)o.anchors;
    if ((e = cudaMalloc(&o.perm, 4 * (size_t)m)) != cudaSuccess ||
        (e = cudaMalloc(&o.rows, 4 * (size_t)m * P)) != cudaSuccess ||
        (e = cudaMalloc(&o.anchor_B16, 128 * (size_t)o.anchors_pad)) != cudaSuccess ||
        (e = cudaMalloc(&o.anchor_rank, 4 * na)) != cudaSuccess ||
        (e = cudaMalloc(&o.cell_start, 4 * (na + 1))) != cudaSuccess ||
        (e = cudaMalloc(&o.cell_nb, 4 * na * kAnchorNeighbours)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o.perm, ord.perm, 4 * (size_t)m, cudaMemcpyDeviceToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o.anchor_B16, ord.anchor_B16, 128 * (size_t)o.anchors_pad, cudaMemcpyDeviceToDevice,
                             s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o.anchor_rank, ord.anchor_rank, 4 * na, cudaMemcpyDeviceToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(o.cell_start, ord.cell_start, 4 * (na + 1), cudaMemcpyDeviceToDevice, s)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(o.cell_nb, ord.cell_nb, 4 * na * kAnchorNeighbours, cudaMemcpyDeviceToDevice, s)) !=
            cudaSuccess ||
        (e = launch_gather_rows(atlas, ord.perm, m, d, P, o.rows, s)) != cudaSuccess ||
        (e = launch_tensor_bounds(m, bA, beps, words + 1, words + 2, bdelta, beps2, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(base + o_th, 0, 4 * 2 * (size_t)o.m_pad, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(balls.nseg + tiles, 0, sizeof(uint32_t), s)) != cudaSuccess)
        return bail(cuda_fail(st, e, "atlas ordering"));
    // The cell-segment balls of the atlas tiles (their reach is not used).
    uint32_t* seg_off = (uint32_t*)(base + o_so);
    float* fc = (float*)(base + o_fc);
    launch_tile_balls(bf16, base + o_A, m, d, tiles, ord.cell_of_pos, (const float*)(base + o_th), bA, bdelta,
                              balls, s);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = device_exclusive_scan(ctx, balls.nseg, seg_off, (int64_t)tiles + 1, (uint32_t*)(base + o_scan),
                                   scan_elems)) != cudaSuccess)
        return bail(cuda_fail(st, e, "atlas ordering: tile balls"));
    flatten_segments_kernel<<<tiles, 64, 0, s>>>(balls, d, tiles, seg_off, fc, (float*)(base + o_fr),
                                                 (float*)(base + o_fu), (uint32_t*)(base + o_fo));
    uint32_t segs = 0;
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(&segs, seg_off + tiles, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return bail(cuda_fail(st, e, "atlas ordering: segments"));
    o.segs = segs;
    if ((e = cudaMalloc(&o.seg_centre_t, 4 * 64 * (size_t)std::max<uint32_t>(segs, 1))) != cudaSuccess ||
        (e = cudaMalloc(&o.seg_radius, 4 * (size_t)std::max<uint32_t>(segs, 1))) != cudaSuccess ||
        (e = cudaMalloc(&o.seg_tile, 4 * (size_t)std::max<uint32_t>(segs, 1))) != cudaSuccess ||
        (e = cudaMemcpyAsync(o.seg_radius, base + o_fr, 4 * (size_t)segs, cudaMemcpyDeviceToDevice, s)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(o.seg_tile, base + o_fo, 4 * (size_t)segs, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return bail(cuda_fail(st, e, "atlas ordering: segments"));
    if (segs) transpose_centres_kernel<<<(unsigned)((64 * (int64_t)segs + 255) / 256), 256, 0, s>>>(fc, segs,
                                                                                                 o.seg_centre_t);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return bail(cuda_fail(st, e, "atlas ordering: segments"));
    ctx->launches += 4;
    cudaFree(base);
    *out = o;
    return ok(st);
}

int32_t cross_ordered_enqueue(scrust_context* ctx, const AtlasOrder& at, const float* atlas_rows, const double* means,
                              const uint32_t* words, const float* dq, int64_t q, int k, uint32_t* d_idx,
                              float* d_dist, scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int d = at.d;
    const bool bf16 = at.bf16;
    const int64_t q_pad = (q + 255) / 256 * 256;
    const int items = (int)(q_pad / 256), col_tiles = (int)(at.m_pad / 256), words_t = (col_tiles + 31) / 32;
    // Column segments per row block, so that a small batch still fills the
    // GPU: each segment of a block is its own work item, and the segments of
    // a row share its threshold through HBM.
    // (At most 16: the rerank reads up to 32 lists of a row in registers;
    // and a count the sweep's segment split reproduces.)
    int csegs = std::max(1, std::min({16, col_tiles, (2 * ctx->sm_count + items - 1) / items}));
    while (csegs > 1 && (col_tiles + (col_tiles + csegs - 1) / csegs - 1) / ((col_tiles + csegs - 1) / csegs) != csegs)
        csegs--;
    const int work = items * csegs;
    const int ps = (kQueryPrio + csegs - 1) / csegs, es = (col_tiles + csegs - 1) / csegs;
    const int P = padded_row_floats(d);
    const int nblocks = radix_blocks(q);
    const int64_t smax = (int64_t)items * kSegMax;
    const size_t scan_elems =
        scan_scratch_elems(std::max<int64_t>((int64_t)256 * nblocks, std::max<int64_t>(items, at.anchors) + 1));
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t a = off;
        off = align_up(off + bytes);
        return a;
    };
    const size_t o_A0 = take(128 * (size_t)q_pad), o_B0 = take(128 * (size_t)q_pad), o_t0 = take(4 * 2 * (size_t)q_pad),
                 o_As = take(128 * (size_t)q_pad), o_Bs = take(128 * (size_t)q_pad), o_ts = take(4 * 4 * (size_t)q_pad),
                 o_w = take(64), o_best = take(16 * (size_t)q_pad), o_kA = take(4 * (size_t)q), o_kB = take(4 * (size_t)q),
                 o_vA = take(8 * (size_t)q), o_vB = take(8 * (size_t)q), o_qp = take(4 * (size_t)q),
                 o_cell = take(4 * (size_t)q), o_cc = take(4 * ((size_t)at.anchors + 1)),
                 o_xs = take(4 * (size_t)q * P), o_prio = take(4 * (size_t)items * kQueryPrio),
                 o_pc = take(4 * (size_t)items), o_ps = take(4 * (size_t)work * ps), o_psc = take(4 * (size_t)work),
                 o_po = take(4 * (size_t)work), o_po2 = take(4 * (size_t)work), o_ws = take(work_order_scratch(work)),
                 o_rt = take(4 * (size_t)q_pad), o_th = take(4 * 2 * (size_t)csegs * q_pad),
                 o_th2 = take(4 * 2 * (size_t)q_pad), o_so = take(4 * ((size_t)items + 1)),
                 o_fc = take(4 * 64 * (size_t)smax), o_fr = take(4 * (size_t)smax), o_fu = take(4 * (size_t)smax),
                 o_fo = take(4 * (size_t)smax), o_bm = take(4 * (size_t)items * words_t),
                 o_cnt = take(4 * ((size_t)items + 1)), o_ent = take(4 * (size_t)items * col_tiles),
                 o_es = take(4 * (size_t)work * es), o_esc = take(4 * (size_t)work),
                 o_hist = take(4 * ((size_t)256 * nblocks + 16)), o_scan = take(4 * scan_elems);
    TileBalls qballs;
    const size_t total = carve_balls(nullptr, off, items, d, &qballs);
    char* base = (char*)ws_get(ctx, SLOT_XORDER, total, &e);
    if (!base) return cuda_fail(st, e, "query routing: workspace");
    carve_balls(base, off, items, d, &qballs);
    float* t0 = (float*)(base + o_t0);
    float *bA0 = t0, *eps0 = t0 + q_pad;
    float* ts = (float*)(base + o_ts);
    float *bA = ts, *beps = ts + q_pad, *bdelta = ts + 2 * q_pad, *beps2 = ts + 3 * q_pad;
    uint32_t* qwords = (uint32_t*)(base + o_w);
    uint32_t* qperm = (uint32_t*)(base + o_qp);
    uint32_t* cell_of_pos = (uint32_t*)(base + o_cell);
    uint32_t* prio = (uint32_t*)(base + o_prio);
    uint32_t* prio_cnt = (uint32_t*)(base + o_pc);
    uint32_t* row_theta = (uint32_t*)(base + o_rt);
    float* theta = (float*)(base + o_th);
    float* theta2 = (float*)(base + o_th2);
    float* xs = (float*)(base + o_xs);
    uint32_t* seg_off = (uint32_t*)(base + o_so);
    uint32_t* bitmap = (uint32_t*)(base + o_bm);
    uint32_t* counts = (uint32_t*)(base + o_cnt);
    uint32_t* entries = (uint32_t*)(base + o_ent);
    unsigned long long* best = (unsigned long long*)(base + o_best);

    // The queries' operands, in input order; every query's nearest anchor.
    if ((e = cudaMemsetAsync(qwords, 0, 64, s)) != cudaSuccess ||
        (e = launch_tensor_operands(dq, q, q_pad, d, means, words, false, bf16, nullptr, base + o_A0, base + o_B0, bA0,
                                    eps0, qwords, qwords + 1, s)) != cudaSuccess)
        return cuda_fail(st, e, "query routing: operands");
    KnnPlan px;
    px.nq = q;
    px.nr = at.anchors;
    px.d = d;
    px.k = 1;
    px.self = false;
    px.form = SCRUST_FORM_TENSOR;
    Lists lx;  // no storage: the pass keeps no lists
    lx.cap = 64;
    lx.ctot = 64 + 128;
    lx.segments = 2;
    px.cap = lx.cap;
    px.ctot = lx.ctot;
    px.segments = lx.segments;
    if ((e = launch_tensor_candidates(ctx, px, base + o_A0, q_pad, at.anchor_B16, at.anchors_pad, bA0, eps0, eps0, lx,
                                      bf16, nullptr, false, nullptr, nullptr, nullptr, best)) != cudaSuccess)
        return cuda_fail(st, e, "query routing: nearest anchor");
    const int op_words = (d + 3 + 7) / 8;  // 16-byte words of an operand row holding values
    if (bf16)
        nearest_anchor_kernel<__nv_bfloat16><<<(unsigned)((q * 8 + 255) / 256), 256, 0, s>>>(
            best, q, at.anchors, (const __nv_bfloat16*)(base + o_A0), (const __nv_bfloat16*)at.anchor_B16, op_words,
            (uint32_t*)(base + o_kA), (unsigned long long*)(base + o_vA));
    else
        nearest_anchor_kernel<__half><<<(unsigned)((q * 8 + 255) / 256), 256, 0, s>>>(
            best, q, at.anchors, (const __half*)(base + o_A0), (const __half*)at.anchor_B16, op_words,
            (uint32_t*)(base + o_kA), (unsigned long long*)(base + o_vA));
    anchor_rank_kernel<<<(unsigned)((q + 255) / 256), 256, 0, s>>>((uint32_t*)(base + o_kA), q, at.anchor_rank);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "query routing: nearest anchor");
    ctx->launches += 4;
    // The queries sorted by the walk place of their cell; their operands,
    // bounds and rows in that order.
    int bits = 1;
    while (((int64_t)1 << bits) < at.anchors) bits++;
    uint32_t* skeys = nullptr;
    unsigned long long* svals = nullptr;
    if ((e = radix_sort_pairs(ctx, (uint32_t*)(base + o_kA), (unsigned long long*)(base + o_vA),
                              (uint32_t*)(base + o_kB), (unsigned long long*)(base + o_vB), q, bits,
                              (uint32_t*)(base + o_hist), (uint32_t*)(base + o_scan), scan_elems, &skeys, &svals)) !=
            cudaSuccess ||
        (e = cudaMemsetAsync(base + o_cc, 0, 4 * ((size_t)at.anchors + 1), s)) != cudaSuccess)
        return cuda_fail(st, e, "query routing: sort");
    unpack_perm_kernel<<<(unsigned)((q + 255) / 256), 256, 0, s>>>(skeys, svals, q, qperm, cell_of_pos,
                                                                  (uint32_t*)(base + o_cc));
    gather_operands_kernel<<<(unsigned)((q_pad * 8 + 255) / 256), 256, 0, s>>>(
        (const uint4*)(base + o_A0), (const uint4*)(base + o_B0), bA0, eps0, qperm, q, q_pad, (uint4*)(base + o_As),
        (uint4*)(base + o_Bs), bA, beps);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = launch_tensor_bounds(q, bA, beps, words + 1, words + 2, bdelta, beps2, s)) != cudaSuccess ||
        (e = launch_gather_rows(dq, qperm, q, d, P, xs, s)) != cudaSuccess)
        return cuda_fail(st, e, "query routing: gather");
    // Priority tiles per row block, dealt over its column segments.
    const size_t prio_smem = 8 * (size_t)words_t;
    if ((e = set_smem_limit(ctx, (const void*)query_prio_kernel, (int)prio_smem)) != cudaSuccess)
        return cuda_fail(st, e, "query routing: priority tiles");
    query_prio_kernel<<<items, 256, prio_smem, s>>>(cell_of_pos, q, at.cell_start, (int)at.anchors, at.cell_nb,
                                                    col_tiles, prio, prio_cnt);
    split_lists_kernel<<<items, 256, 0, s>>>(prio, kQueryPrio, prio_cnt, csegs, (uint32_t*)(base + o_ps), ps,
                                             (uint32_t*)(base + o_psc));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "query routing: priority tiles");
    if ((e = sort_by_work(ctx, (uint32_t*)(base + o_psc), work, base + o_ws, (uint32_t*)(base + o_po))) != cudaSuccess)
        return cuda_fail(st, e, "query routing: work order");
    ctx->launches += 7;

    // The threshold pass over the priority tiles.
    KnnPlan plan;
    plan.nq = q;
    plan.nr = at.m;
    plan.d = d;
    plan.k = k;
    plan.self = false;
    plan.form = SCRUST_FORM_TENSOR;
    plan.precision = bf16 ? SCRUST_PRECISION_BF16 : SCRUST_PRECISION_FP16;
    Lists lists;
    lists.cap = 256;
    lists.ctot = 256 + 128;
    lists.segments = 2 * csegs;
    int32_t rc = alloc_lists(ctx, q_pad, &lists, st);
    if (rc) return rc;
    plan.cap = lists.cap;
    plan.ctot = lists.ctot;
    plan.segments = lists.segments;
    TileLists first;
    first.tiles = (const uint32_t*)(base + o_ps);
    first.count = (const uint32_t*)(base + o_psc);
    first.stride = ps;
    first.order = (const uint32_t*)(base + o_po);
    first.row_theta = row_theta;
    // A list the pass leaves without a threshold (a segment with no tile)
    // keeps a huge one; a row without any keeps reach everywhere.
    if ((e = cudaMemsetAsync(theta, 0x7f, 4 * 2 * (size_t)csegs * q_pad, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(row_theta, 0xff, 4 * (size_t)q_pad, s)) != cudaSuccess)
        return cuda_fail(st, e, "query knn: memset");
    if ((e = launch_tensor_candidates(ctx, plan, base + o_As, q_pad, at.B16, at.m_pad, bA, bdelta, beps2, lists, bf16,
                                      &first, false, theta, nullptr, nullptr, nullptr, kPassThresholds)) != cudaSuccess)
        return cuda_fail(st, e, "query knn: threshold pass");
    // The atlas tiles each row block cannot rule out: its segment balls
    // (reach from the rows' shared thresholds) against the atlas segment
    // balls.
    row_theta_pairs_kernel<<<(unsigned)((q + 255) / 256), 256, 0, s>>>(row_theta, q, theta2);
    if ((e = cudaMemsetAsync(qballs.nseg + items, 0, sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(bitmap, 0, 4 * (size_t)items * words_t, s)) != cudaSuccess)
        return cuda_fail(st, e, "query knn: memset");
    launch_tile_balls(bf16, base + o_As, q, d, items, cell_of_pos, theta2, bA, bdelta, qballs, s);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = device_exclusive_scan(ctx, qballs.nseg, seg_off, (int64_t)items + 1, (uint32_t*)(base + o_scan),
                                   scan_elems)) != cudaSuccess)
        return cuda_fail(st, e, "query knn: query balls");
    flatten_segments_kernel<<<items, 64, 0, s>>>(qballs, d, items, seg_off, (float*)(base + o_fc),
                                                 (float*)(base + o_fr), (float*)(base + o_fu),
                                                 (uint32_t*)(base + o_fo));
    cross_segment_pairs_kernel<<<(unsigned)std::min<int64_t>(smax, 8 * ctx->sm_count), 256, 0, s>>>(
        (const float*)(base + o_fc), (const float*)(base + o_fr), (const float*)(base + o_fu),
        (const uint32_t*)(base + o_fo), seg_off + items, at.seg_centre_t, at.seg_radius, at.seg_tile, at.segs, d,
        words_t, bitmap);
    const size_t lists_smem = 4 * (size_t)words_t;
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = set_smem_limit(ctx, (const void*)tile_lists_kernel, (int)lists_smem)) != cudaSuccess)
        return cuda_fail(st, e, "query knn: tile lists");
    tile_lists_kernel<<<items, 256, lists_smem, s>>>(bitmap, words_t, col_tiles, prio, prio_cnt, counts, entries,
                                                     kQueryPrio);
    split_lists_kernel<<<items, 256, 0, s>>>(entries, col_tiles, counts, csegs, (uint32_t*)(base + o_es), es,
                                             (uint32_t*)(base + o_esc));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "query knn: tile lists");
    ctx->launches += 7;
    // The thresholds tightened over the kept tiles too: a query's neighbours
    // spread over its cluster, so a block whose queries fall in many cells
    // leaves the first pass with loose thresholds, and collecting at those
    // would overflow the lists.
    TileLists second;
    second.tiles = (const uint32_t*)(base + o_es);
    second.count = (const uint32_t*)(base + o_esc);
    second.stride = es;
    second.row_theta = row_theta;
    if ((e = sort_by_work(ctx, (uint32_t*)(base + o_esc), work, base + o_ws, (uint32_t*)(base + o_po2))) != cudaSuccess)
        return cuda_fail(st, e, "query knn: work order");
    second.order = (const uint32_t*)(base + o_po2);
    if ((e = launch_tensor_candidates(ctx, plan, base + o_As, q_pad, at.B16, at.m_pad, bA, bdelta, beps2, lists, bf16,
                                      &second, true, theta, nullptr, nullptr, nullptr, kPassThresholds)) != cudaSuccess)
        return cuda_fail(st, e, "query knn: second threshold pass");
    // One collect pass over both lists, then the exact finish.
    TileLists both = first;
    both.tiles2 = second.tiles;
    both.count2 = second.count;
    both.stride2 = es;
    if ((e = launch_tensor_candidates(ctx, plan, base + o_As, q_pad, at.B16, at.m_pad, bA, bdelta, beps2, lists, bf16,
                                      &both, false, theta, nullptr, nullptr, nullptr, kPassCollect)) != cudaSuccess)
        return cuda_fail(st, e, "query knn: collect pass");
    RowBounds bounds;
    bounds.A = bA;
    bounds.delta = bdelta;
    bounds.eps2 = beps2;
    if ((e = launch_rerank(ctx, plan, dq, atlas_rows, nullptr, nullptr, nullptr, nullptr, dq, atlas_rows, bounds,
                           lists, at.perm, xs, theta, d_idx, d_dist, nullptr, nullptr, at.rows, P, true, qperm)) !=
        cudaSuccess)
        return cuda_fail(st, e, "query knn: rerank");
    ctx->launches += 3;
    return ok(st);
}

}  // namespace scrust
