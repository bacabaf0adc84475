// cluster.cu -- Leiden and Louvain community detection on the GPU, on the
// connectivities graph this library builds (crates/scrust-core/src/cluster.rs:88,125).
//
// The objective is the reference's RBConfiguration modularity
// Q = (1/2m) sum_ij (A_ij - gamma k_i k_j / 2m) [c_i = c_j] on the graph
// (A + A^T) / 2 (cluster.rs:214-290), and the structure is the reference's:
// local moving, then (Leiden) refinement of every community into
// well-connected subcommunities, aggregation, and repeat until nothing
// moves; Leiden restarts from its own result n_iterations times, stopping
// early when a pass changes nothing; labels are numbered by descending
// community size (cluster.rs:828-850).
//
// The reference moves one node at a time from a queue.  Here every pass is
// parallel and deterministic (the same graph and seed give the same labels):
//   - Local moving runs in rounds.  In each round half of the nodes (chosen
//     by a hash of node, seed and level, alternating) look at the
//     communities of their neighbours as the round began, and move to the
//     one of largest gain, ties to the smaller id, if that beats staying
//     (cluster.rs:425-455).  A node alone in its community joins another
//     lone node's community only when that id is smaller, so two lone
//     nodes never swap.  Rounds continue until two in a row move nothing.
//   - A block of 32 threads per node sums the node's edge weight per
//     neighbouring community in a shared-memory table, 32 neighbours at a
//     time, each community's partial in lane order, so every sum is formed
//     in one fixed order.
//   - Community strengths are fixed-point (int64, scale 2^s with
//     2m * 2^s <= 2^61) and change by integer atomics, whose result does not
//     depend on their order.
//   - Refinement: within each community, lone well-connected nodes merge
//     into a neighbouring subcommunity of non-negative gain that is well
//     connected to the rest of the community (cluster.rs:507-641), drawn with
//     probability proportional to exp((gain - max) / 0.01) by a counter-based
//     hash; a node moving in a round never joins a subcommunity whose own
//     lone node may move in that round.  Cuts are recomputed each round.
//   - Aggregation: entries keyed by (community, community) with two stable
//     radix sorts and per-key sums in sorted order.
// Nodes whose neighbours span more than 4096 communities do not move (the
// table's limit); on kNN graphs no node comes near it.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kSmallTable = 128;  // nodes with at most 64 neighbour entries, 4 warps a block
constexpr int kSmallWarps = 4;
constexpr int kBigTable = 2048;   // the rest, one warp a block
constexpr int kSmallDegree = 64;
constexpr int kMaxRounds = 200;
constexpr double kTheta = 0.01;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t mix_host(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ bool active_in(uint32_t v, int round, uint64_t salt) {
    return ((mix64(salt ^ (uint64_t)v) + (uint64_t)round) & 1ull) == 0ull;
}

// ---- the symmetric graph ----------------------------------------------------

__global__ void cl_rows_kernel(const uint32_t* __restrict__ indptr, int64_t n, uint32_t* __restrict__ erow) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (uint32_t e = indptr[r], e1 = indptr[r + 1]; e < e1; ++e) erow[e] = (uint32_t)r;
}

__global__ void cl_check_kernel(const float* __restrict__ values, int64_t nnz, int* __restrict__ bad) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        const float v = values[e];
        if (!(v >= 0.f) || isinf(v)) atomicExch(bad, 1);
    }
}

// Entry i < nnz is row(i) -> col(i), entry nnz + i the reverse; keyed by
// their first node.
__global__ void cl_sym_keys_kernel(const uint32_t* __restrict__ erow, const uint32_t* __restrict__ indices,
                                   int64_t nnz, uint32_t* __restrict__ keys, unsigned long long* __restrict__ vals) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * nnz) return;
    keys[i] = i < nnz ? erow[i] : indices[i - nnz];
    vals[i] = (unsigned long long)i;
}

// start[c] = number of sorted keys below c, c in [0, n].
__global__ void cl_starts_kernel(const uint32_t* __restrict__ keys, int64_t m, int64_t n, uint32_t* __restrict__ start) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p > m) return;
    const int64_t lo = p == 0 ? 0 : (int64_t)keys[p - 1] + 1;
    const int64_t hi = p == m ? n : (int64_t)keys[p];
    for (int64_t c = lo; c <= hi && c <= n; ++c) start[c] = (uint32_t)p;
}

__global__ void cl_sym_fill_kernel(const unsigned long long* __restrict__ order, int64_t m, int64_t nnz,
                                   const uint32_t* __restrict__ erow, const uint32_t* __restrict__ indices,
                                   const float* __restrict__ values, uint32_t* __restrict__ nb,
                                   double* __restrict__ w) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    const int64_t i = (int64_t)(order[p] & 0xffffffffull);
    const int64_t e = i < nnz ? i : i - nnz;
    nb[p] = i < nnz ? indices[e] : erow[e];
    w[p] = (double)values[e] / 2.0;
}

// Node strengths (row sums in row order).
__global__ void cl_strength_kernel(const uint32_t* __restrict__ ptr, const double* __restrict__ w, int64_t n,
                                   double* __restrict__ k) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    double s = 0.0;
    for (uint32_t p = ptr[v], p1 = ptr[v + 1]; p < p1; ++p) s += w[p];
    k[v] = s;
}

// Sum of `count` doubles in index order by one block, into out[0].
__global__ void cl_sum_kernel(const double* __restrict__ x, int64_t count, double* __restrict__ out) {
    __shared__ double part[256];
    double total = 0.0;
    for (int64_t base = 0; base < count; base += 256) {
        const int64_t i = base + threadIdx.x;
        part[threadIdx.x] = i < count ? x[i] : 0.0;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) total += part[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = total;
}

__global__ void cl_fix_kernel(const double* __restrict__ x, int64_t count, double scale, long long* __restrict__ fx) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) fx[i] = llrint(x[i] * scale);
}

// ---- community bookkeeping --------------------------------------------------

__global__ void cl_iota_kernel(int64_t n, uint32_t* __restrict__ out) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) out[v] = (uint32_t)v;
}

__global__ void cl_comm_init_kernel(const uint32_t* __restrict__ labels, const long long* __restrict__ kfix, int64_t n,
                                    long long* __restrict__ K, int* __restrict__ size) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    atomicAdd((unsigned long long*)(K + labels[v]), (unsigned long long)kfix[v]);
    atomicAdd(size + labels[v], 1);
}

// The per-node table of edge weight to each neighbouring community (or
// subcommunity), one warp per node: neighbours in chunks of 32; in a chunk
// each community's partial is summed by its lowest lane in lane order, then
// added to the table, so each entry is summed in one fixed order.  With
// `group_of`, only neighbours in the node's own group count.  Returns false
// when the table overflowed.
template <int T>
__device__ bool gather_table(const uint32_t* __restrict__ nb, const double* __restrict__ w, uint32_t p0, uint32_t p1,
                             uint32_t self, const uint32_t* __restrict__ label, const uint32_t* __restrict__ group_of,
                             uint32_t group, uint32_t* keys, double* vals, double* wbuf, int* overflow) {
    const int lane = threadIdx.x & 31;
    for (int t = lane; t < T; t += 32) keys[t] = kEmpty;
    if (lane == 0) *overflow = 0;
    __syncwarp();
    for (uint32_t base = p0; base < p1; base += 32) {
        const uint32_t p = base + lane;
        uint32_t c = kEmpty;
        double wt = 0.0;
        if (p < p1) {
            const uint32_t u = nb[p];
            if (u != self && (!group_of || group_of[u] == group)) {
                c = label[u];
                wt = w[p];
            }
        }
        wbuf[lane] = wt;
        __syncwarp();
        const uint32_t peers = __match_any_sync(0xffffffffu, c);
        if (c != kEmpty && (__ffs(peers) - 1) == lane) {
            double s = 0.0;
            for (uint32_t b = peers; b; b &= b - 1) s += wbuf[__ffs(b) - 1];
            uint32_t slot = (uint32_t)(mix64(c) & (T - 1));
            bool placed = false;
            for (int probe = 0; probe < T; ++probe) {
                const uint32_t prev = atomicCAS(keys + slot, kEmpty, c);
                if (prev == kEmpty || prev == c) {
                    if (prev == kEmpty) vals[slot] = 0.0;
                    vals[slot] += s;
                    placed = true;
                    break;
                }
                slot = (slot + 1) & (T - 1);
            }
            if (!placed) *overflow = 1;
        }
        __syncwarp();
    }
    return *overflow == 0;
}

// Local moving, one round, one warp per node: the nodes of this round's half
// each take the neighbouring community of largest gain (ties to the smaller
// id) when it beats staying (cluster.rs:420-455).  A node whose best gain,
// staying included, is negative goes alone to its reserved id n + v, when
// that community is empty.  Community ids are below 2n.
template <int T, int W>
__global__ void __launch_bounds__(32 * W) cl_move_kernel(const uint32_t* __restrict__ ptr,
                                                         const uint32_t* __restrict__ nb,
                                                         const double* __restrict__ w,
                                                         const long long* __restrict__ kfix,
                                                         const uint32_t* __restrict__ nodes, int64_t count,
                                                         int64_t n_level, const uint32_t* __restrict__ comm,
                                                         const long long* __restrict__ K,
                                                         const int* __restrict__ size, double inv_scale, double res,
                                                         double total, int round, uint64_t salt,
                                                         uint32_t* __restrict__ next,
                                                         unsigned int* __restrict__ moves) {
    __shared__ uint32_t keys[W][T];
    __shared__ double vals[W][T];
    __shared__ double wbuf[W][32];
    __shared__ int overflow[W];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t idx = (int64_t)blockIdx.x * W + warp;
    if (idx >= count) return;
    const uint32_t v = nodes[idx];
    if (!active_in(v, round, salt)) return;
    const uint32_t own = comm[v];
    if (!gather_table<T>(nb, w, ptr[v], ptr[v + 1], v, comm, nullptr, 0, keys[warp], vals[warp], wbuf[warp],
                         &overflow[warp]))
        return;
    const double kv = (double)kfix[v] * inv_scale;
    double e_own = 0.0;
    double best = -INFINITY;
    uint32_t best_c = kEmpty;
    const bool alone = size[own] == 1;
    for (int t = lane; t < T; t += 32) {
        const uint32_t c = keys[warp][t];
        if (c == kEmpty) continue;
        if (c == own) {
            e_own = vals[warp][t];
            continue;
        }
        if (alone && size[c] == 1 && c > own) continue;  // lone nodes only join smaller lone ids
        const double g = vals[warp][t] - res * ((double)K[c] * inv_scale) * kv / total;
        if (g > best || (g == best && c < best_c)) {
            best = g;
            best_c = c;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const uint32_t oc = __shfl_xor_sync(0xffffffffu, best_c, o);
        e_own += __shfl_xor_sync(0xffffffffu, e_own, o);  // one lane holds it, the rest hold 0
        if (ob > best || (ob == best && oc < best_c)) {
            best = ob;
            best_c = oc;
        }
    }
    if (lane != 0) return;
    const double stay = e_own - res * ((double)(K[own] - kfix[v]) * inv_scale) * kv / total;
    uint32_t to = own;
    if (best_c != kEmpty && best > stay) to = best_c;
    const double top = to == own ? stay : best;
    const uint32_t fresh = (uint32_t)(n_level + v);
    if (top < 0.0 && own != fresh && size[fresh] == 0) to = fresh;
    if (to != own) {
        next[v] = to;
        atomicAdd(moves, 1u);
    }
}

__global__ void cl_apply_kernel(int64_t n, const long long* __restrict__ kfix, uint32_t* __restrict__ comm,
                                const uint32_t* __restrict__ next, long long* __restrict__ K, int* __restrict__ size) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t a = comm[v], b = next[v];
    if (a == b) return;
    atomicAdd((unsigned long long*)(K + a), (unsigned long long)(-kfix[v]));
    atomicAdd((unsigned long long*)(K + b), (unsigned long long)kfix[v]);
    atomicSub(size + a, 1);
    atomicAdd(size + b, 1);
    comm[v] = b;
}

// ---- refinement -------------------------------------------------------------

// Per node: its weight to the rest of its community (fixed order), and
// whether it is well connected to it (cluster.rs:507-515).
__global__ void cl_to_subset_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ nb,
                                    const double* __restrict__ w, const double* __restrict__ k, int64_t n,
                                    const uint32_t* __restrict__ part, const long long* __restrict__ K,
                                    double inv_scale, double res, double total, double* __restrict__ to_subset,
                                    unsigned char* __restrict__ well) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t c = part[v];
    double s = 0.0;
    for (uint32_t p = ptr[v], p1 = ptr[v + 1]; p < p1; ++p) {
        const uint32_t u = nb[p];
        if (u != (uint32_t)v && part[u] == c) s += w[p];
    }
    to_subset[v] = s;
    const double kc = (double)K[c] * inv_scale;
    well[v] = s >= res * k[v] * (kc - k[v]) / total;
}

// Per subcommunity, its cut to the rest of its community:
// sum over members of (to_subset - weight to the subcommunity), fixed point.
__global__ void cl_cut_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ nb,
                              const double* __restrict__ w, int64_t n, const uint32_t* __restrict__ sub,
                              const double* __restrict__ to_subset, double scale, long long* __restrict__ cut) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t s = sub[v];
    double inside = 0.0;
    for (uint32_t p = ptr[v], p1 = ptr[v + 1]; p < p1; ++p) {
        const uint32_t u = nb[p];
        if (u != (uint32_t)v && sub[u] == s) inside += w[p];
    }
    atomicAdd((unsigned long long*)(cut + s), (unsigned long long)llrint((to_subset[v] - inside) * scale));
}

// Refinement, one round, one warp per node (cluster.rs:560-641): a lone,
// well-connected node of this round's half merges into a subcommunity of
// its community with non-negative gain whose cut to the rest of the
// community passes the well-connectedness test, drawn with probability
// proportional to exp(gain / 0.01) by the Gumbel-max rule (the largest
// gain / 0.01 + G, G a Gumbel variate from a hash of seed, node,
// subcommunity and round).  A lone node that may itself move in this round
// is not a target.
template <int T, int W>
__global__ void __launch_bounds__(32 * W) cl_refine_kernel(const uint32_t* __restrict__ ptr,
                                                           const uint32_t* __restrict__ nb,
                                                           const double* __restrict__ w,
                                                           const long long* __restrict__ kfix,
                                                           const uint32_t* __restrict__ nodes, int64_t count,
                                                           const uint32_t* __restrict__ part,
                                                           const uint32_t* __restrict__ sub,
                                                           const long long* __restrict__ Ksub,
                                                           const int* __restrict__ subsize,
                                                           const long long* __restrict__ K,
                                                           const long long* __restrict__ cut,
                                                           const unsigned char* __restrict__ well, double inv_scale,
                                                           double res, double total, int round, uint64_t salt,
                                                           uint32_t* __restrict__ next,
                                                           unsigned int* __restrict__ moves) {
    __shared__ uint32_t keys[W][T];
    __shared__ double vals[W][T];
    __shared__ double wbuf[W][32];
    __shared__ int overflow[W];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t idx = (int64_t)blockIdx.x * W + warp;
    if (idx >= count) return;
    const uint32_t v = nodes[idx];
    if (sub[v] != v || subsize[v] != 1 || !well[v] || !active_in(v, round, salt)) return;
    const uint32_t c = part[v];
    if (!gather_table<T>(nb, w, ptr[v], ptr[v + 1], v, sub, part, c, keys[warp], vals[warp], wbuf[warp],
                         &overflow[warp]))
        return;
    const double kv = (double)kfix[v] * inv_scale;
    const double kc = (double)K[c] * inv_scale;
    double best = -INFINITY;
    uint32_t best_s = kEmpty;
    for (int t = lane; t < T; t += 32) {
        const uint32_t s = keys[warp][t];
        if (s == kEmpty) continue;
        const double ks = (double)Ksub[s] * inv_scale;
        const double gain = vals[warp][t] - res * ks * kv / total;
        const bool frozen = !(subsize[s] == 1 && well[s] && active_in(s, round, salt));
        if (!(gain >= 0.0 && frozen && (double)cut[s] * inv_scale >= res * ks * (kc - ks) / total)) continue;
        const uint64_t h = mix64(salt ^ mix64(((uint64_t)v << 32 | s) ^ mix64((uint64_t)round + 0x51ed27ull)));
        const double u = ((double)(h >> 11) + 0.5) * 1.1102230246251565e-16;
        const double key = gain / kTheta - log(-log(u));
        if (key > best || (key == best && s < best_s)) {
            best = key;
            best_s = s;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const uint32_t os = __shfl_xor_sync(0xffffffffu, best_s, o);
        if (ob > best || (ob == best && os < best_s)) {
            best = ob;
            best_s = os;
        }
    }
    if (lane == 0 && best_s != kEmpty) {
        next[v] = best_s;
        atomicAdd(moves, 1u);
    }
}

// ---- aggregation ------------------------------------------------------------

__global__ void cl_flag_kernel(const uint32_t* __restrict__ labels, int64_t n, uint32_t* __restrict__ flag) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) flag[labels[v]] = 1u;
}

__global__ void cl_relabel_kernel(const uint32_t* __restrict__ in, int64_t n, const uint32_t* __restrict__ id,
                                  uint32_t* __restrict__ out) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) out[v] = id[in[v]];
}

__global__ void cl_agg_keys_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ nb, int64_t n,
                                   const uint32_t* __restrict__ lab, uint32_t* __restrict__ krow,
                                   uint32_t* __restrict__ kcol) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    for (uint32_t p = ptr[v], p1 = ptr[v + 1]; p < p1; ++p) {
        krow[p] = lab[v];
        kcol[p] = lab[nb[p]];
    }
}

__global__ void cl_seq_kernel(int64_t m, unsigned long long* __restrict__ vals) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < m) vals[p] = (unsigned long long)p;
}

// kA[p] = kcol[order[p]] for the second (stable) sort, by row.
__global__ void cl_gather_u32_kernel(const uint32_t* __restrict__ src, const unsigned long long* __restrict__ order,
                                     int64_t m, uint32_t* __restrict__ dst) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < m) dst[p] = src[order[p] & 0xffffffffull];
}

// Segment heads of the sorted (row, col) keys.
__global__ void cl_heads_kernel(const unsigned long long* __restrict__ order, const uint32_t* __restrict__ krow,
                                const uint32_t* __restrict__ kcol, int64_t m, uint32_t* __restrict__ head) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m) return;
    const int64_t e = (int64_t)(order[p] & 0xffffffffull);
    if (p == 0) {
        head[p] = 1u;
        return;
    }
    const int64_t f = (int64_t)(order[p - 1] & 0xffffffffull);
    head[p] = (krow[e] != krow[f] || kcol[e] != kcol[f]) ? 1u : 0u;
}

// One thread per coarse entry: its weight summed over its run in sorted order.
__global__ void cl_segsum_kernel(const unsigned long long* __restrict__ order, const uint32_t* __restrict__ head,
                                 const uint32_t* __restrict__ pos, const uint32_t* __restrict__ krow,
                                 const uint32_t* __restrict__ kcol, const double* __restrict__ w, int64_t m,
                                 uint32_t* __restrict__ out_row, uint32_t* __restrict__ out_nb,
                                 double* __restrict__ out_w) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m || !head[p]) return;
    const int64_t e0 = (int64_t)(order[p] & 0xffffffffull);
    double s = 0.0;
    for (int64_t q = p; q < m && (q == p || !head[q]); ++q) s += w[order[q] & 0xffffffffull];
    const uint32_t id = pos[p];
    out_row[id] = krow[e0];
    out_nb[id] = kcol[e0];
    out_w[id] = s;
}

// ---- scoring and output -----------------------------------------------------

__global__ void cl_score_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ nb,
                                const double* __restrict__ w, const long long* __restrict__ kfix, int64_t n,
                                const uint32_t* __restrict__ lab, double scale, long long* __restrict__ internal,
                                long long* __restrict__ strength) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint32_t c = lab[v];
    double s = 0.0;
    for (uint32_t p = ptr[v], p1 = ptr[v + 1]; p < p1; ++p)
        if (lab[nb[p]] == c) s += w[p];
    atomicAdd((unsigned long long*)(internal + c), (unsigned long long)llrint(s * scale));
    atomicAdd((unsigned long long*)(strength + c), (unsigned long long)kfix[v]);
}

__global__ void cl_q_kernel(const long long* __restrict__ internal, const long long* __restrict__ strength, int64_t nc,
                            double inv_scale, double res, double total, double* __restrict__ out) {
    __shared__ double part[256];
    double q = 0.0;
    for (int64_t base = 0; base < nc; base += 256) {
        const int64_t c = base + threadIdx.x;
        double t = 0.0;
        if (c < nc) {
            const double in = (double)internal[c] * inv_scale, st = (double)strength[c] * inv_scale;
            t = in / total - res * (st / total) * (st / total);
        }
        part[threadIdx.x] = t;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) q += part[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = q;
}

__global__ void cl_differ_kernel(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, int64_t n,
                                 unsigned int* __restrict__ differ) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n && a[v] != b[v]) *differ = 1u;
}

__global__ void cl_size_keys_kernel(const int* __restrict__ size, int64_t nc, uint32_t* __restrict__ keys,
                                    unsigned long long* __restrict__ vals) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    keys[c] = 0xffffffffu - (uint32_t)size[c];
    vals[c] = (unsigned long long)c;
}

__global__ void cl_rank_kernel(const unsigned long long* __restrict__ order, int64_t nc, uint32_t* __restrict__ rank) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nc) rank[order[i] & 0xffffffffull] = (uint32_t)i;
}

__global__ void cl_small_big_kernel(const uint32_t* __restrict__ ptr, int64_t n, uint32_t* __restrict__ small,
                                    uint32_t* __restrict__ big, unsigned int* __restrict__ counts) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    if (ptr[v + 1] - ptr[v] <= (uint32_t)kSmallDegree)
        small[atomicAdd(counts, 1u)] = (uint32_t)v;
    else
        big[atomicAdd(counts + 1, 1u)] = (uint32_t)v;
}

__global__ void cl_scatter_kernel(const uint32_t* __restrict__ collapse, const uint32_t* __restrict__ partition,
                                  int64_t n, uint32_t* __restrict__ out) {
    // Every member of a subcommunity lies in the same community, so the
    // writes to one slot agree.
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) out[collapse[v]] = partition[v];
}

struct Level {
    int64_t n = 0, m = 0;
    uint32_t* ptr = nullptr;
    uint32_t* nb = nullptr;
    double* w = nullptr;
    double* k = nullptr;
    long long* kfix = nullptr;
};

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + 255) / 256); }

}  // namespace

// The whole algorithm on device buffers, under the context lock.  Buffers
// are allocated per call and released when the object goes.
class Clusterer {
public:
    Clusterer(scrust_context* ctx, scrust_status* st) : ctx_(ctx), st_(st), s_(ctx->stream) {}
    ~Clusterer() {
        cudaStreamSynchronize(s_);
        for (void* p : owned_) cudaFree(p);
    }

    template <class T>
    T* alloc(size_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            ok_ = false;
            return nullptr;
        }
        owned_.push_back(p);
        return (T*)p;
    }

    int32_t build(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n, int64_t nnz);
    int32_t run(bool leiden, double res, int n_iterations, uint64_t seed, uint32_t* out_labels, double* out_q,
                uint64_t* out_nc);
    int32_t score_only(const uint32_t* labels, int64_t nc, double res, double* out_q);

private:
    int32_t oom() { return fail(st_, SCRUST_OOM, "clustering: device allocation failed"); }
    template <class V>
    bool download(V* host, const V* dev, size_t count) {
        if (cudaMemcpyAsync(host, dev, sizeof(V) * count, cudaMemcpyDeviceToHost, s_) != cudaSuccess ||
            cudaStreamSynchronize(s_) != cudaSuccess) {
            cudaGetLastError();
            ok_ = false;
        }
        return ok_;
    }
    cudaError_t sort_pairs(uint32_t* kA, unsigned long long* vA, uint32_t* kB, unsigned long long* vB, int64_t m,
                           int bits, uint32_t** kout, unsigned long long** vout);
    int64_t compact(const uint32_t* labels, int64_t n, int64_t width, uint32_t* out);
    int32_t node_lists(const Level& L);
    int32_t local_moving(const Level& L, uint32_t* comm, long long* K, int* size, double res, uint64_t salt,
                         bool* moved_any);
    int32_t refine(const Level& L, const uint32_t* part, const long long* K, double res, uint64_t salt,
                   uint32_t* sub);
    int32_t aggregate(const Level& L, const uint32_t* lab, int64_t nc, Level* out);
    int32_t optimise(const uint32_t* initial, double res, bool leiden, uint64_t salt, uint32_t* out,
                     int64_t* out_nc);
    double score(const Level& L, const uint32_t* lab, int64_t nc, double res);

    scrust_context* ctx_;
    scrust_status* st_;
    cudaStream_t s_;
    bool ok_ = true;
    std::vector<void*> owned_;
    Level g0_;
    double total_ = 0.0, scale_ = 1.0, inv_scale_ = 1.0;
    unsigned int* counter_ = nullptr;
    // node lists of the current level: small-degree nodes, then the rest
    uint32_t* small_ = nullptr;
    uint32_t* big_ = nullptr;
    int64_t n_small_ = 0, n_big_ = 0;
};

cudaError_t Clusterer::sort_pairs(uint32_t* kA, unsigned long long* vA, uint32_t* kB, unsigned long long* vB,
                                  int64_t m, int bits, uint32_t** kout, unsigned long long** vout) {
    const int nb = radix_blocks(std::max<int64_t>(m, 1));
    const size_t scan_elems = scan_scratch_elems((int64_t)256 * nb);
    uint32_t* hist = alloc<uint32_t>((size_t)256 * nb + 16);
    uint32_t* scan = alloc<uint32_t>(scan_elems);
    if (!ok_) return cudaErrorMemoryAllocation;
    return radix_sort_pairs(ctx_, kA, vA, kB, vB, m, bits, hist, scan, scan_elems, kout, vout);
}

// Ids in use (below `width`) renumbered 0.. in ascending order (cluster.rs:807-826).
int64_t Clusterer::compact(const uint32_t* labels, int64_t n, int64_t width, uint32_t* out) {
    uint32_t* flag = alloc<uint32_t>((size_t)width + 1);
    uint32_t* scan = alloc<uint32_t>(scan_scratch_elems(width + 1));
    if (!ok_) return -1;
    cudaMemsetAsync(flag, 0, sizeof(uint32_t) * ((size_t)width + 1), s_);
    cl_flag_kernel<<<grid_for(n), 256, 0, s_>>>(labels, n, flag);
    if (device_exclusive_scan(ctx_, flag, flag, width + 1, scan, scan_scratch_elems(width + 1)) != cudaSuccess) {
        ok_ = false;
        return -1;
    }
    cl_relabel_kernel<<<grid_for(n), 256, 0, s_>>>(labels, n, flag, out);
    ctx_->launches += 2;
    uint32_t nc = 0;
    if (!download(&nc, flag + width, 1)) return -1;
    return (int64_t)nc;
}

int32_t Clusterer::build(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n,
                         int64_t nnz) {
    if (nnz == 0)
        return fail(st_, SCRUST_INVALID_PARAMETER, "the graph needs at least one edge of positive weight");
    int* bad = alloc<int>(1);
    uint32_t* erow = alloc<uint32_t>(nnz);
    const int64_t m = 2 * nnz;
    uint32_t* kA = alloc<uint32_t>(m);
    uint32_t* kB = alloc<uint32_t>(m);
    unsigned long long* vA = alloc<unsigned long long>(m);
    unsigned long long* vB = alloc<unsigned long long>(m);
    g0_.n = n;
    g0_.m = m;
    g0_.ptr = alloc<uint32_t>(n + 1);
    g0_.nb = alloc<uint32_t>(m);
    g0_.w = alloc<double>(m);
    g0_.k = alloc<double>(n);
    g0_.kfix = alloc<long long>(n);
    double* tot = alloc<double>(1);
    counter_ = alloc<unsigned int>(4);
    if (!ok_) return oom();
    cudaMemsetAsync(bad, 0, sizeof(int), s_);
    cl_check_kernel<<<(unsigned)std::min<int64_t>(1024, nnz / 256 + 1), 256, 0, s_>>>(values, nnz, bad);
    int hbad = 0;
    if (!download(&hbad, bad, 1)) return fail(st_, SCRUST_KERNEL, "clustering: graph check");
    if (hbad) return fail(st_, SCRUST_INVALID_PARAMETER, "graph weights must be finite and non-negative");
    cl_rows_kernel<<<grid_for(n), 256, 0, s_>>>(indptr, n, erow);
    cl_sym_keys_kernel<<<grid_for(m), 256, 0, s_>>>(erow, indices, nnz, kA, vA);
    int bits = 1;
    while (((int64_t)1 << bits) <= n) bits++;
    uint32_t* keys = nullptr;
    unsigned long long* order = nullptr;
    cudaError_t e;
    if ((e = sort_pairs(kA, vA, kB, vB, m, bits, &keys, &order)) != cudaSuccess)
        return cuda_fail(st_, e, "clustering: graph");
    cl_starts_kernel<<<grid_for(m + 1), 256, 0, s_>>>(keys, m, n, g0_.ptr);
    cl_sym_fill_kernel<<<grid_for(m), 256, 0, s_>>>(order, m, nnz, erow, indices, values, g0_.nb, g0_.w);
    cl_strength_kernel<<<grid_for(n), 256, 0, s_>>>(g0_.ptr, g0_.w, n, g0_.k);
    cl_sum_kernel<<<1, 256, 0, s_>>>(g0_.k, n, tot);
    ctx_->launches += 7;
    if (!download(&total_, tot, 1)) return fail(st_, SCRUST_KERNEL, "clustering: graph");
    if (!(total_ > 0.0))
        return fail(st_, SCRUST_INVALID_PARAMETER, "the graph needs at least one edge of positive weight");
    // Fixed point for strengths: the total at 2^61 leaves room for the
    // rounding of up to 2^31 terms below 2^63.
    const int sexp = (int)std::floor(61.0 - std::log2(total_));
    scale_ = std::ldexp(1.0, sexp);
    inv_scale_ = std::ldexp(1.0, -sexp);
    cl_fix_kernel<<<grid_for(n), 256, 0, s_>>>(g0_.k, n, scale_, g0_.kfix);
    ctx_->launches += 1;
    return ok(st_);
}

int32_t Clusterer::node_lists(const Level& L) {
    small_ = alloc<uint32_t>(L.n);
    big_ = alloc<uint32_t>(L.n);
    if (!ok_) return oom();
    cudaMemsetAsync(counter_, 0, 2 * sizeof(unsigned int), s_);
    cl_small_big_kernel<<<grid_for(L.n), 256, 0, s_>>>(L.ptr, L.n, small_, big_, counter_);
    ctx_->launches += 1;
    unsigned int counts[2] = {0, 0};
    if (!download(counts, counter_, 2)) return fail(st_, SCRUST_KERNEL, "clustering: node lists");
    n_small_ = counts[0];
    n_big_ = counts[1];
    return ok(st_);
}

int32_t Clusterer::local_moving(const Level& L, uint32_t* comm, long long* K, int* size, double res, uint64_t salt,
                                bool* moved_any) {
    uint32_t* next = alloc<uint32_t>(L.n);
    if (!ok_) return oom();
    *moved_any = false;
    int quiet = 0;
    for (int round = 0; round < kMaxRounds && quiet < 2; ++round) {
        cudaMemcpyAsync(next, comm, sizeof(uint32_t) * L.n, cudaMemcpyDeviceToDevice, s_);
        cudaMemsetAsync(counter_ + 2, 0, sizeof(unsigned int), s_);
        if (n_small_)
            cl_move_kernel<kSmallTable, kSmallWarps>
                <<<(unsigned)((n_small_ + kSmallWarps - 1) / kSmallWarps), 32 * kSmallWarps, 0, s_>>>(
                    L.ptr, L.nb, L.w, L.kfix, small_, n_small_, L.n, comm, K, size, inv_scale_, res, total_, round,
                    salt, next, counter_ + 2);
        if (n_big_)
            cl_move_kernel<kBigTable, 1><<<(unsigned)n_big_, 32, 0, s_>>>(L.ptr, L.nb, L.w, L.kfix, big_, n_big_,
                                                                          L.n, comm, K, size, inv_scale_, res,
                                                                          total_, round, salt, next, counter_ + 2);
        cl_apply_kernel<<<grid_for(L.n), 256, 0, s_>>>(L.n, L.kfix, comm, next, K, size);
        ctx_->launches += 3;
        unsigned int moves = 0;
        if (!download(&moves, counter_ + 2, 1)) return fail(st_, SCRUST_KERNEL, "clustering: local moving");
        if (moves) {
            *moved_any = true;
            quiet = 0;
        } else {
            ++quiet;
        }
    }
    return ok(st_);
}

int32_t Clusterer::refine(const Level& L, const uint32_t* part, const long long* K, double res, uint64_t salt,
                          uint32_t* sub) {
    const int64_t n = L.n;
    double* to_subset = alloc<double>(n);
    unsigned char* well = alloc<unsigned char>(n);
    long long* Ksub = alloc<long long>(n);
    int* subsize = alloc<int>(n);
    long long* cut = alloc<long long>(n);
    uint32_t* next = alloc<uint32_t>(n);
    if (!ok_) return oom();
    const unsigned nb = grid_for(n);
    cl_to_subset_kernel<<<nb, 256, 0, s_>>>(L.ptr, L.nb, L.w, L.k, n, part, K, inv_scale_, res, total_, to_subset,
                                           well);
    cl_iota_kernel<<<nb, 256, 0, s_>>>(n, sub);
    cudaMemcpyAsync(Ksub, L.kfix, sizeof(long long) * n, cudaMemcpyDeviceToDevice, s_);
    ctx_->launches += 2;
    {
        std::vector<int> ones((size_t)n, 1);
        cudaMemcpyAsync(subsize, ones.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s_);
        cudaStreamSynchronize(s_);
    }
    int quiet = 0;
    for (int round = 0; round < kMaxRounds && quiet < 2; ++round) {
        cudaMemsetAsync(cut, 0, sizeof(long long) * n, s_);
        cl_cut_kernel<<<nb, 256, 0, s_>>>(L.ptr, L.nb, L.w, n, sub, to_subset, scale_, cut);
        cudaMemcpyAsync(next, sub, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s_);
        cudaMemsetAsync(counter_ + 2, 0, sizeof(unsigned int), s_);
        if (n_small_)
            cl_refine_kernel<kSmallTable, kSmallWarps>
                <<<(unsigned)((n_small_ + kSmallWarps - 1) / kSmallWarps), 32 * kSmallWarps, 0, s_>>>(
                    L.ptr, L.nb, L.w, L.kfix, small_, n_small_, part, sub, Ksub, subsize, K, cut, well, inv_scale_,
                    res, total_, round, salt, next, counter_ + 2);
        if (n_big_)
            cl_refine_kernel<kBigTable, 1><<<(unsigned)n_big_, 32, 0, s_>>>(
                L.ptr, L.nb, L.w, L.kfix, big_, n_big_, part, sub, Ksub, subsize, K, cut, well, inv_scale_, res,
                total_, round, salt, next, counter_ + 2);
        cl_apply_kernel<<<nb, 256, 0, s_>>>(n, L.kfix, sub, next, Ksub, subsize);
        ctx_->launches += 4;
        unsigned int moves = 0;
        if (!download(&moves, counter_ + 2, 1)) return fail(st_, SCRUST_KERNEL, "clustering: refinement");
        quiet = moves ? 0 : quiet + 1;
    }
    return ok(st_);
}

// The graph of communities (cluster.rs:681-730): entries keyed by
// (community of row, community of neighbour) in ascending order, weights
// summed per key in the order of the finer graph's entries.
int32_t Clusterer::aggregate(const Level& L, const uint32_t* lab, int64_t nc, Level* out) {
    const int64_t m = L.m;
    uint32_t* krow = alloc<uint32_t>(m);
    uint32_t* kcol = alloc<uint32_t>(m);
    uint32_t* kA = alloc<uint32_t>(m);
    uint32_t* kB = alloc<uint32_t>(m);
    unsigned long long* vA = alloc<unsigned long long>(m);
    unsigned long long* vB = alloc<unsigned long long>(m);
    uint32_t* head = alloc<uint32_t>(m + 1);
    uint32_t* pos = alloc<uint32_t>(m + 1);
    uint32_t* scan = alloc<uint32_t>(scan_scratch_elems(m + 1));
    uint32_t* orow = alloc<uint32_t>(m);
    if (!ok_) return oom();
    const unsigned eb = grid_for(m);
    cl_agg_keys_kernel<<<grid_for(L.n), 256, 0, s_>>>(L.ptr, L.nb, L.n, lab, krow, kcol);
    cl_seq_kernel<<<eb, 256, 0, s_>>>(m, vA);
    cudaMemcpyAsync(kA, kcol, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s_);
    ctx_->launches += 2;
    int bits = 1;
    while (((int64_t)1 << bits) <= nc) bits++;
    uint32_t* keys = nullptr;
    unsigned long long* order = nullptr;
    cudaError_t e;
    if ((e = sort_pairs(kA, vA, kB, vB, m, bits, &keys, &order)) != cudaSuccess)
        return cuda_fail(st_, e, "clustering: aggregate");
    // Then a stable pass by row.
    unsigned long long* o2 = order == vA ? vB : vA;
    uint32_t* k2 = keys == kA ? kB : kA;
    cl_gather_u32_kernel<<<eb, 256, 0, s_>>>(krow, order, m, k2);
    ctx_->launches += 1;
    if ((e = sort_pairs(k2, order, keys, o2, m, bits, &keys, &order)) != cudaSuccess)
        return cuda_fail(st_, e, "clustering: aggregate");
    cl_heads_kernel<<<eb, 256, 0, s_>>>(order, krow, kcol, m, head);
    cudaMemsetAsync(head + m, 0, sizeof(uint32_t), s_);
    if ((e = device_exclusive_scan(ctx_, head, pos, m + 1, scan, scan_scratch_elems(m + 1))) != cudaSuccess)
        return cuda_fail(st_, e, "clustering: aggregate");
    ctx_->launches += 1;
    uint32_t mo = 0;
    if (!download(&mo, pos + m, 1)) return fail(st_, SCRUST_KERNEL, "clustering: aggregate");
    out->n = nc;
    out->m = mo;
    out->ptr = alloc<uint32_t>(nc + 1);
    out->nb = alloc<uint32_t>(mo);
    out->w = alloc<double>(mo);
    out->k = alloc<double>(nc);
    out->kfix = alloc<long long>(nc);
    if (!ok_) return oom();
    cl_segsum_kernel<<<eb, 256, 0, s_>>>(order, head, pos, krow, kcol, L.w, m, orow, out->nb, out->w);
    cl_starts_kernel<<<grid_for(mo + 1), 256, 0, s_>>>(orow, mo, nc, out->ptr);
    cl_strength_kernel<<<grid_for(nc), 256, 0, s_>>>(out->ptr, out->w, nc, out->k);
    cl_fix_kernel<<<grid_for(nc), 256, 0, s_>>>(out->k, nc, scale_, out->kfix);
    ctx_->launches += 4;
    return ok(st_);
}

double Clusterer::score(const Level& L, const uint32_t* lab, int64_t nc, double res) {
    long long* internal = alloc<long long>(nc);
    long long* strength = alloc<long long>(nc);
    double* q = alloc<double>(1);
    if (!ok_) return NAN;
    cudaMemsetAsync(internal, 0, sizeof(long long) * nc, s_);
    cudaMemsetAsync(strength, 0, sizeof(long long) * nc, s_);
    cl_score_kernel<<<grid_for(L.n), 256, 0, s_>>>(L.ptr, L.nb, L.w, L.kfix, L.n, lab, scale_, internal, strength);
    cl_q_kernel<<<1, 256, 0, s_>>>(internal, strength, nc, inv_scale_, res, total_, q);
    ctx_->launches += 2;
    double h = NAN;
    download(&h, q, 1);
    return h;
}

// One pass (cluster.rs:732-784) from `initial` labels of the nodes; writes
// the nodes' labels, compacted, and their count.
int32_t Clusterer::optimise(const uint32_t* initial, double res, bool leiden, uint64_t salt, uint32_t* out,
                            int64_t* out_nc) {
    Level level = g0_;
    const int64_t n0 = g0_.n;
    uint32_t* fold = alloc<uint32_t>(n0);
    uint32_t* labels = alloc<uint32_t>(n0);
    if (!ok_) return oom();
    cl_iota_kernel<<<grid_for(n0), 256, 0, s_>>>(n0, fold);
    cudaMemcpyAsync(labels, initial, sizeof(uint32_t) * n0, cudaMemcpyDeviceToDevice, s_);
    ctx_->launches += 1;
    for (int depth = 0; depth < 64; ++depth) {
        const int64_t n = level.n;
        // Community ids below 2n: the labels in use, and n + v reserved for v.
        long long* K = alloc<long long>(2 * n);
        int* size = alloc<int>(2 * n);
        uint32_t* partition = alloc<uint32_t>(n);
        if (!ok_) return oom();
        cudaMemsetAsync(K, 0, sizeof(long long) * 2 * n, s_);
        cudaMemsetAsync(size, 0, sizeof(int) * 2 * n, s_);
        cl_comm_init_kernel<<<grid_for(n), 256, 0, s_>>>(labels, level.kfix, n, K, size);
        ctx_->launches += 1;
        const uint64_t level_salt = mix_host(salt ^ ((uint64_t)depth * 0xD1B54A32D192ED03ull));
        int32_t rc = node_lists(level);
        if (rc) return rc;
        bool moved = false;
        if ((rc = local_moving(level, labels, K, size, res, level_salt, &moved))) return rc;
        const int64_t nc = compact(labels, n, 2 * n, partition);
        if (nc < 0) return fail(st_, SCRUST_KERNEL, "clustering: compact");
        if (!moved || nc == n) {
            cl_relabel_kernel<<<grid_for(n0), 256, 0, s_>>>(fold, n0, partition, out);
            ctx_->launches += 1;
            *out_nc = nc;
            return ok(st_);
        }
        uint32_t* collapse = alloc<uint32_t>(n);
        if (!ok_) return oom();
        int64_t ncol = nc;
        if (leiden) {
            long long* Kp = alloc<long long>(nc);
            int* sp = alloc<int>(nc);
            uint32_t* sub = alloc<uint32_t>(n);
            if (!ok_) return oom();
            cudaMemsetAsync(Kp, 0, sizeof(long long) * nc, s_);
            cudaMemsetAsync(sp, 0, sizeof(int) * nc, s_);
            cl_comm_init_kernel<<<grid_for(n), 256, 0, s_>>>(partition, level.kfix, n, Kp, sp);
            ctx_->launches += 1;
            if ((rc = refine(level, partition, Kp, res, mix_host(level_salt ^ 0x5bd1e995ull), sub))) return rc;
            ncol = compact(sub, n, n, collapse);
            if (ncol < 0) return fail(st_, SCRUST_KERNEL, "clustering: compact");
        } else {
            cudaMemcpyAsync(collapse, partition, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s_);
        }
        Level next;
        if ((rc = aggregate(level, collapse, ncol, &next))) return rc;
        // The coarser level starts with each node in its members' community.
        uint32_t* next_labels = alloc<uint32_t>(ncol);
        uint32_t* fold2 = alloc<uint32_t>(n0);
        if (!ok_) return oom();
        cl_scatter_kernel<<<grid_for(n), 256, 0, s_>>>(collapse, partition, n, next_labels);
        cl_relabel_kernel<<<grid_for(n0), 256, 0, s_>>>(fold, n0, collapse, fold2);
        ctx_->launches += 2;
        fold = fold2;
        level = next;
        labels = next_labels;
    }
    return fail(st_, SCRUST_KERNEL, "clustering: no convergence after 64 levels");
}

int32_t Clusterer::run(bool leiden, double res, int n_iterations, uint64_t seed, uint32_t* out_labels,
                       double* out_q, uint64_t* out_nc) {
    const int64_t n = g0_.n;
    uint32_t* cur = alloc<uint32_t>(n);
    uint32_t* found = alloc<uint32_t>(n);
    unsigned int* differ = alloc<unsigned int>(1);
    if (!ok_) return oom();
    cl_iota_kernel<<<grid_for(n), 256, 0, s_>>>(n, cur);
    ctx_->launches += 1;
    int64_t nc = n;
    const int passes = leiden ? n_iterations : 1;
    for (int pass = 0; pass < passes; ++pass) {
        int64_t fnc = 0;
        int32_t rc = optimise(cur, res, leiden, mix_host(seed ^ ((uint64_t)pass << 40)), found, &fnc);
        if (rc) return rc;
        if (leiden) {
            // A pass that returns its own input has converged (cluster.rs:104-118).
            cudaMemsetAsync(differ, 0, sizeof(unsigned int), s_);
            cl_differ_kernel<<<grid_for(n), 256, 0, s_>>>(found, cur, n, differ);
            ctx_->launches += 1;
            unsigned int hd = 0;
            if (!download(&hd, differ, 1)) return fail(st_, SCRUST_KERNEL, "clustering: compare");
            if (!hd) break;
        }
        cudaMemcpyAsync(cur, found, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s_);
        nc = fnc;
    }
    // Labels by descending community size, ties to the smaller id (cluster.rs:828-850).
    int* size = alloc<int>(nc);
    long long* strength = alloc<long long>(nc);
    uint32_t* kA = alloc<uint32_t>(nc);
    uint32_t* kB = alloc<uint32_t>(nc);
    unsigned long long* vA = alloc<unsigned long long>(nc);
    unsigned long long* vB = alloc<unsigned long long>(nc);
    uint32_t* rank = alloc<uint32_t>(nc);
    if (!ok_) return oom();
    cudaMemsetAsync(size, 0, sizeof(int) * nc, s_);
    cudaMemsetAsync(strength, 0, sizeof(long long) * nc, s_);
    cl_comm_init_kernel<<<grid_for(n), 256, 0, s_>>>(cur, g0_.kfix, n, strength, size);
    cl_size_keys_kernel<<<grid_for(nc), 256, 0, s_>>>(size, nc, kA, vA);
    ctx_->launches += 2;
    uint32_t* keys = nullptr;
    unsigned long long* order = nullptr;
    cudaError_t e;
    if ((e = sort_pairs(kA, vA, kB, vB, nc, 32, &keys, &order)) != cudaSuccess)
        return cuda_fail(st_, e, "clustering: label order");
    cl_rank_kernel<<<grid_for(nc), 256, 0, s_>>>(order, nc, rank);
    cl_relabel_kernel<<<grid_for(n), 256, 0, s_>>>(cur, n, rank, out_labels);
    ctx_->launches += 2;
    *out_q = score(g0_, out_labels, nc, res);
    *out_nc = (uint64_t)nc;
    if (!ok_) return fail(st_, SCRUST_KERNEL, "clustering: score");
    return ok(st_);
}

int32_t Clusterer::score_only(const uint32_t* labels, int64_t nc, double res, double* out_q) {
    *out_q = score(g0_, labels, nc, res);
    if (!ok_) return fail(st_, SCRUST_KERNEL, "clustering: score");
    return ok(st_);
}

}  // namespace scrust

using namespace scrust;

namespace {

int32_t check_graph(const uint32_t* indptr, const uint32_t* indices, uint64_t n, uint64_t n_cols, scrust_status* st) {
    if (n == 0 || n_cols != n)
        return fail(st, SCRUST_SHAPE, "expected a square graph with at least one node, got %llu x %llu",
                    (unsigned long long)n, (unsigned long long)n_cols);
    if (!indptr) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    const uint64_t nnz = indptr[n];
    if (nnz && !indices) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    if (indptr[0] != 0) return fail(st, SCRUST_SHAPE, "expected indptr to start at 0");
    for (uint64_t r = 0; r < n; ++r)
        if (indptr[r + 1] < indptr[r]) return fail(st, SCRUST_SHAPE, "expected a non-decreasing indptr");
    for (uint64_t i = 0; i < nnz; ++i)
        if (indices[i] >= n_cols) return fail(st, SCRUST_SHAPE, "expected column indices below %llu", (unsigned long long)n_cols);
    if (n >= 0x7fffff00ull || 2 * nnz >= 0xffffff00ull) return fail(st, SCRUST_SHAPE, "expected fewer than 2^31 entries");
    return SCRUST_OK;
}

int32_t check_resolution(double res, scrust_status* st) {
    if (!std::isfinite(res) || res <= 0.0)
        return fail(st, SCRUST_INVALID_PARAMETER, "resolution must be finite and greater than zero, got %g", res);
    return SCRUST_OK;
}

// Host CSR in; runs `body` with the device copy.
template <class Fn>
int32_t with_device_graph(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                          uint64_t n, scrust_status* st, Fn body) {
    const uint64_t nnz = indptr[n];
    cudaError_t e;
    const size_t o_ix = ((sizeof(uint32_t) * (n + 1)) + 255) & ~(size_t)255;
    const size_t o_vl = o_ix + (((sizeof(uint32_t) * std::max<uint64_t>(nnz, 1)) + 255) & ~(size_t)255);
    const size_t bytes = o_vl + sizeof(float) * std::max<uint64_t>(nnz, 1);
    char* buf = (char*)ws_get(ctx, SLOT_HOST_IN, bytes, &e);
    if (!buf) return cuda_fail(st, e, "workspace");
    if ((e = cudaMemcpyAsync(buf, indptr, sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, ctx->stream)) !=
            cudaSuccess ||
        (nnz && (e = cudaMemcpyAsync(buf + o_ix, indices, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, ctx->stream)) !=
                    cudaSuccess) ||
        (nnz && (e = cudaMemcpyAsync(buf + o_vl, values, sizeof(float) * nnz, cudaMemcpyHostToDevice, ctx->stream)) !=
                    cudaSuccess))
        return cuda_fail(st, e, "upload");
    return body((const uint32_t*)buf, (const uint32_t*)(buf + o_ix), (const float*)(buf + o_vl), (int64_t)nnz);
}

int32_t cluster_host(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                     uint64_t n, uint64_t n_cols, bool leiden, double res, uint32_t n_iterations, uint64_t seed,
                     uint32_t* out_labels, double* out_q, uint64_t* out_nc, scrust_status* st) {
    int32_t rc = check_resolution(res, st);
    if (rc) return rc;
    if (leiden && n_iterations == 0) return fail(st, SCRUST_INVALID_PARAMETER, "n_iterations must be at least 1, got 0");
    if ((rc = check_graph(indptr, indices, n, n_cols, st))) return rc;
    if (!out_labels || !out_q || !out_nc || (indptr[n] && !values)) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    return with_device_graph(ctx, indptr, indices, values, n, st,
                             [&](const uint32_t* dip, const uint32_t* dix, const float* dvl, int64_t nnz) -> int32_t {
                                 Clusterer c(ctx, st);
                                 int32_t r = c.build(dip, dix, dvl, (int64_t)n, nnz);
                                 if (r) return r;
                                 uint32_t* dl = c.alloc<uint32_t>(n);
                                 if (!dl) return fail(st, SCRUST_OOM, "clustering: device allocation failed");
                                 if ((r = c.run(leiden, res, (int)n_iterations, seed, dl, out_q, out_nc))) return r;
                                 cudaError_t e = cudaMemcpyAsync(out_labels, dl, sizeof(uint32_t) * n,
                                                                 cudaMemcpyDeviceToHost, ctx->stream);
                                 if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                                 if (e != cudaSuccess) return cuda_fail(st, e, "download");
                                 return collect_device_errors(ctx, st);
                             });
}

}  // namespace

extern "C" {

int32_t scrust_cuda_leiden(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                           uint64_t n_rows, uint64_t n_cols, double resolution, uint32_t n_iterations, uint64_t seed,
                           uint32_t* out_labels, double* out_modularity, uint64_t* out_n_communities,
                           scrust_status* st) {
    return cluster_host(ctx, indptr, indices, values, n_rows, n_cols, true, resolution, n_iterations, seed, out_labels,
                        out_modularity, out_n_communities, st);
}

int32_t scrust_cuda_louvain(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                            uint64_t n_rows, uint64_t n_cols, double resolution, uint64_t seed, uint32_t* out_labels,
                            double* out_modularity, uint64_t* out_n_communities, scrust_status* st) {
    return cluster_host(ctx, indptr, indices, values, n_rows, n_cols, false, resolution, 1, seed, out_labels,
                        out_modularity, out_n_communities, st);
}

int32_t scrust_cuda_modularity(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices,
                               const float* values, uint64_t n_rows, uint64_t n_cols, const uint32_t* labels,
                               uint64_t n_labels, double resolution, double* out, scrust_status* st) {
    int32_t rc = check_resolution(resolution, st);
    if (rc) return rc;
    if ((rc = check_graph(indptr, indices, n_rows, n_cols, st))) return rc;
    if (!labels || !out || (indptr[n_rows] && !values)) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    if (n_labels != n_rows)
        return fail(st, SCRUST_SHAPE, "expected %llu labels, one per node, got %llu", (unsigned long long)n_rows,
                    (unsigned long long)n_labels);
    uint32_t mx = 0;
    for (uint64_t i = 0; i < n_labels; ++i) mx = std::max(mx, labels[i]);
    if ((uint64_t)mx + 1 > n_rows)
        return fail(st, SCRUST_INVALID_PARAMETER, "labels must be community ids below the node count, got %u", mx);
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    return with_device_graph(ctx, indptr, indices, values, n_rows, st,
                             [&](const uint32_t* dip, const uint32_t* dix, const float* dvl, int64_t nnz) -> int32_t {
                                 Clusterer c(ctx, st);
                                 int32_t r = c.build(dip, dix, dvl, (int64_t)n_rows, nnz);
                                 if (r) return r;
                                 uint32_t* dl = c.alloc<uint32_t>(n_rows);
                                 if (!dl) return fail(st, SCRUST_OOM, "clustering: device allocation failed");
                                 cudaMemcpyAsync(dl, labels, sizeof(uint32_t) * n_rows, cudaMemcpyHostToDevice,
                                                 ctx->stream);
                                 return c.score_only(dl, (int64_t)mx + 1, resolution, out);
                             });
}

}  // extern "C"
