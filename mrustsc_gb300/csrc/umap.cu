// umap.cu -- the UMAP layout of a connectivities graph on the GPU, the
// consumer of the graph this library builds (crates/scrust-core/src/umap.rs:64).
//
// The reference optimises the layout with umap-learn's sequential SGD: edges
// in CSR order, every update applied at once to the shared layout
// (umap.rs:393-452).  A sequential sweep has no parallel form, and the
// reference's own GPU kernel (crates/scrust-gpu/src/kernels/umap_sgd.rs) is
// Hogwild: racing writes, so not reproducible even against itself.  This
// layout is deterministic instead: within an epoch every update is computed
// from the layout as it stood when the epoch began, and applied as one sum
// per cell in a fixed order.
//   - One thread per cell walks its CSR row in order, as the reference walks
//     the edges whose head is that cell: the same firing schedule
//     (epochs_per_sample from max / weight, umap.rs:113-170), the same
//     per-cell Tausworthe stream for the negative samples (seeded from the
//     seed and the cell id, umap.rs:407-412), so every cell draws exactly the
//     reference's negative samples, and the same attraction, repulsion and
//     +-4 clip (umap.rs:454-509).  It sums the cell's own moves in row order
//     and keeps each attraction's move of the edge's tail.
//   - One thread per cell then adds the moves its incoming edges gave it,
//     in edge order (a stable transpose made once), and writes the cell's
//     next position.
// Two runs with the same inputs give the same bits.  The layout differs from
// the reference's sequential one by the usual Jacobi-versus-Gauss-Seidel
// amount; the tests hold it to the reference's own quality bars and to the
// sequential restatement's trustworthiness within a stated tolerance.
//
// The initial layout is umap-learn's init="random" as the reference does it
// (uniform in [-10, 10], then each component rescaled to [0, 10]), drawn
// from one Tausworthe stream per cell instead of one stream for all cells,
// so the cells draw in parallel.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

constexpr int kUmapMaxDim = 16;
constexpr float kClip = 4.0f;
constexpr float kRepulsionEps = 0.001f;
constexpr float kInitRange = 10.0f;
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;
constexpr uint64_t kInitSalt = 0x5CA1AB1E0DDBA11ull;

struct Tau {
    uint32_t s0, s1, s2;
};

__host__ __device__ __forceinline__ uint64_t splitmix_word(uint64_t* st) {
    *st += kGolden;
    uint64_t z = *st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// TauRng::new (umap.rs:179-193): three splitmix64 words, low bits forced.
__device__ __forceinline__ Tau tau_seed(uint64_t seed) {
    uint64_t sm = seed;
    Tau t;
    t.s0 = (uint32_t)splitmix_word(&sm) | 0x2u;
    t.s1 = (uint32_t)splitmix_word(&sm) | 0x8u;
    t.s2 = (uint32_t)splitmix_word(&sm) | 0x10u;
    return t;
}

// TauRng::next_u32 (umap.rs:195-201), umap-learn's tau88 recurrence.
__device__ __forceinline__ uint32_t tau_next(Tau& t) {
    t.s0 = ((t.s0 & 4294967294u) << 12) ^ (((t.s0 << 13) ^ t.s0) >> 19);
    t.s1 = ((t.s1 & 4294967288u) << 4) ^ (((t.s1 << 2) ^ t.s1) >> 25);
    t.s2 = ((t.s2 & 4294967280u) << 17) ^ (((t.s2 << 3) ^ t.s2) >> 11);
    return t.s0 ^ t.s1 ^ t.s2;
}

__device__ __forceinline__ float clip4(float v) { return fminf(fmaxf(v, -kClip), kClip); }

// Order-preserving key of a float for atomicMin / atomicMax on u32.
__device__ __forceinline__ uint32_t fkey(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fval(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void umap_max_weight_kernel(const float* __restrict__ w, int64_t nnz, uint32_t* __restrict__ key) {
    uint32_t best = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
        best = max(best, fkey(w[e]));
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(key, best);
}

// EdgeList::from_graph (umap.rs:126-169) in CSR order: an edge fires every
// max / weight epochs; weights at or below 0 or below max / n_epochs never
// fire.  Counts the edges that fire.
__global__ void umap_edges_kernel(const float* __restrict__ w, int64_t nnz, const uint32_t* __restrict__ max_key,
                                  int n_epochs, int neg_rate, double* __restrict__ eps, double* __restrict__ eps_neg,
                                  double* __restrict__ next, double* __restrict__ next_neg,
                                  unsigned long long* __restrict__ live) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    const float maxw = fval(*max_key);
    const float threshold = __fdiv_rn(maxw, (float)n_epochs);
    const float we = w[e];
    const bool fires = !(we <= 0.f || we < threshold);
    const double ep = fires ? (double)maxw / (double)we : INFINITY;
    const double en = fires && neg_rate ? ep / (double)neg_rate : INFINITY;
    eps[e] = ep;
    eps_neg[e] = en;
    next[e] = ep;
    next_neg[e] = en;
    if (fires) atomicAdd(live, 1ull);
}

// The initial layout: uniform in [-10, 10] from each cell's own stream, and
// each component's range for the rescale.
__global__ void umap_init_kernel(int64_t n, int dim, uint64_t seed, float* __restrict__ y, uint32_t* __restrict__ lo,
                                 uint32_t* __restrict__ hi, Tau* __restrict__ rng) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    Tau t = tau_seed(seed ^ ((uint64_t)v * kGolden) ^ kInitSalt);
    for (int c = 0; c < dim; ++c) {
        const float u = __fdiv_rn((float)tau_next(t), 4294967296.0f);
        const float val = __fmul_rn(__fsub_rn(__fmul_rn(u, 2.0f), 1.0f), kInitRange);
        y[v * dim + c] = val;
        atomicMin(lo + c, fkey(val));
        atomicMax(hi + c, fkey(val));
    }
    rng[v] = tau_seed(seed ^ ((uint64_t)v * kGolden));
}

// rescale_to_init_range (umap.rs:241-257).
__global__ void umap_rescale_kernel(int64_t n, int dim, const uint32_t* __restrict__ lo,
                                    const uint32_t* __restrict__ hi, float* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * dim) return;
    const int c = (int)(i % dim);
    const float l = fval(lo[c]), h = fval(hi[c]);
    const float range = __fsub_rn(h, l);
    y[i] = range > 0.f ? __fdiv_rn(__fmul_rn(kInitRange, __fsub_rn(y[i], l)), range) : 0.f;
}

// One epoch, the cells' own edges: attraction of every firing edge (its
// tail's move kept in tmove) and the negative samples, summed per cell in
// row order into own.
__global__ void umap_rows_kernel(const uint32_t* __restrict__ indptr, const uint32_t* __restrict__ indices,
                                 int64_t n, int dim, double now, float alpha, float a, float b, int neg_rate,
                                 const float* __restrict__ y, const double* __restrict__ eps,
                                 const double* __restrict__ eps_neg, double* __restrict__ next,
                                 double* __restrict__ next_neg, Tau* __restrict__ rng, float* __restrict__ tmove,
                                 float* __restrict__ own) {
    const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= n) return;
    float yh[kUmapMaxDim], acc[kUmapMaxDim];
#pragma unroll
    for (int d = 0; d < kUmapMaxDim; ++d) {
        yh[d] = d < dim ? y[h * dim + d] : 0.f;
        acc[d] = 0.f;
    }
    Tau t = rng[h];
    const float two_ab = __fmul_rn(__fmul_rn(-2.0f, a), b);
    const float two_b = __fmul_rn(2.0f, b);  // 2 * REPULSION_STRENGTH(1) * b
    for (uint32_t e = indptr[h], e1 = indptr[h + 1]; e < e1; ++e) {
        if (next[e] > now) {
            for (int d = 0; d < dim; ++d) tmove[(int64_t)e * dim + d] = 0.f;
            continue;
        }
        const int64_t tail = indices[e];
        float dist = 0.f;
#pragma unroll
        for (int d = 0; d < kUmapMaxDim; ++d) {
            if (d < dim) {
                const float diff = __fsub_rn(yh[d], y[tail * dim + d]);
                dist = __fadd_rn(dist, __fmul_rn(diff, diff));
            }
        }
        float coef = 0.f;
        if (dist > 0.f)
            coef = __fdiv_rn(__fmul_rn(two_ab, powf(dist, __fsub_rn(b, 1.0f))),
                             __fadd_rn(__fmul_rn(a, powf(dist, b)), 1.0f));
#pragma unroll
        for (int d = 0; d < kUmapMaxDim; ++d) {
            if (d < dim) {
                const float g = clip4(__fmul_rn(coef, __fsub_rn(yh[d], y[tail * dim + d])));
                const float step = __fmul_rn(g, alpha);
                acc[d] = __fadd_rn(acc[d], step);
                tmove[(int64_t)e * dim + d] = step;
            }
        }
        next[e] += eps[e];
        if (neg_rate == 0) continue;
        double q = (now - next_neg[e]) / eps_neg[e];
        const int64_t n_neg = q > 0.0 ? (int64_t)q : 0;
        for (int64_t s = 0; s < n_neg; ++s) {
            const int64_t j = (int64_t)(tau_next(t) % (uint32_t)n);
            if (j == h) continue;
            float dj = 0.f;
#pragma unroll
            for (int d = 0; d < kUmapMaxDim; ++d) {
                if (d < dim) {
                    const float diff = __fsub_rn(yh[d], y[j * dim + d]);
                    dj = __fadd_rn(dj, __fmul_rn(diff, diff));
                }
            }
            if (dj <= 0.f) continue;
            const float cr = __fdiv_rn(two_b, __fmul_rn(__fadd_rn(kRepulsionEps, dj),
                                                          __fadd_rn(__fmul_rn(a, powf(dj, b)), 1.0f)));
#pragma unroll
            for (int d = 0; d < kUmapMaxDim; ++d)
                if (d < dim)
                    acc[d] = __fadd_rn(acc[d], __fmul_rn(clip4(__fmul_rn(cr, __fsub_rn(yh[d], y[j * dim + d]))),
                                                         alpha));
        }
        next_neg[e] += (double)n_neg * eps_neg[e];
    }
    rng[h] = t;
#pragma unroll
    for (int d = 0; d < kUmapMaxDim; ++d)
        if (d < dim) own[h * dim + d] = acc[d];
}

// One epoch, the moves a cell receives as the tail of its incoming edges, in
// edge order, then the cell's next position.
__global__ void umap_apply_kernel(int64_t n, int dim, const uint32_t* __restrict__ tstart,
                                  const unsigned long long* __restrict__ tedge, const float* __restrict__ tmove,
                                  const float* __restrict__ own, const float* __restrict__ y,
                                  float* __restrict__ y_next) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    float acc[kUmapMaxDim];
#pragma unroll
    for (int d = 0; d < kUmapMaxDim; ++d) acc[d] = d < dim ? own[v * dim + d] : 0.f;
    for (uint32_t p = tstart[v], p1 = tstart[v + 1]; p < p1; ++p) {
        const int64_t e = (int64_t)(tedge[p] & 0xffffffffull);
#pragma unroll
        for (int d = 0; d < kUmapMaxDim; ++d)
            if (d < dim) acc[d] = __fsub_rn(acc[d], tmove[e * dim + d]);
    }
#pragma unroll
    for (int d = 0; d < kUmapMaxDim; ++d)
        if (d < dim) y_next[v * dim + d] = __fadd_rn(y[v * dim + d], acc[d]);
}

__global__ void umap_keys_kernel(const uint32_t* __restrict__ indices, int64_t nnz, uint32_t* __restrict__ keys,
                                 unsigned long long* __restrict__ vals) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    keys[e] = indices[e];
    vals[e] = (unsigned long long)e;
}

// start[c] = number of sorted keys below c, for c in [0, n].
__global__ void umap_starts_kernel(const uint32_t* __restrict__ keys, int64_t nnz, int64_t n,
                                   uint32_t* __restrict__ start) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p > nnz) return;
    const int64_t lo = p == 0 ? 0 : (int64_t)keys[p - 1] + 1;
    const int64_t hi = p == nnz ? n : (int64_t)keys[p];
    for (int64_t c = lo; c <= hi && c <= n; ++c) start[c] = (uint32_t)p;
}

// Damped Gauss-Newton fit of 1 / (1 + a x^(2b)) to the offset exponential on
// 300 points of [0, 3 spread] (umap.rs:272-391): the two curve parameters of
// the layout, fixed before any device work.
bool fit_ab(float min_dist_f, float spread_f, float* a_out, float* b_out) {
    if (!(spread_f > 0.0f) || !(min_dist_f >= 0.0f && min_dist_f <= spread_f * 3.0f)) return false;
    const int S = 300;
    std::vector<double> xs(S), ys(S);
    const double md = (double)min_dist_f, sp = (double)spread_f;
    for (int i = 0; i < S; ++i) {
        xs[i] = 3.0 * sp * (double)i / (double)(S - 1);
        ys[i] = xs[i] < md ? 1.0 : exp(-(xs[i] - md) / sp);
    }
    auto term_of = [](double x, double b, double* lf) {
        if (x <= 0.0) {
            *lf = 0.0;
            return 0.0;
        }
        *lf = 2.0 * log(x);
        return pow(x, 2.0 * b);
    };
    auto cost_of = [&](double a, double b) {
        double s = 0.0;
        for (int i = 0; i < S; ++i) {
            double lf;
            const double r = 1.0 / (1.0 + a * term_of(xs[i], b, &lf)) - ys[i];
            s += r * r;
        }
        return s;
    };
    double a = 1.0, b = 1.0, damping = 1e-3, cost = cost_of(a, b);
    for (int it = 0; it < 200; ++it) {
        double jaa = 0, jab = 0, jbb = 0, ga = 0, gb = 0;
        for (int i = 0; i < S; ++i) {
            double lf;
            const double t = term_of(xs[i], b, &lf);
            const double den = 1.0 + a * t, sq = den * den;
            const double r = 1.0 / den - ys[i], da = -t / sq, db = -a * t * lf / sq;
            jaa += da * da;
            jab += da * db;
            jbb += db * db;
            ga += da * r;
            gb += db * r;
        }
        const double daa = jaa * (1.0 + damping), dbb = jbb * (1.0 + damping);
        const double det = daa * dbb - jab * jab;
        if (fabs(det) < 2.220446049250313e-16) break;
        const double ta = a - (dbb * ga - jab * gb) / det, tb = b - (daa * gb - jab * ga) / det;
        if (ta <= 0.0 || tb <= 0.0) {
            damping *= 10.0;
            continue;
        }
        const double tc = cost_of(ta, tb);
        if (tc < cost) {
            const double improvement = cost - tc;
            a = ta;
            b = tb;
            cost = tc;
            damping = damping * 0.1 > 1e-12 ? damping * 0.1 : 1e-12;
            if (improvement < 1e-14) break;
        } else {
            damping *= 10.0;
            if (damping > 1e12) break;
        }
    }
    *a_out = (float)a;
    *b_out = (float)b;
    return true;
}

int32_t check_umap_params(const scrust_umap_params& p, scrust_status* st) {
    if (p.n_components == 0) return fail(st, SCRUST_INVALID_PARAMETER, "n_components must be at least 1, got 0");
    if (p.n_components > (uint32_t)kUmapMaxDim)
        return fail(st, SCRUST_INVALID_PARAMETER, "n_components must be at most %d, got %u", kUmapMaxDim,
                    p.n_components);
    if (p.n_epochs == 0) return fail(st, SCRUST_INVALID_PARAMETER, "n_epochs must be at least 1, got 0");
    if (!(p.spread > 0.f)) return fail(st, SCRUST_INVALID_PARAMETER, "spread must be greater than 0, got %g", p.spread);
    if (!(p.min_dist >= 0.f && p.min_dist <= p.spread * 3.0f))
        return fail(st, SCRUST_INVALID_PARAMETER, "min_dist must be in [0, 3 * spread], got %g", p.min_dist);
    return SCRUST_OK;
}

size_t al(size_t v) { return (v + 255) & ~(size_t)255; }

// The layout of a device-resident CSR graph (n x n, nnz entries) into
// out (n x dim, device), enqueued on ctx->stream; synchronises once to learn
// whether any edge fires.
int32_t umap_device_impl(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                         int64_t n, int64_t nnz, const scrust_umap_params& p, float* out, scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int dim = (int)p.n_components;
    float a = 0.f, b = 0.f;
    if (!fit_ab(p.min_dist, p.spread, &a, &b)) return fail(st, SCRUST_INVALID_PARAMETER, "min_dist / spread out of range");
    // Workspace: per edge schedules (4 f64), tail moves (dim f32), transpose
    // keys and payloads (2 x u32, 2 x u64); per cell the second layout, own
    // moves, stream state, bucket starts; small counters.
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t r = off;
        off = al(off + bytes);
        return r;
    };
    const size_t o_eps = take(8 * (size_t)nnz), o_epsn = take(8 * (size_t)nnz), o_nx = take(8 * (size_t)nnz),
                 o_nxn = take(8 * (size_t)nnz), o_tm = take(4 * (size_t)nnz * dim), o_ka = take(4 * (size_t)nnz),
                 o_kb = take(4 * (size_t)nnz), o_va = take(8 * (size_t)nnz), o_vb = take(8 * (size_t)nnz),
                 o_y2 = take(4 * (size_t)n * dim), o_own = take(4 * (size_t)n * dim),
                 o_rng = take(sizeof(Tau) * (size_t)n), o_ts = take(4 * (size_t)(n + 1)), o_small = take(256);
    const int nb = radix_blocks(nnz);
    const size_t scan_elems = scan_scratch_elems((int64_t)256 * nb);
    const size_t o_hist = take(4 * ((size_t)256 * nb + 16)), o_scan = take(4 * scan_elems);
    char* base = (char*)ws_get(ctx, SLOT_UMAP, off, &e);
    if (!base) return cuda_fail(st, e, "umap: workspace");
    double* eps = (double*)(base + o_eps);
    double* eps_neg = (double*)(base + o_epsn);
    double* next = (double*)(base + o_nx);
    double* next_neg = (double*)(base + o_nxn);
    float* tmove = (float*)(base + o_tm);
    uint32_t* kA = (uint32_t*)(base + o_ka);
    uint32_t* kB = (uint32_t*)(base + o_kb);
    unsigned long long* vA = (unsigned long long*)(base + o_va);
    unsigned long long* vB = (unsigned long long*)(base + o_vb);
    float* y2 = (float*)(base + o_y2);
    float* own = (float*)(base + o_own);
    Tau* rng = (Tau*)(base + o_rng);
    uint32_t* tstart = (uint32_t*)(base + o_ts);
    uint32_t* small = (uint32_t*)(base + o_small);  // [0] max key, [2..3] live edges, [8..) lo, [24..) hi
    unsigned long long* live = (unsigned long long*)(small + 2);
    uint32_t* lo = small + 8;
    uint32_t* hi = small + 8 + kUmapMaxDim;
    if ((e = cudaMemsetAsync(small, 0, 8 * sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(lo, 0xff, sizeof(uint32_t) * kUmapMaxDim, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(hi, 0, sizeof(uint32_t) * kUmapMaxDim, s)) != cudaSuccess)
        return cuda_fail(st, e, "umap: memset");
    const unsigned eb = (unsigned)((nnz + 255) / 256);
    umap_max_weight_kernel<<<std::min<unsigned>(eb, 4 * (unsigned)ctx->sm_count), 256, 0, s>>>(values, nnz, small);
    umap_edges_kernel<<<eb, 256, 0, s>>>(values, nnz, small, (int)p.n_epochs, (int)p.negative_sample_rate, eps,
                                         eps_neg, next, next_neg, live);
    unsigned long long live_h = 0;
    if ((e = cudaMemcpyAsync(&live_h, live, sizeof(live_h), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(st, e, "umap: edges");
    if (live_h == 0) return fail(st, SCRUST_SHAPE, "expected a graph with at least one edge, got no edges");
    // Stable transpose: edges by tail, then by edge id.
    umap_keys_kernel<<<eb, 256, 0, s>>>(indices, nnz, kA, vA);
    int bits = 1;
    while (((int64_t)1 << bits) <= n) bits++;
    uint32_t* keys = nullptr;
    unsigned long long* vals = nullptr;
    if ((e = radix_sort_pairs(ctx, kA, vA, kB, vB, nnz, bits, (uint32_t*)(base + o_hist), (uint32_t*)(base + o_scan),
                              scan_elems, &keys, &vals)) != cudaSuccess)
        return cuda_fail(st, e, "umap: transpose");
    umap_starts_kernel<<<(unsigned)((nnz + 1 + 255) / 256), 256, 0, s>>>(keys, nnz, n, tstart);
    const unsigned vb = (unsigned)((n + 127) / 128);
    umap_init_kernel<<<vb, 128, 0, s>>>(n, dim, p.seed, out, lo, hi, rng);
    umap_rescale_kernel<<<(unsigned)((n * dim + 255) / 256), 256, 0, s>>>(n, dim, lo, hi, out);
    ctx->launches += 8;
    float* cur = out;
    float* nxt = y2;
    float alpha = p.learning_rate;
    for (uint32_t epoch = 0; epoch < p.n_epochs; ++epoch) {
        umap_rows_kernel<<<vb, 128, 0, s>>>(indptr, indices, n, dim, (double)epoch, alpha, a, b,
                                            (int)p.negative_sample_rate, cur, eps, eps_neg, next, next_neg, rng,
                                            tmove, own);
        umap_apply_kernel<<<vb, 128, 0, s>>>(n, dim, tstart, vals, tmove, own, cur, nxt);
        std::swap(cur, nxt);
        alpha = p.learning_rate * (1.0f - (float)epoch / (float)p.n_epochs);
    }
    ctx->launches += 2ull * p.n_epochs;
    if (cur != out &&
        (e = cudaMemcpyAsync(out, cur, sizeof(float) * (size_t)n * dim, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail(st, e, "umap: copy");
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "umap");
    return ok(st);
}

}  // namespace

}  // namespace scrust

using namespace scrust;

extern "C" {

void scrust_umap_params_default(scrust_umap_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(*p);
    p->n_components = 2;
    p->n_epochs = 200;
    p->min_dist = 0.5f;
    p->spread = 1.0f;
    p->learning_rate = 1.0f;
    p->negative_sample_rate = 5;
    p->seed = 0;
}

int32_t scrust_cuda_umap_device(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices,
                                const float* values, uint64_t n_rows, uint64_t n_cols, uint64_t nnz,
                                const scrust_umap_params* params, float* out_embedding, scrust_status* st) {
    scrust_umap_params p;
    scrust_umap_params_default(&p);
    if (params) p = *params;
    int32_t rc = check_umap_params(p, st);
    if (rc) return rc;
    if (n_rows == 0 || nnz == 0) return fail(st, SCRUST_SHAPE, "expected a non-empty connectivity graph, got empty graph");
    if (n_cols != n_rows)
        return fail(st, SCRUST_SHAPE, "expected a square %llux%llu graph, got %llux%llu", (unsigned long long)n_rows,
                    (unsigned long long)n_rows, (unsigned long long)n_rows, (unsigned long long)n_cols);
    if (n_rows >= 0xffffff00ull || nnz >= 0xffffff00ull)
        return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 cells and entries");
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!indptr || !indices || !values || !out_embedding) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    return umap_device_impl(ctx, indptr, indices, values, (int64_t)n_rows, (int64_t)nnz, p, out_embedding, st);
}

int32_t scrust_cuda_umap(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                         uint64_t n_rows, uint64_t n_cols, const scrust_umap_params* params, float* out_embedding,
                         scrust_status* st) {
    scrust_umap_params p;
    scrust_umap_params_default(&p);
    if (params) p = *params;
    int32_t rc = check_umap_params(p, st);
    if (rc) return rc;
    if (!indptr) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    const uint64_t nnz = n_rows ? indptr[n_rows] : 0;
    if (n_rows == 0 || nnz == 0) return fail(st, SCRUST_SHAPE, "expected a non-empty connectivity graph, got empty graph");
    if (n_cols != n_rows)
        return fail(st, SCRUST_SHAPE, "expected a square %llux%llu graph, got %llux%llu", (unsigned long long)n_rows,
                    (unsigned long long)n_rows, (unsigned long long)n_rows, (unsigned long long)n_cols);
    if (!indices || !values || !out_embedding) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    // CsrMatrix::new's structural checks (crates/scrust-core/src/sparse.rs:18-90).
    if (indptr[0] != 0) return fail(st, SCRUST_SHAPE, "expected indptr to start at 0");
    for (uint64_t r = 0; r < n_rows; ++r)
        if (indptr[r + 1] < indptr[r]) return fail(st, SCRUST_SHAPE, "expected a non-decreasing indptr");
    for (uint64_t i = 0; i < nnz; ++i)
        if (indices[i] >= n_cols) return fail(st, SCRUST_SHAPE, "expected column indices below %llu", (unsigned long long)n_cols);
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (n_rows >= 0xffffff00ull || nnz >= 0xffffff00ull)
        return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 cells and entries");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    const size_t y_bytes = sizeof(float) * n_rows * p.n_components;
    const size_t o_ind = (sizeof(uint32_t) * (n_rows + 1) + 255) & ~(size_t)255;
    const size_t o_val = o_ind + ((sizeof(uint32_t) * nnz + 255) & ~(size_t)255);
    const size_t o_y = o_val + ((sizeof(float) * nnz + 255) & ~(size_t)255);
    char* dbuf = (char*)ws_get(ctx, SLOT_HOST_IN, o_y + y_bytes, &e);
    if (!dbuf) return cuda_fail(st, e, "workspace");
    uint32_t* d_indptr = (uint32_t*)dbuf;
    uint32_t* d_indices = (uint32_t*)(dbuf + o_ind);
    float* d_values = (float*)(dbuf + o_val);
    float* d_y = (float*)(dbuf + o_y);
    if ((e = cudaMemcpyAsync(d_indptr, indptr, sizeof(uint32_t) * (n_rows + 1), cudaMemcpyHostToDevice, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(d_indices, indices, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(d_values, values, sizeof(float) * nnz, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "upload");
    if ((rc = umap_device_impl(ctx, d_indptr, d_indices, d_values, (int64_t)n_rows, (int64_t)nnz, p, d_y, st))) return rc;
    if ((e = cudaMemcpyAsync(out_embedding, d_y, y_bytes, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "download");
    return collect_device_errors(ctx, st);
}

}  // extern "C"
