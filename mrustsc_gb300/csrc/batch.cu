// batch.cu -- many independent self-kNN solves (samples of different cell
// counts) in one tensor sweep.
//
// The samples' rows are laid out block-diagonally: sample s occupies the
// 256-row blocks [P_s, P_s + ceil(n_s / 256)), padded with rows that can
// never become candidates.  Every row block sweeps only its own sample's
// column tiles, so one persistent launch of the tensor kernel covers all
// samples, the heaviest row blocks first.  Because every solve is exact,
// each sample's neighbour lists and distances are the same bits as a solve
// of that sample alone.
//
// Graphs: each sample's UMAP connectivities follow in the same sequence.  The
// sample-local neighbour ids are made batch-global (sample offset added), so
// the batch is one block-diagonal kNN graph; smooth_knn and the directed
// weights are row-local and the fuzzy union of a block-diagonal graph is
// block-diagonal, so one connectivities pass over the whole batch gives
// every sample's rows exactly as a pass over that sample alone would.  A
// last pass makes the column ids sample-local again.
//
// A plan fixes the layout, the buffers and the options, autotunes the
// candidate over-provisioning (list capacity), the register top-k width and
// the operand precision on the actual batch, and captures the whole sequence
// in a CUDA graph; each run is one graph launch.  The tile shape (two 128-row
// MMA halves against 256-column tiles, K = 64) is the sweep kernel's fixed
// design and is not a tuning choice.
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"
#include "internal.h"

struct scrust_batch_plan {
    scrust_context* ctx = nullptr;
    uint32_t n_samples = 0;
    uint64_t n_total = 0, d = 0;
    uint32_t k = 0;
    scrust_knn_options opts{};
    const float* x = nullptr;
    uint32_t* out_idx = nullptr;
    float* out_dist = nullptr;
    void* table = nullptr;  // device copy of the sample table
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    float tuned_ms = 0.f;
    int32_t topk_width = 0;            // the autotuner's register top-k width (0: by k, -1: lists)
    bool graphs = false;               // the launch also builds the connectivities
    scrust::CsrBuffers csr;            // the batch's connectivities (sample-local columns)
};

namespace scrust {

namespace {

struct SampleRow {
    uint32_t start;  // first 256-row block position of the sample (P_s * 256)
    uint32_t off;    // first input row
    uint32_t n;      // rows
    uint32_t pad;
};

__device__ __forceinline__ int sample_of(const SampleRow* t, int S, uint32_t v, bool by_position) {
    int lo = 0, hi = S - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((by_position ? t[mid].start : t[mid].off) <= v)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Position -> input row (0xffffffff for padding), input row -> its sample's
// [first, end) rows, and per row block its sample's column tiles.
__global__ void batch_maps_kernel(const SampleRow* __restrict__ t, int S, int64_t n_pad, int64_t n_total,
                                  uint32_t* __restrict__ row_map, uint32_t* __restrict__ row_lo,
                                  uint32_t* __restrict__ row_hi, uint2* __restrict__ range,
                                  uint32_t* __restrict__ counts) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_pad) {
        const SampleRow r = t[sample_of(t, S, (uint32_t)i, true)];
        const uint32_t o = (uint32_t)i - r.start;
        row_map[i] = o < r.n ? r.off + o : 0xffffffffu;
        if ((i & 255) == 0) {
            const uint32_t t0 = r.start / 256, t1 = (r.start + (r.n + 255) / 256 * 256) / 256;
            range[i / 256] = make_uint2(t0, t1);
            counts[i / 256] = t1 - t0;
        }
    }
    if (i < n_total) {
        const SampleRow r = t[sample_of(t, S, (uint32_t)i, false)];
        row_lo[i] = r.off;
        row_hi[i] = r.off + r.n;
    }
}

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

// Sample-local neighbour ids -> batch-global ids (the sample's first row added).
__global__ void batch_global_ids_kernel(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ row_lo,
                                        int64_t n_total, int k, uint32_t* __restrict__ gidx) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_total * k) return;
    gidx[s] = idx[s] + row_lo[s / k];
}

// Column ids of the batch's CSR back to sample-local ids.
__global__ void batch_local_cols_kernel(const uint32_t* __restrict__ indptr, const uint32_t* __restrict__ row_lo,
                                        int64_t n_total, uint32_t* __restrict__ cols) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_total) return;
    const uint32_t lo = row_lo[i];
    for (uint32_t p = indptr[i], e = indptr[i + 1]; p < e; ++p) cols[p] -= lo;
}

}  // namespace

// Enqueues the batch solve on ctx->stream.  No allocation once the
// workspace has grown to this batch's size and nothing that synchronises,
// so a second call with the same arguments can be captured in a graph.
// With `csr` non-null the sequence ends with every sample's connectivities
// in it (sample-local columns, rows in input order).  `topk_width` is the
// sweep's register top-k width (KnnPlan::topk_width).
int32_t batch_enqueue(scrust_context* ctx, const float* x, const void* table, uint32_t S, int64_t n_total,
                      int64_t n_pad, int d, int k, const scrust_knn_options& o, uint32_t* out_idx, float* out_dist,
                      scrust_status* st, CsrBuffers* csr = nullptr, int topk_width = 0) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int items = (int)(n_pad / 256);
    const bool bf16 = o.precision == SCRUST_PRECISION_BF16;
    const bool cosine = o.metric == SCRUST_METRIC_COSINE;
    const float* xwork = x;
    double* norm64 = nullptr;
    if (cosine) {
        float* xn = (float*)ws_get(ctx, SLOT_XWORK, sizeof(float) * (size_t)n_total * d, &e);
        norm64 = (double*)ws_get(ctx, SLOT_NORM64, sizeof(double) * (size_t)n_total, &e);
        if (!xn || !norm64) return cuda_fail(st, e, "workspace");
        if ((e = launch_normalise_rows(x, n_total, d, xn, norm64, ctx->d_err, s)) != cudaSuccess)
            return cuda_fail(st, e, "normalise");
        ctx->launches += 1;
        xwork = xn;
    }
    // Maps.
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t r = off;
        off = align_up(off + bytes);
        return r;
    };
    const size_t o_map = take(4 * (size_t)n_pad), o_lo = take(4 * (size_t)n_total), o_hi = take(4 * (size_t)n_total),
                 o_rng = take(8 * (size_t)items), o_cnt = take(4 * (size_t)items), o_ord = take(4 * (size_t)items),
                 o_ws = take(work_order_scratch(items)), o_th = take(8 * (size_t)n_pad);
    char* base = (char*)ws_get(ctx, SLOT_BATCH, off, &e);
    if (!base) return cuda_fail(st, e, "batch: workspace");
    uint32_t* row_map = (uint32_t*)(base + o_map);
    uint32_t* row_lo = (uint32_t*)(base + o_lo);
    uint32_t* row_hi = (uint32_t*)(base + o_hi);
    uint2* range = (uint2*)(base + o_rng);
    uint32_t* counts = (uint32_t*)(base + o_cnt);
    uint32_t* order = (uint32_t*)(base + o_ord);
    float* theta = (float*)(base + o_th);
    const int64_t span = std::max(n_pad, n_total);
    batch_maps_kernel<<<(unsigned)((span + 255) / 256), 256, 0, s>>>((const SampleRow*)table, (int)S, n_pad, n_total,
                                                                     row_map, row_lo, row_hi, range, counts);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "batch: maps");
    if ((e = sort_by_work(ctx, counts, items, base + o_ws, order)) != cudaSuccess)
        return cuda_fail(st, e, "batch: work order");
    ctx->launches += 1;

    // Centring over all samples (exact for every sample: the bound uses the
    // actual quantised rows), norms, operands in the padded layout, bounds.
    const int mean_blocks = (int)((n_total + 2047) / 2048);
    double* means = (double*)ws_get(ctx, SLOT_MEANS, sizeof(double) * ((size_t)d * (mean_blocks + 1)), &e);
    float* norm2 = (float*)ws_get(ctx, SLOT_NORM2, sizeof(float) * (size_t)n_pad, &e);
    float* cnorm = (float*)ws_get(ctx, SLOT_CNORM, sizeof(float) * (size_t)n_pad, &e);
    float* margin = (float*)ws_get(ctx, SLOT_MARGIN, sizeof(float) * (size_t)n_pad + 64, &e);
    void* A16 = ws_get(ctx, SLOT_A16, (size_t)n_pad * 64 * 2, &e);
    void* B16 = ws_get(ctx, SLOT_B16, (size_t)n_pad * 64 * 2, &e);
    float* rb = (float*)ws_get(ctx, SLOT_QERR, sizeof(float) * 4 * (size_t)n_pad, &e);
    if (!means || !norm2 || !cnorm || !margin || !A16 || !B16 || !rb) return cuda_fail(st, e, "workspace");
    uint32_t* max_bits = (uint32_t*)(margin + n_pad);
    float *bA = rb, *beps = rb + n_pad, *bdelta = rb + 2 * n_pad, *beps2 = rb + 3 * n_pad;
    if ((e = cudaMemsetAsync(max_bits, 0, 4 * sizeof(uint32_t), s)) != cudaSuccess ||
        (e = launch_column_means_centre(xwork, n_total, d, means, means + d, s)) != cudaSuccess ||
        (e = launch_max_centred_norm(xwork, n_total, d, means, max_bits, ctx->sm_count, s)) != cudaSuccess ||
        (e = launch_tensor_operands(xwork, n_pad, n_pad, d, means, max_bits, cosine, bf16, row_map, A16, B16, bA, beps,
                                    max_bits + 1, max_bits + 2, s)) != cudaSuccess ||
        (e = launch_tensor_bounds(n_pad, bA, beps, max_bits + 1, max_bits + 2, bdelta, beps2, s)) != cudaSuccess)
        return cuda_fail(st, e, "batch: prep");
    ctx->launches += 5;

    // One sweep over every sample's block-diagonal tiles.
    KnnPlan plan;
    plan.nq = plan.nr = n_pad;
    plan.d = d;
    plan.k = k;
    plan.self = true;
    plan.form = SCRUST_FORM_TENSOR;
    plan.metric = o.metric;
    plan.mode = SCRUST_MODE_EXACT;
    plan.precision = o.precision;
    plan.topk_width = topk_width;
    Lists lists;
    lists.cap = std::max<int>(o.list_capacity ? (int)o.list_capacity : 64, k + 32);
    lists.cap = (lists.cap + 3) / 4 * 4;
    lists.ctot = lists.cap + 128;
    lists.segments = 2;
    if (lists.ctot > 512) return fail(st, SCRUST_INVALID_PARAMETER, "list_capacity must be at most 384, got %d", lists.cap);
    int32_t rc = alloc_lists(ctx, n_pad, &lists, st);
    if (rc) return rc;
    plan.cap = lists.cap;
    plan.ctot = lists.ctot;
    plan.segments = lists.segments;
    TileLists tl;
    tl.range = range;
    tl.row_map = row_map;
    tl.order = order;
    mark(ctx, PH_PREP);
    if ((e = launch_tensor_candidates(ctx, plan, A16, n_pad, B16, n_pad, bA, bdelta, beps2, lists, bf16, &tl, false,
                                      theta, nullptr, sweep_stats(ctx))) != cudaSuccess)
        return cuda_fail(st, e, "batch: knn_candidates_tc");
    ctx->launches += 1;
    mark(ctx, PH_CAND);

    // Exact rerank over the rows in the padded layout; ids relative to each
    // sample's first row.
    float* xs = (float*)ws_get(ctx, SLOT_XSORTED, sizeof(float) * (size_t)n_pad * padded_row_floats(d), &e);
    if (!xs) return cuda_fail(st, e, "workspace");
    if ((e = launch_gather_rows(xwork, row_map, n_pad, d, padded_row_floats(d), xs, s)) != cudaSuccess)
        return cuda_fail(st, e, "batch: gather rows");
    RowBounds bounds;
    bounds.A = bA;
    bounds.delta = bdelta;
    bounds.eps2 = beps2;
    if ((e = launch_rerank(ctx, plan, xwork, xwork, norm2, norm2, norm64, norm64, x, x, bounds, lists, row_map, xs, theta,
                           out_idx, out_dist, row_lo, row_hi, nullptr, padded_row_floats(d))) != cudaSuccess)
        return cuda_fail(st, e, "batch: knn_rerank");
    ctx->launches += 1;  // the row gather (the rerank counts its own)
    mark(ctx, PH_RERANK);
    if (!csr) return ok(st);
    uint32_t* gidx = (uint32_t*)ws_get(ctx, SLOT_BATCH_GIDX, sizeof(uint32_t) * (size_t)n_total * k, &e);
    if (!gidx) return cuda_fail(st, e, "batch: workspace");
    batch_global_ids_kernel<<<(unsigned)((n_total * k + 255) / 256), 256, 0, s>>>(out_idx, row_lo, n_total, k, gidx);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "batch: global ids");
    int32_t rc2 = run_connectivities(ctx, gidx, out_dist, n_total, k, false, csr, st, true);
    if (rc2) return rc2;
    batch_local_cols_kernel<<<(unsigned)((n_total + 255) / 256), 256, 0, s>>>(csr->indptr, row_lo, n_total,
                                                                              csr->indices);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "batch: local columns");
    ctx->launches += 2;
    mark(ctx, PH_CONN);
    return ok(st);
}

namespace {

int32_t check_batch(const uint64_t* offsets, uint32_t S, uint64_t d, uint32_t k, const scrust_knn_options* opt,
                    std::vector<SampleRow>* rows, int64_t* n_total, int64_t* n_pad, scrust_status* st) {
    if (!offsets || S == 0) return fail(st, SCRUST_SHAPE, "expected at least one sample");
    if (d == 0 || d > 61)
        return fail(st, SCRUST_SHAPE, "expected 1 to 61 dimensions for a batched solve, got %llu", (unsigned long long)d);
    if (k == 0) return fail(st, SCRUST_INVALID_PARAMETER, "k must be at least 1, got 0");
    if (k > 128) return fail(st, SCRUST_INVALID_PARAMETER, "k must be within the supported maximum of 128, got %u", k);
    if (offsets[0] != 0) return fail(st, SCRUST_SHAPE, "expected row offsets starting at 0");
    if (opt && opt->mode != SCRUST_MODE_EXACT)
        return fail(st, SCRUST_INVALID_PARAMETER, "batched solves run in exact mode only");
    uint64_t pos = 0;
    rows->resize(S);
    for (uint32_t i = 0; i < S; ++i) {
        if (offsets[i + 1] < offsets[i]) return fail(st, SCRUST_SHAPE, "expected non-decreasing row offsets");
        const uint64_t n = offsets[i + 1] - offsets[i];
        if (n == 0) return fail(st, SCRUST_SHAPE, "expected every sample to hold at least one cell, sample %u is empty", i);
        if ((uint64_t)k >= n)
            return fail(st, SCRUST_INVALID_PARAMETER,
                        "k must be smaller than the number of cells of every sample, got %u for a sample of %llu", k,
                        (unsigned long long)n);
        (*rows)[i] = SampleRow{(uint32_t)pos, (uint32_t)offsets[i], (uint32_t)n, 0u};
        pos += (n + 255) / 256 * 256;
        if (pos >= 0xffffff00ull) return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 cells in a batch");
    }
    *n_total = (int64_t)offsets[S];
    *n_pad = (int64_t)pos;
    return SCRUST_OK;
}

}  // namespace

}  // namespace scrust

using namespace scrust;

extern "C" {

int32_t scrust_cuda_knn_batch_device(scrust_context* ctx, const float* x, const uint64_t* row_offsets,
                                     uint32_t n_samples, uint64_t d, uint32_t k, const scrust_knn_options* opt,
                                     uint32_t* out_idx, float* out_dist, scrust_status* st) {
    std::vector<SampleRow> rows;
    int64_t n_total = 0, n_pad = 0;
    int32_t rc = check_batch(row_offsets, n_samples, d, k, opt, &rows, &n_total, &n_pad, st);
    if (rc) return rc;
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist) return fail(st, SCRUST_SHAPE, "expected non-null device pointers");
    scrust_knn_options o;
    scrust_knn_options_default(&o);
    if (opt) o = *opt;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    void* table = ws_get(ctx, SLOT_BATCH_TABLE, sizeof(SampleRow) * rows.size(), &e);
    if (!table) return cuda_fail(st, e, "workspace");
    // The table is small; a synchronous copy keeps the host vector's lifetime simple.
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpy(table, rows.data(), sizeof(SampleRow) * rows.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(st, e, "batch: table upload");
    mark(ctx, PH_START);
    return batch_enqueue(ctx, x, table, n_samples, n_total, n_pad, (int)d, (int)k, o, out_idx, out_dist, st);
}

int32_t scrust_cuda_knn_batch(scrust_context* ctx, const float* x, const uint64_t* row_offsets, uint32_t n_samples,
                              uint64_t d, uint32_t k, const scrust_knn_options* opt, uint32_t* out_idx, float* out_dist,
                              scrust_status* st) {
    std::vector<SampleRow> rows;
    int64_t n_total = 0, n_pad = 0;
    int32_t rc = check_batch(row_offsets, n_samples, d, k, opt, &rows, &n_total, &n_pad, st);
    if (rc) return rc;
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist) return fail(st, SCRUST_SHAPE, "expected non-null host pointers");
    float* dx;
    uint32_t* di;
    float* dd;
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        DeviceGuard device_guard(ctx->device);
        cudaError_t e;
        dx = (float*)ws_get(ctx, SLOT_HOST_IN, sizeof(float) * (size_t)n_total * d, &e);
        di = (uint32_t*)ws_get(ctx, SLOT_HOST_IDX, sizeof(uint32_t) * (size_t)n_total * k, &e);
        dd = (float*)ws_get(ctx, SLOT_HOST_DIST, sizeof(float) * (size_t)n_total * k, &e);
        if (!dx || !di || !dd) return cuda_fail(st, e, "workspace");
        if ((e = cudaMemcpyAsync(dx, x, sizeof(float) * (size_t)n_total * d, cudaMemcpyHostToDevice, ctx->stream)) !=
            cudaSuccess)
            return cuda_fail(st, e, "upload");
    }
    if ((rc = scrust_cuda_knn_batch_device(ctx, dx, row_offsets, n_samples, d, k, opt, di, dd, st))) return rc;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(out_idx, di, sizeof(uint32_t) * (size_t)n_total * k, cudaMemcpyDeviceToHost,
                             ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_dist, dd, sizeof(float) * (size_t)n_total * k, cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess)
        return cuda_fail(st, e, "download");
    return collect_device_errors(ctx, st);
}

int32_t scrust_cuda_neighbors_graph_batch(scrust_context* ctx, const float* x, const uint64_t* row_offsets,
                                          uint32_t n_samples, uint64_t d, uint32_t k,
                                          const scrust_knn_options* opt, uint32_t* out_idx, float* out_dist,
                                          scrust_csr** conn, scrust_status* st) {
    std::vector<SampleRow> rows;
    int64_t n_total = 0, n_pad = 0;
    int32_t rc = check_batch(row_offsets, n_samples, d, k, opt, &rows, &n_total, &n_pad, st);
    if (rc) return rc;
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist || !conn) return fail(st, SCRUST_SHAPE, "expected non-null host pointers");
    if ((uint64_t)n_total * k * 2 >= 0xffffffffull)
        return fail(st, SCRUST_SHAPE, "expected fewer than 2^31 graph entries in a batch");
    scrust_knn_options o;
    scrust_knn_options_default(&o);
    if (opt) o = *opt;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    float* dx = (float*)ws_get(ctx, SLOT_HOST_IN, sizeof(float) * (size_t)n_total * d, &e);
    uint32_t* di = (uint32_t*)ws_get(ctx, SLOT_HOST_IDX, sizeof(uint32_t) * (size_t)n_total * k, &e);
    float* dd = (float*)ws_get(ctx, SLOT_HOST_DIST, sizeof(float) * (size_t)n_total * k, &e);
    void* table = ws_get(ctx, SLOT_BATCH_TABLE, sizeof(SampleRow) * rows.size(), &e);
    if (!dx || !di || !dd || !table) return cuda_fail(st, e, "workspace");
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpy(table, rows.data(), sizeof(SampleRow) * rows.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dx, x, sizeof(float) * (size_t)n_total * d, cudaMemcpyHostToDevice, ctx->stream)) !=
            cudaSuccess)
        return cuda_fail(st, e, "upload");
    CsrBuffers b;
    if ((rc = csr_take(ctx, (uint64_t)n_total, 2 * (uint64_t)n_total * k, &b, st))) return rc;
    mark(ctx, PH_START);
    rc = batch_enqueue(ctx, dx, table, n_samples, n_total, n_pad, (int)d, (int)k, o, di, dd, st, &b);
    if (rc == SCRUST_OK &&
        ((e = cudaMemcpyAsync(out_idx, di, sizeof(uint32_t) * (size_t)n_total * k, cudaMemcpyDeviceToHost,
                              ctx->stream)) != cudaSuccess ||
         (e = cudaMemcpyAsync(out_dist, dd, sizeof(float) * (size_t)n_total * k, cudaMemcpyDeviceToHost,
                              ctx->stream)) != cudaSuccess))
        rc = cuda_fail(st, e, "download");
    if (rc == SCRUST_OK) rc = csr_download(ctx, b, (uint64_t)n_total, (uint64_t)n_total, conn, st);
    csr_give(ctx, b);
    if (rc) return rc;
    if ((rc = collect_device_errors(ctx, st))) {
        scrust_csr_free(*conn);
        *conn = nullptr;
    }
    return rc;
}

}  // extern "C"

namespace {

scrust_batch_plan* plan_create(scrust_context* ctx, const uint64_t* row_offsets, uint32_t n_samples, uint64_t d,
                               uint32_t k, const scrust_knn_options* opt, const float* x, uint32_t* out_idx,
                               float* out_dist, bool graphs, scrust_status* st) {
    std::vector<SampleRow> rows;
    int64_t n_total = 0, n_pad = 0;
    if (check_batch(row_offsets, n_samples, d, k, opt, &rows, &n_total, &n_pad, st)) return nullptr;
    if (!ctx) {
        fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
        return nullptr;
    }
    if (!x || !out_idx || !out_dist) {
        fail(st, SCRUST_SHAPE, "expected non-null device pointers");
        return nullptr;
    }
    scrust_batch_plan* p = new (std::nothrow) scrust_batch_plan;
    if (!p) {
        fail(st, SCRUST_OOM, "host allocation failed");
        return nullptr;
    }
    p->ctx = ctx;
    p->n_samples = n_samples;
    p->n_total = (uint64_t)n_total;
    p->d = d;
    p->k = k;
    scrust_knn_options_default(&p->opts);
    if (opt) p->opts = *opt;
    p->x = x;
    p->out_idx = out_idx;
    p->out_dist = out_dist;
    p->graphs = graphs;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e = cudaMalloc(&p->table, sizeof(SampleRow) * rows.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(p->table, rows.data(), sizeof(SampleRow) * rows.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && graphs) {
        p->csr.rows_cap = (size_t)n_total;
        p->csr.nnz_cap = 2 * (size_t)n_total * k;
        e = cudaMalloc(&p->csr.indptr, sizeof(uint32_t) * ((size_t)n_total + 1));
        if (e == cudaSuccess) e = cudaMalloc(&p->csr.indices, sizeof(uint32_t) * p->csr.nnz_cap);
        if (e == cudaSuccess) e = cudaMalloc(&p->csr.values, sizeof(float) * p->csr.nnz_cap);
    }
    auto release = [&]() {
        cudaFree(p->table);
        cudaFree(p->csr.indptr);
        cudaFree(p->csr.indices);
        cudaFree(p->csr.values);
        delete p;
    };
    if (e != cudaSuccess) {
        cuda_fail(st, e, "batch plan: allocation");
        release();
        return nullptr;
    }
    CsrBuffers* csr = graphs ? &p->csr : nullptr;
    // Autotune the candidate over-provisioning (list capacity) and the
    // register top-k width unless the caller fixed the capacity, and the
    // operand precision, timing each candidate on this batch; then capture
    // the winner.
    const bool tune_cap = p->opts.list_capacity == 0;
    struct Cand {
        scrust_knn_options o;
        int width;
    };
    std::vector<Cand> cands;
    const uint32_t caps[3] = {64, 128, 256};
    std::vector<int> widths = {0};
    if (k > 1 && k <= 16) widths.push_back(32);
    if (k > 1 && k <= 32) widths.push_back(-1);
    for (int c = 0; c < (tune_cap ? 3 : 1); ++c)
        for (int w : widths)
            for (int prec = 0; prec < 2; ++prec) {
                scrust_knn_options o = p->opts;
                if (tune_cap) o.list_capacity = caps[c];
                o.precision = prec;
                cands.push_back(Cand{o, w});
            }
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best = 1e30f;
    Cand chosen = cands[0];
    int32_t rc = SCRUST_OK;
    for (const auto& c : cands) {
        for (int rep = 0; rep < 2 && rc == SCRUST_OK; ++rep) {  // first run sizes the workspace
            cudaEventRecord(t0, ctx->stream);
            rc = batch_enqueue(ctx, x, p->table, n_samples, n_total, n_pad, (int)d, (int)k, c.o, out_idx, out_dist, st,
                               csr, c.width);
            cudaEventRecord(t1, ctx->stream);
        }
        if (rc) break;
        float ms = 0.f;
        if ((e = cudaEventSynchronize(t1)) != cudaSuccess || (e = cudaEventElapsedTime(&ms, t0, t1)) != cudaSuccess) {
            rc = cuda_fail(st, e, "batch plan: autotune");
            break;
        }
        if (ms < best) {
            best = ms;
            chosen = c;
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (rc == SCRUST_OK) {
        // Size the workspace for the chosen options, then capture.
        rc = batch_enqueue(ctx, x, p->table, n_samples, n_total, n_pad, (int)d, (int)k, chosen.o, out_idx, out_dist,
                           st, csr, chosen.width);
        if (rc == SCRUST_OK && (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
            rc = cuda_fail(st, e, "batch plan: synchronise");
    }
    if (rc == SCRUST_OK) {
        const bool timing = ctx->timing;
        ctx->timing = false;
        e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = batch_enqueue(ctx, x, p->table, n_samples, n_total, n_pad, (int)d, (int)k, chosen.o, out_idx,
                               out_dist, st, csr, chosen.width);
            const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &p->graph);
            if (rc == SCRUST_OK && e2 != cudaSuccess) rc = cuda_fail(st, e2, "batch plan: capture");
        } else {
            rc = cuda_fail(st, e, "batch plan: capture");
        }
        ctx->timing = timing;
        if (rc == SCRUST_OK && (e = cudaGraphInstantiate(&p->exec, p->graph, 0)) != cudaSuccess)
            rc = cuda_fail(st, e, "batch plan: instantiate");
    }
    if (rc != SCRUST_OK) {
        cudaGetLastError();
        if (p->exec) cudaGraphExecDestroy(p->exec);
        if (p->graph) cudaGraphDestroy(p->graph);
        release();
        return nullptr;
    }
    p->opts = chosen.o;
    p->topk_width = chosen.width;
    p->tuned_ms = best;
    ok(st);
    return p;
}

}  // namespace

extern "C" {

scrust_batch_plan* scrust_cuda_batch_plan_create(scrust_context* ctx, const uint64_t* row_offsets, uint32_t n_samples,
                                                 uint64_t d, uint32_t k, const scrust_knn_options* opt,
                                                 const float* x, uint32_t* out_idx, float* out_dist,
                                                 scrust_status* st) {
    return plan_create(ctx, row_offsets, n_samples, d, k, opt, x, out_idx, out_dist, false, st);
}

scrust_batch_plan* scrust_cuda_batch_plan_create_graphs(scrust_context* ctx, const uint64_t* row_offsets,
                                                        uint32_t n_samples, uint64_t d, uint32_t k,
                                                        const scrust_knn_options* opt, const float* x,
                                                        uint32_t* out_idx, float* out_dist, scrust_status* st) {
    if (row_offsets && n_samples && row_offsets[n_samples] * (uint64_t)k * 2 >= 0xffffffffull) {
        fail(st, SCRUST_SHAPE, "expected fewer than 2^31 graph entries in a batch");
        return nullptr;
    }
    return plan_create(ctx, row_offsets, n_samples, d, k, opt, x, out_idx, out_dist, true, st);
}

int32_t scrust_cuda_batch_plan_graph(const scrust_batch_plan* p, const uint32_t** indptr, const uint32_t** indices,
                                     const float** values) {
    if (!p || !p->graphs) return 0;
    if (indptr) *indptr = p->csr.indptr;
    if (indices) *indices = p->csr.indices;
    if (values) *values = p->csr.values;
    return 1;
}

int32_t scrust_cuda_batch_plan_topk_width(const scrust_batch_plan* p) {
    if (!p) return -1;
    const int w = p->topk_width;
    if (w < 0 || p->k > 32) return 0;
    if (w == 32 || p->k > 16) return 32;
    return p->k == 1 ? 1 : 16;
}

int32_t scrust_cuda_batch_plan_launch(scrust_batch_plan* p, scrust_status* st) {
    if (!p) return fail(st, SCRUST_SHAPE, "expected a batch plan");
    std::lock_guard<std::mutex> lock(p->ctx->mu);
    DeviceGuard device_guard(p->ctx->device);
    const cudaError_t e = cudaGraphLaunch(p->exec, p->ctx->stream);
    if (e != cudaSuccess) return cuda_fail(st, e, "batch plan: launch");
    p->ctx->launches += 1;
    return ok(st);
}

int32_t scrust_cuda_batch_plan_choice(const scrust_batch_plan* p, uint32_t* list_capacity, int32_t* precision,
                                      float* tuned_ms) {
    if (!p) return 0;
    if (list_capacity) *list_capacity = p->opts.list_capacity;
    if (precision) *precision = p->opts.precision;
    if (tuned_ms) *tuned_ms = p->tuned_ms;
    return 1;
}

void scrust_cuda_batch_plan_destroy(scrust_batch_plan* p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lock(p->ctx->mu);
        DeviceGuard device_guard(p->ctx->device);
        cudaStreamSynchronize(p->ctx->stream);
        if (p->exec) cudaGraphExecDestroy(p->exec);
        if (p->graph) cudaGraphDestroy(p->graph);
        cudaFree(p->table);
        cudaFree(p->csr.indptr);
        cudaFree(p->csr.indices);
        cudaFree(p->csr.values);
    }
    delete p;
}

}  // extern "C"
