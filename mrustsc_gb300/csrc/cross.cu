// cross.cu -- query-versus-reference solves: the k nearest rows of a
// reference set for each query row, exact.  Used by the query service (the
// reference is a resident atlas) and by row-range solves, in which the
// queries are a block of the reference's own rows (one shard of a graph
// build spread over several GPUs), each excluding itself.
//
// The reference fixes the centring means and the operand scale; its
// quantisation radius and largest |b_hat| enter every query row's bound.  The
// queries sweep every reference tile (no ordering), split into column
// segments so that small query sets still fill the GPU; the segments of a
// row share its threshold through HBM, and the rerank needs no selection.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

int32_t reference_prepare(scrust_context* ctx, const float* x, int64_t n, int d, bool bf16, Reference* out,
                          scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int64_t n_pad = (int64_t)round_up((size_t)n, 256);
    const int mean_blocks = (int)((n + 2047) / 2048);
    double* means = (double*)ws_get(ctx, SLOT_MEANS, sizeof(double) * ((size_t)d * (mean_blocks + 1)), &e);
    float* terms = (float*)ws_get(ctx, SLOT_QERR, sizeof(float) * 4 * (size_t)n_pad + 64, &e);
    void* A16 = ws_get(ctx, SLOT_A16, (size_t)n_pad * 128, &e);
    void* B16 = ws_get(ctx, SLOT_B16, (size_t)n_pad * 128, &e);
    if (!means || !terms || !A16 || !B16) return cuda_fail(st, e, "reference: workspace");
    uint32_t* words = (uint32_t*)(terms + 4 * n_pad);
    if ((e = cudaMemsetAsync(words, 0, 16, s)) != cudaSuccess ||
        (e = launch_column_means_centre(x, n, d, means, means + d, s)) != cudaSuccess ||
        (e = launch_max_centred_norm(x, n, d, means, words, ctx->sm_count, s)) != cudaSuccess ||
        (e = launch_tensor_operands(x, n, n_pad, d, means, words, false, bf16, nullptr, A16, B16, terms + 2 * n_pad,
                                    terms + 3 * n_pad, words + 1, words + 2, s)) != cudaSuccess)
        return cuda_fail(st, e, "reference: operands");
    ctx->launches += 4;
    out->rows = x;
    out->n = n;
    out->n_pad = n_pad;
    out->d = d;
    out->means = means;
    out->words = words;
    out->B16 = B16;
    out->bf16 = bf16;
    return SCRUST_OK;
}

int32_t cross_knn_enqueue(scrust_context* ctx, const Reference& ref, const float* dq, int64_t q, int k,
                          int64_t self_offset, uint32_t* d_idx, float* d_dist, scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int d = ref.d;
    const int64_t q_pad = (int64_t)round_up((size_t)q, 256);
    // The query operands go to their own slots: the reference's B (and, for
    // a resident atlas, nothing else) must stay intact.
    void* A16 = ws_get(ctx, SLOT_XWORK, (size_t)q_pad * 128, &e);
    void* B16 = ws_get(ctx, SLOT_QSCRATCH, (size_t)q_pad * 128, &e);
    float* rb = (float*)ws_get(ctx, SLOT_QTERMS, sizeof(float) * 4 * (size_t)q_pad + 64, &e);
    if (!A16 || !B16 || !rb) return cuda_fail(st, e, "cross: workspace");
    float *bA = rb, *eps = rb + q_pad, *bdelta = rb + 2 * q_pad, *beps2 = rb + 3 * q_pad;
    uint32_t* scratch_words = (uint32_t*)(rb + 4 * q_pad);
    if ((e = launch_tensor_operands(dq, q, q_pad, d, ref.means, ref.words, false, ref.bf16, nullptr, A16, B16, bA, eps,
                                    scratch_words, scratch_words + 1, s)) != cudaSuccess ||
        (e = launch_tensor_bounds(q, bA, eps, ref.words + 1, ref.words + 2, bdelta, beps2, s)) != cudaSuccess)
        return cuda_fail(st, e, "cross: query operands");
    const int items = (int)(q_pad / 256), col_tiles = (int)(ref.n_pad / 256);
    int csegs = std::max(1, std::min((2 * ctx->sm_count + items - 1) / items, std::min(col_tiles, 16)));
    const int per = (col_tiles + csegs - 1) / csegs;
    csegs = (col_tiles + per - 1) / per;
    KnnPlan plan;
    plan.nq = q;
    plan.nr = ref.n;
    plan.d = d;
    plan.k = k;
    plan.self = self_offset >= 0;
    plan.self_offset = self_offset >= 0 ? self_offset : 0;
    plan.form = SCRUST_FORM_TENSOR;
    plan.precision = ref.bf16 ? SCRUST_PRECISION_BF16 : SCRUST_PRECISION_FP16;
    Lists lists;
    lists.cap = std::max(64, (2 * k + 32 + 31) / 32 * 32);
    lists.ctot = lists.cap + 128;
    lists.segments = 2 * csegs;
    int32_t rc = alloc_lists(ctx, q_pad, &lists, st);
    if (rc) return rc;
    plan.cap = lists.cap;
    plan.ctot = lists.ctot;
    plan.segments = lists.segments;
    float* theta = (float*)ws_get(ctx, SLOT_THETA, sizeof(float) * (size_t)q_pad * lists.segments, &e);
    uint32_t* row_theta = (uint32_t*)ws_get(ctx, SLOT_ROWTHETA, sizeof(uint32_t) * (size_t)q_pad, &e);
    if (!theta || !row_theta) return cuda_fail(st, e, "cross: workspace");
    if ((e = cudaMemsetAsync(row_theta, 0xff, sizeof(uint32_t) * (size_t)q_pad, s)) != cudaSuccess)
        return cuda_fail(st, e, "cross: memset");
    TileLists shared;  // the column segments of a row share its threshold
    shared.row_theta = row_theta;
    if ((e = launch_tensor_candidates(ctx, plan, A16, q_pad, ref.B16, ref.n_pad, bA, bdelta, beps2, lists, ref.bf16,
                                      &shared, false, theta, nullptr, nullptr)) != cudaSuccess)
        return cuda_fail(st, e, "cross: knn_candidates_tc");
    ctx->launches += 3;
    RowBounds bounds;
    bounds.A = bA;
    bounds.delta = bdelta;
    bounds.eps2 = beps2;
    if ((e = launch_rerank(ctx, plan, dq, ref.rows, nullptr, nullptr, nullptr, nullptr, dq, ref.rows, bounds, lists,
                           nullptr, dq, theta, d_idx, d_dist, nullptr, nullptr, ref.rows)) != cudaSuccess)
        return cuda_fail(st, e, "cross: knn_rerank");
    return SCRUST_OK;
}

}  // namespace scrust

using namespace scrust;

extern "C" {

int32_t scrust_cuda_knn_rows_device(scrust_context* ctx, const float* x, uint64_t n, uint64_t d, uint32_t k,
                                    uint64_t row_begin, uint64_t row_end, const scrust_knn_options* opt,
                                    uint32_t* out_idx, float* out_dist, scrust_status* st) {
    if (n == 0 || d == 0)
        return fail(st, SCRUST_SHAPE, "expected a non-empty (cells, dimensions) embedding, got %llu x %llu",
                    (unsigned long long)n, (unsigned long long)d);
    if (d > 61) return fail(st, SCRUST_SHAPE, "expected at most 61 dimensions for a row-range solve, got %llu",
                            (unsigned long long)d);
    if (k == 0 || k > 128 || (uint64_t)k >= n)
        return fail(st, SCRUST_INVALID_PARAMETER, "k must be between 1 and min(128, cells - 1), got %u", k);
    if (row_begin >= row_end || row_end > n)
        return fail(st, SCRUST_SHAPE, "expected 0 <= row_begin < row_end <= %llu, got [%llu, %llu)",
                    (unsigned long long)n, (unsigned long long)row_begin, (unsigned long long)row_end);
    if (n >= 0xffffff00ull) return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 cells");
    if (opt && (opt->mode != SCRUST_MODE_EXACT || opt->metric != SCRUST_METRIC_EUCLIDEAN))
        return fail(st, SCRUST_INVALID_PARAMETER, "row-range solves are exact Euclidean");
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist) return fail(st, SCRUST_SHAPE, "expected non-null device pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    const bool bf16 = opt && opt->precision == SCRUST_PRECISION_BF16;
    Reference ref;
    int32_t rc = reference_prepare(ctx, x, (int64_t)n, (int)d, bf16, &ref, st);
    if (rc) return rc;
    mark(ctx, PH_START);
    rc = cross_knn_enqueue(ctx, ref, x + row_begin * d, (int64_t)(row_end - row_begin), (int)k, (int64_t)row_begin,
                           out_idx, out_dist, st);
    if (rc) return rc;
    return ok(st);
}

}  // extern "C"
