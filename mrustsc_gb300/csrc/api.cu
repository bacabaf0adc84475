// api.cu -- the C ABI (include/scrust_cuda.h): argument checks that mirror
// the reference, the per-device context and its workspace arena, and the
// orchestration of prep -> candidates -> exact rerank -> connectivities on
// the context's stream.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <utility>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace scrust {

int32_t fail(scrust_status* st, int32_t code, const char* fmt, ...) {
    if (st) {
        st->code = code;
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(st->message, sizeof(st->message), fmt, ap);
        va_end(ap);
    }
    return code;
}

int32_t ok(scrust_status* st) {
    if (st) {
        st->code = SCRUST_OK;
        st->message[0] = '\0';
    }
    return SCRUST_OK;
}

int32_t cuda_fail(scrust_status* st, cudaError_t e, const char* what) {
    const int32_t code = e == cudaErrorMemoryAllocation ? SCRUST_OOM : SCRUST_KERNEL;
    return fail(st, code, "CUDA kernel %s: %s", what, cudaGetErrorString(e));
}

void* ws_get(scrust_context* ctx, Slot slot, size_t bytes, cudaError_t* err) {
    Workspace& ws = ctx->ws;
    if (bytes == 0) bytes = 16;
    if (ws.ptr[slot] && ws.bytes[slot] >= bytes) return ws.ptr[slot];
    // Queued work may still read the old buffer.
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess && ws.ptr[slot]) e = cudaFree(ws.ptr[slot]);
    ws.ptr[slot] = nullptr;
    ws.bytes[slot] = 0;
    if (e == cudaSuccess) {
        size_t want = bytes + bytes / 8;
        want = (want + (2u << 20) - 1) & ~(size_t)((2u << 20) - 1);
        void* p = nullptr;
        e = cudaMalloc(&p, want);
        if (e == cudaSuccess) {
            ws.ptr[slot] = p;
            ws.bytes[slot] = want;
        } else {
            cudaGetLastError();
        }
    }
    if (err) *err = e;
    return ws.ptr[slot];
}

cudaError_t set_smem_limit(scrust_context* ctx, const void* func, int bytes) {
    for (auto& pr : ctx->smem_limits)
        if (pr.first == func) {
            if (pr.second >= bytes) return cudaSuccess;
            const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e == cudaSuccess) pr.second = bytes;
            return e;
        }
    const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) ctx->smem_limits.emplace_back(func, bytes);
    return e;
}

cudaError_t set_smem_carveout(scrust_context* ctx, const void* func, int percent) {
    for (const void* f : ctx->carveouts)
        if (f == func) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
    if (e == cudaSuccess) ctx->carveouts.push_back(func);
    return e;
}

bool encode_2d(scrust_context* ctx, CUtensorMap* map, CUtensorMapDataType dtype, void* base,
               uint64_t inner, uint64_t outer, uint64_t row_bytes, uint32_t box_inner,
               uint32_t box_outer, CUtensorMapSwizzle swizzle) {
    if (!ctx->encode_tiled) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = ctx->encode_tiled(map, dtype, 2, base, dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

size_t plain_smem_bytes(int dp);

// The counter block of the next sweep launch, or null when statistics are off.
unsigned long long* sweep_stats(scrust_context* ctx) {
    if (!ctx->d_stats) return nullptr;
    const int slot = std::min(ctx->stats_launch, kStatSlots - 1);
    ctx->stats_launch++;
    return ctx->d_stats + kStatWords * slot;
}

void mark(scrust_context* ctx, Phase p) {
    if (!ctx->timing) return;
    if (!ctx->ev[p] && cudaEventCreate(&ctx->ev[p]) != cudaSuccess) return;
    if (p == PH_START)
        for (int i = 0; i < PH_COUNT; i++) ctx->ev_recorded[i] = false;
    if (cudaEventRecord(ctx->ev[p], ctx->stream) == cudaSuccess) ctx->ev_recorded[p] = true;
}

// Maps the device error block to a status, then clears it.
int32_t collect_device_errors(scrust_context* ctx, scrust_status* st) {
    int h[DERR_COUNT] = {0};
    cudaError_t e = cudaMemcpyAsync(h, ctx->d_err, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(st, e, "synchronize");
    bool any = false;
    for (int i = 0; i < DERR_COUNT; i++) any |= h[i] != 0;
    if (!any) return ok(st);
    cudaMemsetAsync(ctx->d_err, 0, sizeof(int) * DERR_COUNT, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (h[DERR_ZERO_ROW])
        return fail(st, SCRUST_SHAPE, "expected rows with a non-zero norm for the cosine metric, got an all-zero row");
    if (h[DERR_BAD_INDEX]) return fail(st, SCRUST_SHAPE, "expected neighbour ids below n, got an out-of-range neighbour id");
    if (h[DERR_TIMEOUT]) return fail(st, SCRUST_TIMEOUT, "CUDA kernel knn: a bounded device wait ran out");
    if (h[DERR_TIE_OVERFLOW])
        return fail(st, SCRUST_KERNEL,
                    "CUDA kernel knn_rerank: more than 4096 cells are equidistant from one cell within f32 resolution");
    return fail(st, SCRUST_KERNEL, "CUDA kernel knn_rerank: inconsistent candidate set");
}

namespace {

constexpr uint32_t kMaxK = 128;
constexpr int64_t kOrderMinRows = 1024;  // automatic ordering from this many rows

int32_t check_knn_args(uint64_t n, uint64_t d, uint32_t k, scrust_status* st) {
    if (n == 0 || d == 0)
        return fail(st, SCRUST_SHAPE, "expected a non-empty (cells, dimensions) embedding, got %llu x %llu",
                    (unsigned long long)n, (unsigned long long)d);
    if (k == 0) return fail(st, SCRUST_INVALID_PARAMETER, "k must be at least 1, got 0");
    if ((uint64_t)k >= n)
        return fail(st, SCRUST_INVALID_PARAMETER,
                    "k must be smaller than the number of cells, since a cell is not its own neighbour, got %u",
                    k);
    if (k > kMaxK)
        return fail(st, SCRUST_INVALID_PARAMETER, "k must be within the supported maximum of %u, got %u", kMaxK, k);
    if (n >= 0xffffffffull)
        return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 - 1 cells, got %llu", (unsigned long long)n);
    if (d > 65536) return fail(st, SCRUST_SHAPE, "expected at most 65536 dimensions, got %llu", (unsigned long long)d);
    return SCRUST_OK;
}

int32_t check_options(const scrust_knn_options* o, scrust_status* st) {
    if (!o) return SCRUST_OK;
    if (o->form != SCRUST_FORM_PLAIN && o->form != SCRUST_FORM_TENSOR && o->form != SCRUST_FORM_AUTO)
        return fail(st, SCRUST_INVALID_PARAMETER, "form must be plain, tensor or auto, got %d", o->form);
    if (o->metric != SCRUST_METRIC_EUCLIDEAN && o->metric != SCRUST_METRIC_COSINE)
        return fail(st, SCRUST_INVALID_PARAMETER, "metric must be euclidean or cosine, got %d", o->metric);
    if (o->mode != SCRUST_MODE_EXACT && o->mode != SCRUST_MODE_REFERENCE_SNAP)
        return fail(st, SCRUST_INVALID_PARAMETER, "mode must be exact or reference_snap, got %d", o->mode);
    if (o->mode == SCRUST_MODE_REFERENCE_SNAP && o->metric == SCRUST_METRIC_COSINE)
        return fail(st, SCRUST_INVALID_PARAMETER,
                    "metric must be euclidean in reference_snap mode (the reference has no cosine), got cosine");
    if (o->precision != SCRUST_PRECISION_FP16 && o->precision != SCRUST_PRECISION_BF16)
        return fail(st, SCRUST_INVALID_PARAMETER, "precision must be fp16 or bf16, got %d", o->precision);
    if (o->ordering != SCRUST_ORDERING_AUTO && o->ordering != SCRUST_ORDERING_OFF && o->ordering != SCRUST_ORDERING_ON)
        return fail(st, SCRUST_INVALID_PARAMETER, "ordering must be auto, off or on, got %d", o->ordering);
    return SCRUST_OK;
}


struct KnnBuffers {
    const float* xr = nullptr;   // rows the rerank measures
    float* xwork = nullptr;
    double* norm64 = nullptr;
    float* norm2 = nullptr;
};

// Candidate-list geometry: column segments per row block (so small inputs
// still fill the GPU) and the list capacity that triggers a prune.
int32_t plan_lists(scrust_context* ctx, const scrust_knn_options& o, int k, int row_blocks, int col_tiles,
                   int blocks_wanted, int headroom, int default_cap, Lists* lists, scrust_status* st) {
    int segments = 1;
    if (o.segments) {
        segments = (int)o.segments;
    } else if (row_blocks < blocks_wanted) {
        segments = (blocks_wanted + row_blocks - 1) / row_blocks;
        segments = std::min(segments, std::max(1, kRerankUnion / (4 * k)));
    }
    segments = std::max(1, std::min(segments, col_tiles));
    const int per = (col_tiles + segments - 1) / segments;
    segments = (col_tiles + per - 1) / per;  // no empty segment
    int cap = (int)o.list_capacity;
    if (cap == 0) cap = std::max(default_cap, (2 * k + 32 + 31) / 32 * 32);
    cap = std::max(cap, k + 32);
    cap = (cap + 3) / 4 * 4;  // lists start on 16-byte boundaries
    const int ctot = cap + headroom;
    if (ctot > 512)
        return fail(st, SCRUST_INVALID_PARAMETER, "list_capacity must be at most %d, got %d", 512 - headroom, cap);
    lists->cap = cap;
    lists->ctot = ctot;
    lists->segments = segments;
    (void)ctx;
    return SCRUST_OK;
}

}  // namespace

int32_t alloc_lists(scrust_context* ctx, int64_t rows_pad, Lists* lists, scrust_status* st) {
    cudaError_t e = cudaSuccess;
    const size_t slots = (size_t)rows_pad * lists->segments;
    lists->ids = (uint32_t*)ws_get(ctx, SLOT_LIST_IDS, sizeof(uint32_t) * slots * lists->ctot, &e);
    lists->vals = (float*)ws_get(ctx, SLOT_LIST_VALS, sizeof(float) * slots * lists->ctot, &e);
    lists->cnt = (uint32_t*)ws_get(ctx, SLOT_LIST_CNT, sizeof(uint32_t) * slots, &e);
    lists->overflow = (uint32_t*)ws_get(ctx, SLOT_OVERFLOW, sizeof(uint32_t) * (size_t)rows_pad, &e);
    if (!lists->ids || !lists->vals || !lists->cnt || !lists->overflow) return cuda_fail(st, e, "workspace");
    if ((e = cudaMemsetAsync(lists->overflow, 0, sizeof(uint32_t) * (size_t)rows_pad, ctx->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(lists->cnt, 0, sizeof(uint32_t) * slots, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "memset");
    return SCRUST_OK;
}

namespace {

// Whether the tensor form applies: the mode is exact and the row plus the
// three norm columns fits one 64-wide operand row.
bool tensor_form_applies(const scrust_knn_options& o, int d) {
    return o.mode == SCRUST_MODE_EXACT && d + 3 <= 64;
}

// Whether a solve runs the tensor form: asked for (or automatic) and applies.
bool uses_tensor_form(const scrust_knn_options& o, int d) {
    return (o.form == SCRUST_FORM_TENSOR || o.form == SCRUST_FORM_AUTO) && tensor_form_applies(o, d);
}

// Success, noting in the message when an explicit tensor-form request ran the
// plain form instead.
int32_t ok_form(scrust_status* st, const scrust_knn_options* opt, int d) {
    ok(st);
    if (st && opt && opt->form == SCRUST_FORM_TENSOR && !tensor_form_applies(*opt, d))
        snprintf(st->message, sizeof(st->message),
                 "ran the plain form: the tensor form needs exact mode and at most 61 dimensions, got %s mode "
                 "and %d dimensions",
                 opt->mode == SCRUST_MODE_EXACT ? "exact" : "reference_snap", d);
    return SCRUST_OK;
}

// The kNN solve on device pointers, enqueued on ctx->stream.
int32_t knn_device_impl(scrust_context* ctx, const float* x, uint64_t n64, uint64_t d64, uint32_t k,
                        const scrust_knn_options* opt, uint32_t* out_idx, float* out_dist,
                        scrust_status* st) {
    cudaError_t e = cudaSuccess;
    scrust_knn_options o;
    scrust_knn_options_default(&o);
    if (opt) o = *opt;
    KnnPlan plan;
    plan.nq = plan.nr = (int64_t)n64;
    plan.d = (int)d64;
    plan.k = (int)k;
    plan.self = true;
    plan.form = o.form;
    plan.metric = o.metric;
    plan.mode = o.mode;
    plan.precision = o.precision;
    const int64_t n = plan.nq;
    const int d = plan.d;
    const bool ref = o.mode == SCRUST_MODE_REFERENCE_SNAP;
    const bool cosine = o.metric == SCRUST_METRIC_COSINE;
    const bool tensor = uses_tensor_form(o, d);
    const int64_t n_pad = tensor ? (n + 255) / 256 * 256 : (n + 127) / 128 * 128;
    const int dp = d <= 64 ? (d + 3) / 4 * 4 : (d + 63) / 64 * 64;
    cudaStream_t s = ctx->stream;

    const float* xwork = x;
    float* xcentred = nullptr;
    double* norm64 = nullptr;
    ctx->stats_launch = 0;
    mark(ctx, PH_START);
    if (cosine) {
        float* xn = (float*)ws_get(ctx, SLOT_XWORK, sizeof(float) * (size_t)n * d, &e);
        norm64 = (double*)ws_get(ctx, SLOT_NORM64, sizeof(double) * (size_t)n, &e);
        if (!xn || !norm64) return cuda_fail(st, e, "workspace");
        if ((e = launch_normalise_rows(x, n, d, xn, norm64, ctx->d_err, s)) != cudaSuccess)
            return cuda_fail(st, e, "normalise");
        ctx->launches += 1;
        xwork = xn;
    } else if (ref) {
        xcentred = (float*)ws_get(ctx, SLOT_XWORK, sizeof(float) * (size_t)n * d, &e);
        if (!xcentred) return cuda_fail(st, e, "workspace");
    }
    const int mean_blocks = (int)((n + 2047) / 2048);
    double* means = (double*)ws_get(ctx, SLOT_MEANS, sizeof(double) * ((size_t)d * (mean_blocks + 1)), &e);
    float* norm2 = (float*)ws_get(ctx, SLOT_NORM2, sizeof(float) * (size_t)n_pad, &e);
    float* cnorm = (float*)ws_get(ctx, SLOT_CNORM, sizeof(float) * (size_t)n_pad, &e);
    float* margin = (float*)ws_get(ctx, SLOT_MARGIN, sizeof(float) * (size_t)n_pad + 64, &e);
    if (!means || !norm2 || !cnorm || !margin) return cuda_fail(st, e, "workspace");
    uint32_t* max_bits = (uint32_t*)(margin + n_pad);  // spare words: max norm, max eps, max |b_hat|
    if ((e = cudaMemsetAsync(max_bits, 0, 4 * sizeof(uint32_t), s)) != cudaSuccess) return cuda_fail(st, e, "memset");
    if ((e = tensor ? launch_column_means_centre(xwork, n, d, means, means + d, s)
                    : launch_column_means(xwork, n, d, ref, means, means + d, s)) != cudaSuccess)
        return cuda_fail(st, e, "column means");
    ctx->launches += ref ? 1 : 2;

    Lists lists;
    RowBounds bounds;
    const uint32_t* perm = nullptr;  // rows of the lists -> input rows (tensor form with ordering)
    const float* rerank_xs = nullptr;
    const float* rerank_theta = nullptr;
    int rerank_stride = 0;  // floats per row of rerank_xs
    bool rerank_ids_only = false;  // the lists were filled by collect passes (ids, no values)
    if (tensor) {
        const bool bf16 = o.precision == SCRUST_PRECISION_BF16;
        void* A16 = ws_get(ctx, SLOT_A16, (size_t)n_pad * 64 * 2, &e);
        void* B16 = ws_get(ctx, SLOT_B16, (size_t)n_pad * 64 * 2, &e);
        float* rb = (float*)ws_get(ctx, SLOT_QERR, sizeof(float) * 4 * (size_t)n_pad, &e);
        if (!A16 || !B16 || !rb) return cuda_fail(st, e, "workspace");
        float *bA = rb, *beps = rb + n_pad, *bdelta = rb + 2 * n_pad, *beps2 = rb + 3 * n_pad;
        if ((e = launch_max_centred_norm(xwork, n, d, means, max_bits, ctx->sm_count, s)) != cudaSuccess)
            return cuda_fail(st, e, "centre");
        ctx->launches += 1;
        const int items = (int)(n_pad / 256);
        // Ordering needs one column segment: it is on for large solves, where
        // the row blocks alone fill the GPU, or when asked for.
        const bool order_rows = n <= kOrderMaxRows &&
                                (o.ordering == SCRUST_ORDERING_ON     ? (o.segments <= 1)
                                 : o.ordering == SCRUST_ORDERING_AUTO ? (o.segments <= 1 && n >= kOrderMinRows)
                                                                      : false);
        // One column segment (two column parts) unless asked otherwise: every
        // list then sees all of its row's columns, its threshold is the row's
        // own, and the rerank needs no selection.
        scrust_knn_options lo = o;
        if (order_rows || o.segments == 0) lo.segments = 1;

        RowOrder order;
        if (order_rows) {
            int32_t rc = build_row_order(ctx, xwork, n, d, means, max_bits, cosine, bf16, A16, B16, bA, beps, bdelta,
                                         beps2, &order, st);
            if (rc) return rc;
        }
        // An ordered solve has its operands in list order already.
        if (!order_rows) {
            if ((e = launch_tensor_operands(xwork, n, n_pad, d, means, max_bits, cosine, bf16, nullptr, A16, B16, bA,
                                            beps, max_bits + 1, max_bits + 2, s)) != cudaSuccess)
                return cuda_fail(st, e, "tensor operands");
            ctx->launches += 1;
        }
        if ((e = launch_tensor_bounds(n, bA, beps, max_bits + 1, max_bits + 2, bdelta, beps2, s)) != cudaSuccess)
            return cuda_fail(st, e, "tensor bounds");
        ctx->launches += 1;
        // Headroom of 128: a tensor-form list is checked once per tile, after
        // its warp has appended up to 128 columns.
        // Ordered solves keep long lists (256): a row block's first tiles
        // fill its lists before any threshold exists, and every prune is a
        // latency the row block waits for.
        int32_t rc = plan_lists(ctx, lo, (int)k, items, (int)(n_pad / 256), 8 * ctx->sm_count, 128,
                                order_rows ? 256 : 64, &lists, st);
        if (rc) return rc;
        lists.segments *= 2;  // one list per (column segment, column part) of a row
        if ((rc = alloc_lists(ctx, n_pad, &lists, st))) return rc;
        plan.cap = lists.cap;
        plan.ctot = lists.ctot;
        plan.segments = lists.segments;
        mark(ctx, PH_PREP);
        if (order_rows) {
            // The priority tiles first; then the tiles the tile balls cannot
            // rule out.
            TileLists first;
            first.tiles = order.prio;
            first.count = order.prio_cnt;
            first.stride = kPrioMax;
            first.order = order.prio_order;
            // k <= 32: the first pass only tightens the thresholds, and one
            // collect pass over both tile lists appends just the ids of the
            // columns below them.  The thresholds after the priority tiles
            // already bound every row (a threshold pass over the other tiles
            // would lower them by a fraction of a percent of the candidates),
            // so the other tiles are only collected.  Larger k: two passes
            // that keep lists.
            const bool split = k <= 32;
            const int mode = split ? kPassThresholds : kPassFull;
            rerank_ids_only = split;
            // The threshold pass leaves each list's register top-K (a top-16
            // or top-32: k >= 2; k = 1 keeps a single value a lane), and each
            // row's threshold is then taken from its two column parts'
            // lists together.
            const int width = k <= 16 ? 16 : 32;
            const bool merge = split && k >= 2;
            float* topk = nullptr;
            if (merge) {
                topk = (float*)ws_get(ctx, SLOT_TOPK, sizeof(float) * (size_t)lists.segments * width * n_pad, &e);
                if (!topk) return cuda_fail(st, e, "workspace");
            }
            if ((e = launch_tensor_candidates(ctx, plan, A16, n_pad, B16, n_pad, bA, bdelta, beps2, lists, bf16,
                                              &first, false, order.theta, nullptr, sweep_stats(ctx), nullptr, mode,
                                              topk)) != cudaSuccess ||
                (merge && (e = launch_merge_part_thresholds(topk, width, n, n_pad, (int)k, bA, bdelta, beps2,
                                                            order.theta, s)) != cudaSuccess))
                return cuda_fail(st, e, "knn_candidates_tc");
            ctx->launches += merge ? 2 : 1;
            mark(ctx, PH_PASS1);
            TileLists second;
            if ((rc = build_second_pass(ctx, A16, bf16, n, d, order, bA, bdelta, &second, st))) return rc;
            mark(ctx, PH_LISTS);
            if (split) {
                mark(ctx, PH_PASS2);
                TileLists both = first;
                both.tiles2 = second.tiles;
                both.count2 = second.count;
                both.stride2 = second.stride;
                if ((e = launch_tensor_candidates(ctx, plan, A16, n_pad, B16, n_pad, bA, bdelta, beps2, lists, bf16,
                                                  &both, false, order.theta, nullptr, sweep_stats(ctx), nullptr,
                                                  kPassCollect)) != cudaSuccess)
                    return cuda_fail(st, e, "knn_candidates_tc");
                mark(ctx, PH_COLLECT1);
                ctx->launches += 1;
            } else {
                if ((e = launch_tensor_candidates(ctx, plan, A16, n_pad, B16, n_pad, bA, bdelta, beps2, lists, bf16,
                                                  &second, true, order.theta, nullptr, sweep_stats(ctx), nullptr,
                                                  mode)) != cudaSuccess)
                    return cuda_fail(st, e, "knn_candidates_tc");
                mark(ctx, PH_PASS2);
                ctx->launches += 1;
            }
        } else {
            // Every list keeps its threshold, so the rerank needs no selection.
            float* theta = (float*)ws_get(ctx, SLOT_THETA, sizeof(float) * (size_t)lists.segments * n_pad, &e);
            if (!theta) return cuda_fail(st, e, "workspace");
            rerank_xs = xwork;
            rerank_theta = theta;
            rerank_stride = d;
            TileLists shared;  // several column segments share each row's threshold
            if (lists.segments > 2) {
                shared.row_theta = (uint32_t*)ws_get(ctx, SLOT_ROWTHETA, sizeof(uint32_t) * (size_t)n_pad, &e);
                if (!shared.row_theta) return cuda_fail(st, e, "workspace");
                if ((e = cudaMemsetAsync(shared.row_theta, 0xff, sizeof(uint32_t) * (size_t)n_pad, s)) != cudaSuccess)
                    return cuda_fail(st, e, "memset");
            }
            if ((e = launch_tensor_candidates(ctx, plan, A16, n_pad, B16, n_pad, bA, bdelta, beps2, lists, bf16,
                                              &shared, false, theta, nullptr, sweep_stats(ctx))) != cudaSuccess)
                return cuda_fail(st, e, "knn_candidates_tc");
            ctx->launches += 1;
        }
        mark(ctx, PH_CAND);
        perm = order.perm;
        if (order_rows) {
            float* xs = (float*)ws_get(ctx, SLOT_XSORTED, sizeof(float) * (size_t)n * padded_row_floats(d), &e);
            if (!xs) return cuda_fail(st, e, "workspace");
            if ((e = launch_gather_rows(xwork, order.perm, n, d, padded_row_floats(d), xs, s)) != cudaSuccess)
                return cuda_fail(st, e, "gather rows");
            ctx->launches += 1;
            rerank_xs = xs;
            rerank_theta = order.theta;
            rerank_stride = padded_row_floats(d);
        }
        bounds.A = bA;
        bounds.delta = bdelta;
        bounds.eps2 = beps2;
    } else {
        float* coords_t = (float*)ws_get(ctx, SLOT_COORDS_T, sizeof(float) * (size_t)dp * n_pad, &e);
        if (!coords_t) return cuda_fail(st, e, "workspace");
        if ((e = launch_centre_transpose(xwork, n, n_pad, d, dp, means, coords_t, norm2, cnorm, xcentred, max_bits,
                                         s)) != cudaSuccess)
            return cuda_fail(st, e, "centre");
        if ((e = launch_margins(cnorm, norm2, n, d, o.mode, o.metric, SCRUST_FORM_PLAIN, max_bits, nullptr, nullptr,
                                1.0f, margin, s)) != cudaSuccess)
            return cuda_fail(st, e, "margins");
        ctx->launches += 2;
        const int row_tiles = (int)(n_pad / 128);
        int32_t rc = plan_lists(ctx, o, (int)k, row_tiles, row_tiles, 4 * ctx->sm_count, 128, 64, &lists, st);
        if (rc) return rc;
        if ((rc = alloc_lists(ctx, n_pad, &lists, st))) return rc;
        plan.cap = lists.cap;
        plan.ctot = lists.ctot;
        plan.segments = lists.segments;
        mark(ctx, PH_PREP);
        if ((e = launch_plain_candidates(ctx, plan, coords_t, n_pad, coords_t, n_pad, dp, norm2, margin, lists)) !=
            cudaSuccess)
            return cuda_fail(st, e, "knn_candidates_f32");
        ctx->launches += 1;
        mark(ctx, PH_CAND);
        bounds.margin = margin;
    }

    const float* xr = ref ? xcentred : xwork;
    if ((e = launch_rerank(ctx, plan, xr, xr, norm2, norm2, norm64, norm64, x, x, bounds, lists, perm, rerank_xs,
                           rerank_theta, out_idx, out_dist, nullptr, nullptr, nullptr, rerank_stride,
                           rerank_ids_only)) != cudaSuccess)
        return cuda_fail(st, e, "knn_rerank");
    mark(ctx, PH_RERANK);
    return ok_form(st, opt, d);
}

int32_t take_csr_buffers(scrust_context* ctx, uint64_t rows, uint64_t nnz_cap, CsrBuffers* out,
                         scrust_status* st) {
    for (size_t i = 0; i < ctx->csr_pool.size(); ++i) {
        CsrBuffers& b = ctx->csr_pool[i];
        if (b.rows_cap >= rows && b.nnz_cap >= nnz_cap) {
            *out = b;
            ctx->csr_pool.erase(ctx->csr_pool.begin() + (long)i);
            return SCRUST_OK;
        }
    }
    CsrBuffers b;
    b.rows_cap = rows;
    b.nnz_cap = std::max<uint64_t>(nnz_cap, 1);
    cudaError_t e = cudaMalloc(&b.indptr, sizeof(uint32_t) * (rows + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b.indices, sizeof(uint32_t) * b.nnz_cap);
    if (e == cudaSuccess) e = cudaMalloc(&b.values, sizeof(float) * b.nnz_cap);
    if (e != cudaSuccess) {
        cudaFree(b.indptr);
        cudaFree(b.indices);
        cudaFree(b.values);
        cudaGetLastError();
        return cuda_fail(st, e, "csr allocation");
    }
    *out = b;
    return SCRUST_OK;
}

void return_csr_buffers(scrust_context* ctx, const CsrBuffers& b) {
    if (!b.indptr) return;
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->csr_pool.push_back(b);
}

// `distinct_rows`: the graph is one this library's kNN built (every row's ids
// distinct), which the faster bucket transpose relies on.
// `ranges`: run the union in row ranges for a streamed download (see
// CsrStream); *streamed says whether it did.
int32_t conn_device_impl(scrust_context* ctx, const uint32_t* idx, const float* dist, uint64_t n, uint32_t k,
                         bool validate, scrust_csr** out, scrust_status* st, bool distinct_rows = false,
                         bool ranges = false, bool* streamed = nullptr) {
    CsrBuffers b;
    int32_t rc = take_csr_buffers(ctx, n, 2 * n * (uint64_t)k, &b, st);
    if (rc) return rc;
    rc = run_connectivities(ctx, idx, dist, (int64_t)n, (int)k, validate, &b, st, distinct_rows, ranges, streamed);
    mark(ctx, PH_CONN);
    if (rc) {
        ctx->csr_pool.push_back(b);
        return rc;
    }
    scrust_csr* csr = new (std::nothrow) scrust_csr;
    if (!csr) {
        ctx->csr_pool.push_back(b);
        return fail(st, SCRUST_OOM, "host allocation failed");
    }
    csr->n_rows = n;
    csr->n_cols = n;
    csr->nnz = UINT64_MAX;  // read from indptr[n] on first request
    csr->on_device = 1;
    csr->owner = ctx;
    csr->buf = b;
    *out = csr;
    return ok(st);
}

// Copies a device CSR into a new host CSR (synchronising the stream).
// Pinned host slabs for downloaded graphs, reused across calls and
// contexts: a device-to-host copy into pinned memory runs at the link's
// speed, while pageable memory goes through the driver's staging buffers.
// Freed slabs are kept (up to kPinnedKeep of them) for the next download;
// the pool is never torn down (the process exit reclaims it).
std::mutex g_pinned_mu;
std::vector<std::pair<void*, size_t>> g_pinned_free;
constexpr size_t kPinnedKeep = 4;

void* pinned_take(size_t bytes, size_t* got) {
    {
        std::lock_guard<std::mutex> lock(g_pinned_mu);
        size_t best = g_pinned_free.size();
        for (size_t i = 0; i < g_pinned_free.size(); ++i)
            if (g_pinned_free[i].second >= bytes &&
                (best == g_pinned_free.size() || g_pinned_free[i].second < g_pinned_free[best].second))
                best = i;
        if (best < g_pinned_free.size()) {
            const auto slab = g_pinned_free[best];
            g_pinned_free.erase(g_pinned_free.begin() + (long)best);
            *got = slab.second;
            return slab.first;
        }
    }
    const size_t want = (bytes + bytes / 4 + 4095) & ~(size_t)4095;
    void* p = nullptr;
    if (cudaMallocHost(&p, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    *got = want;
    return p;
}

void pinned_give(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    g_pinned_free.emplace_back(p, bytes);
    if (g_pinned_free.size() > kPinnedKeep) {  // drop the smallest
        size_t small = 0;
        for (size_t i = 1; i < g_pinned_free.size(); ++i)
            if (g_pinned_free[i].second < g_pinned_free[small].second) small = i;
        cudaFreeHost(g_pinned_free[small].first);
        g_pinned_free.erase(g_pinned_free.begin() + (long)small);
    }
}

int32_t csr_to_host(scrust_context* ctx, scrust_csr* dev, scrust_csr** out, scrust_status* st) {
    uint32_t nnz = 0;
    cudaError_t e = cudaMemcpyAsync(&nnz, dev->buf.indptr + dev->n_rows, sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(st, e, "csr readback");
    scrust_csr* h = new (std::nothrow) scrust_csr;
    if (!h) return fail(st, SCRUST_OOM, "host allocation failed");
    const size_t ip_bytes = sizeof(uint32_t) * (dev->n_rows + 1);
    const size_t off_idx = (ip_bytes + 255) & ~(size_t)255;
    const size_t off_val = off_idx + ((sizeof(uint32_t) * (size_t)nnz + 255) & ~(size_t)255);
    const size_t bytes = off_val + sizeof(float) * (size_t)nnz;
    h->pinned = pinned_take(bytes, &h->pinned_bytes);
    if (!h->pinned) {
        delete h;
        return fail(st, SCRUST_OOM, "pinned host allocation of %zu bytes failed", bytes);
    }
    h->p_indptr = reinterpret_cast<uint32_t*>(h->pinned);
    h->p_indices = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(h->pinned) + off_idx);
    h->p_values = reinterpret_cast<float*>(reinterpret_cast<char*>(h->pinned) + off_val);
    h->n_rows = dev->n_rows;
    h->n_cols = dev->n_cols;
    h->nnz = nnz;
    h->on_device = 0;
    e = cudaMemcpyAsync(h->p_indptr, dev->buf.indptr, ip_bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && nnz)
        e = cudaMemcpyAsync(h->p_indices, dev->buf.indices, sizeof(uint32_t) * nnz, cudaMemcpyDeviceToHost,
                            ctx->stream);
    if (e == cudaSuccess && nnz)
        e = cudaMemcpyAsync(h->p_values, dev->buf.values, sizeof(float) * nnz, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        pinned_give(h->pinned, h->pinned_bytes);
        delete h;
        return cuda_fail(st, e, "csr readback");
    }
    *out = h;
    return ok(st);
}

}  // namespace

// csr_to_host for a CSR built in ctx->csr_stream's row ranges: the host slab
// is sized by the CSR's capacity, and as each range is placed (its event;
// its end offset is then in h_bounds) its rows and entries are queued on the
// copy stream, so the link carries the early ranges while the later ones
// merge.  Synchronises the copy stream.
int32_t csr_to_host_streamed(scrust_context* ctx, scrust_csr* dev, scrust_csr** out, scrust_status* st) {
    CsrStream& cs = ctx->csr_stream;
    scrust_csr* h = new (std::nothrow) scrust_csr;
    if (!h) return fail(st, SCRUST_OOM, "host allocation failed");
    const uint64_t n = dev->n_rows;
    const size_t cap = dev->buf.nnz_cap;
    const size_t ip_bytes = sizeof(uint32_t) * (n + 1);
    const size_t off_idx = (ip_bytes + 255) & ~(size_t)255;
    const size_t off_val = off_idx + ((sizeof(uint32_t) * cap + 255) & ~(size_t)255);
    const size_t bytes = off_val + sizeof(float) * cap;
    h->pinned = pinned_take(bytes, &h->pinned_bytes);
    if (!h->pinned) {
        delete h;
        return fail(st, SCRUST_OOM, "pinned host allocation of %zu bytes failed", bytes);
    }
    h->p_indptr = reinterpret_cast<uint32_t*>(h->pinned);
    h->p_indices = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(h->pinned) + off_idx);
    h->p_values = reinterpret_cast<float*>(reinterpret_cast<char*>(h->pinned) + off_val);
    h->n_rows = n;
    h->n_cols = dev->n_cols;
    h->on_device = 0;
    cudaStream_t c = ctx->copy_stream;
    cudaError_t e = cudaSuccess;
    uint32_t lo = 0;
    for (int r = 0; r < kCsrRanges && e == cudaSuccess; ++r) {
        if ((e = cudaEventSynchronize(cs.merged[r])) != cudaSuccess) break;
        const uint32_t hi = cs.h_bounds[r];
        if (hi < lo || hi > cap) {
            e = cudaErrorIllegalState;
            break;
        }
        const uint64_t r0 = n * r / kCsrRanges, r1 = n * (r + 1) / kCsrRanges;
        if ((e = cudaStreamWaitEvent(c, cs.merged[r], 0)) != cudaSuccess) break;
        // Rows r0..r1 (indptr[r1] is the next range's first offset, final now).
        e = cudaMemcpyAsync(h->p_indptr + r0, dev->buf.indptr + r0, sizeof(uint32_t) * (r1 - r0 + 1),
                            cudaMemcpyDeviceToHost, c);
        if (e == cudaSuccess && hi > lo)
            e = cudaMemcpyAsync(h->p_indices + lo, dev->buf.indices + lo, sizeof(uint32_t) * (hi - lo),
                                cudaMemcpyDeviceToHost, c);
        if (e == cudaSuccess && hi > lo)
            e = cudaMemcpyAsync(h->p_values + lo, dev->buf.values + lo, sizeof(float) * (hi - lo),
                                cudaMemcpyDeviceToHost, c);
        lo = hi;
    }
    h->nnz = lo;
    const cudaError_t es = cudaStreamSynchronize(c);
    if (e == cudaSuccess) e = es;
    if (e != cudaSuccess) {
        pinned_give(h->pinned, h->pinned_bytes);
        delete h;
        return cuda_fail(st, e, "csr readback");
    }
    *out = h;
    return ok(st);
}

int32_t csr_take(scrust_context* ctx, uint64_t rows, uint64_t nnz_cap, CsrBuffers* out, scrust_status* st) {
    return take_csr_buffers(ctx, rows, nnz_cap, out, st);
}

void csr_give(scrust_context* ctx, const CsrBuffers& b) {
    if (b.indptr) ctx->csr_pool.push_back(b);
}

int32_t csr_download(scrust_context* ctx, const CsrBuffers& b, uint64_t rows, uint64_t cols, scrust_csr** out,
                     scrust_status* st) {
    scrust_csr dev;
    dev.n_rows = rows;
    dev.n_cols = cols;
    dev.on_device = 1;
    dev.buf = b;
    return csr_to_host(ctx, &dev, out, st);
}

}  // namespace scrust

using namespace scrust;

extern "C" {

void scrust_knn_options_default(scrust_knn_options* o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->struct_size = sizeof(*o);
    o->form = SCRUST_FORM_AUTO;
    o->metric = SCRUST_METRIC_EUCLIDEAN;
    o->mode = SCRUST_MODE_EXACT;
    o->precision = SCRUST_PRECISION_FP16;
}

int32_t scrust_cuda_gpu_available(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    for (int i = 0; i < count; i++) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, i) == cudaSuccess && p.major == 10 && p.minor == 3) return 1;
    }
    return 0;
}

scrust_context* scrust_cuda_context_create(int32_t device, scrust_status* st) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        fail(st, SCRUST_NO_GPU, "no CUDA device is available on this machine");
        return nullptr;
    }
    if (device < 0 || device >= count) {
        fail(st, SCRUST_NO_GPU, "no CUDA device %d on this machine (%d present)", device, count);
        return nullptr;
    }
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess || p.major != 10 || p.minor != 3) {
        cudaGetLastError();
        fail(st, SCRUST_NO_GPU, "CUDA device %d is not compute capability 10.3 (sm_103a)", device);
        return nullptr;
    }
    DeviceGuard device_guard(device);
    int current = -1;
    if (cudaGetDevice(&current) != cudaSuccess || current != device) {
        cudaGetLastError();
        fail(st, SCRUST_NO_GPU, "cannot select CUDA device %d", device);
        return nullptr;
    }
    scrust_context* ctx = new (std::nothrow) scrust_context;
    if (!ctx) {
        fail(st, SCRUST_OOM, "host allocation failed");
        return nullptr;
    }
    ctx->device = device;
    ctx->sm_count = p.multiProcessorCount;
    ctx->smem_optin = p.sharedMemPerBlockOptin;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->copy_ev, cudaEventDisableTiming);
    for (int i = 0; i < kCsrRanges && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&ctx->csr_stream.merged[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->csr_stream.h_bounds, sizeof(uint32_t) * (kCsrRanges + 1));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, sizeof(int) * DERR_COUNT);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_counter, sizeof(uint32_t) * 16);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, sizeof(int) * DERR_COUNT);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_counter, 0, sizeof(uint32_t) * 16);
    if (e == cudaSuccess) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e == cudaSuccess && q == cudaDriverEntryPointSuccess)
            ctx->encode_tiled = (PFN_cuTensorMapEncodeTiled_v12000)fn;
        else
            e = cudaErrorNotSupported;
    }
    if (e != cudaSuccess) {
        cuda_fail(st, e, "context creation");
        scrust_cuda_context_destroy(ctx);
        return nullptr;
    }
    ok(st);
    return ctx;
}

void scrust_cuda_context_destroy(scrust_context* ctx) {
    if (!ctx) return;
    DeviceGuard device_guard(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int i = 0; i < SLOT_COUNT; i++)
        if (ctx->ws.ptr[i]) cudaFree(ctx->ws.ptr[i]);
    for (auto& b : ctx->csr_pool) {
        cudaFree(b.indptr);
        cudaFree(b.indices);
        cudaFree(b.values);
    }
    for (int i = 0; i < PH_COUNT; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    for (int i = 0; i < kCsrRanges; i++)
        if (ctx->csr_stream.merged[i]) cudaEventDestroy(ctx->csr_stream.merged[i]);
    if (ctx->csr_stream.h_bounds) cudaFreeHost(ctx->csr_stream.h_bounds);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->copy_ev) cudaEventDestroy(ctx->copy_ev);
    if (ctx->d_stats) cudaFree(ctx->d_stats);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    cudaGetLastError();
    delete ctx;
}

void* scrust_cuda_context_stream(scrust_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

uint32_t scrust_cuda_max_supported_k(const scrust_context* ctx) { return ctx ? kMaxK : 0; }

int32_t scrust_cuda_knn_device(scrust_context* ctx, const float* x, uint64_t n, uint64_t d, uint32_t k,
                               const scrust_knn_options* opt, uint32_t* out_idx, float* out_dist,
                               scrust_status* st) {
    int32_t rc = check_knn_args(n, d, k, st);
    if (rc) return rc;
    if ((rc = check_options(opt, st))) return rc;
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist) return fail(st, SCRUST_SHAPE, "expected non-null device pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    return knn_device_impl(ctx, x, n, d, k, opt, out_idx, out_dist, st);
}

int32_t scrust_cuda_knn(scrust_context* ctx, const float* x, uint64_t n, uint64_t d, uint32_t k,
                        const scrust_knn_options* opt, uint32_t* out_idx, float* out_dist, scrust_status* st) {
    int32_t rc = check_knn_args(n, d, k, st);
    if (rc) return rc;
    if ((rc = check_options(opt, st))) return rc;
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist) return fail(st, SCRUST_SHAPE, "expected non-null host pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    float* dx = (float*)ws_get(ctx, SLOT_HOST_IN, sizeof(float) * n * d, &e);
    uint32_t* di = (uint32_t*)ws_get(ctx, SLOT_HOST_IDX, sizeof(uint32_t) * n * k, &e);
    float* dd = (float*)ws_get(ctx, SLOT_HOST_DIST, sizeof(float) * n * k, &e);
    if (!dx || !di || !dd) return cuda_fail(st, e, "workspace");
    if ((e = cudaMemcpyAsync(dx, x, sizeof(float) * n * d, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "upload");
    if ((rc = knn_device_impl(ctx, dx, n, d, k, opt, di, dd, st))) return rc;
    if ((e = cudaMemcpyAsync(out_idx, di, sizeof(uint32_t) * n * k, cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out_dist, dd, sizeof(float) * n * k, cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess)
        return cuda_fail(st, e, "download");
    if ((rc = collect_device_errors(ctx, st))) return rc;
    return ok_form(st, opt, (int)d);
}

int32_t scrust_cuda_connectivities_device(scrust_context* ctx, const uint32_t* idx, const float* dist, uint64_t n,
                                          uint32_t k, scrust_csr** out, scrust_status* st) {
    if (n == 0 || k == 0)
        return fail(st, SCRUST_SHAPE, "expected a neighbour graph with at least one cell and one neighbour, got %llu x %u",
                    (unsigned long long)n, k);
    if (n >= 0xffffffffull || 2 * n * (uint64_t)k >= 0xffffffffull)
        return fail(st, SCRUST_SHAPE, "expected fewer than 2^31 graph entries, got %llu x %u", (unsigned long long)n, k);
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!idx || !dist || !out) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    return conn_device_impl(ctx, idx, dist, n, k, true, out, st);
}

int32_t scrust_cuda_connectivities(scrust_context* ctx, const uint32_t* idx, const float* dist, uint64_t n,
                                   uint32_t k, scrust_csr** out, scrust_status* st) {
    if (n == 0 || k == 0)
        return fail(st, SCRUST_SHAPE, "expected a neighbour graph with at least one cell and one neighbour, got %llu x %u",
                    (unsigned long long)n, k);
    if (n >= 0xffffffffull || 2 * n * (uint64_t)k >= 0xffffffffull)
        return fail(st, SCRUST_SHAPE, "expected fewer than 2^31 graph entries, got %llu x %u", (unsigned long long)n, k);
    if (!idx || !dist || !out) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    for (uint64_t i = 0; i < n * k; i++)
        if (idx[i] >= n)
            return fail(st, SCRUST_SHAPE, "expected neighbour ids below %llu, got an out-of-range neighbour id",
                        (unsigned long long)n);
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    uint32_t* di = (uint32_t*)ws_get(ctx, SLOT_HOST_IDX, sizeof(uint32_t) * n * k, &e);
    float* dd = (float*)ws_get(ctx, SLOT_HOST_DIST, sizeof(float) * n * k, &e);
    if (!di || !dd) return cuda_fail(st, e, "workspace");
    if ((e = cudaMemcpyAsync(di, idx, sizeof(uint32_t) * n * k, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dd, dist, sizeof(float) * n * k, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "upload");
    scrust_csr* dev = nullptr;
    int32_t rc = conn_device_impl(ctx, di, dd, n, k, false, &dev, st);
    if (rc) return rc;
    rc = csr_to_host(ctx, dev, out, st);
    ctx->csr_pool.push_back(dev->buf);
    delete dev;
    if (rc) return rc;
    return collect_device_errors(ctx, st);
}

int32_t scrust_cuda_smooth_knn_distances(scrust_context* ctx, const float* dist, uint64_t n, uint32_t k,
                                         float* sigmas, float* rhos, scrust_status* st) {
    if (n == 0 || k == 0)
        return fail(st, SCRUST_SHAPE, "expected a distance matrix with at least one cell and one neighbour, got %llu x %u",
                    (unsigned long long)n, k);
    if (!dist || !sigmas || !rhos) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    float* dd = (float*)ws_get(ctx, SLOT_HOST_DIST, sizeof(float) * n * k, &e);
    float* so = (float*)ws_get(ctx, SLOT_CONN_G, sizeof(float) * 2 * n, &e);
    if (!dd || !so) return cuda_fail(st, e, "workspace");
    if ((e = cudaMemcpyAsync(dd, dist, sizeof(float) * n * k, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "upload");
    if ((e = launch_smooth_knn(ctx, dd, (int64_t)n, (int)k, so, so + n, true)) != cudaSuccess)
        return cuda_fail(st, e, "smooth_knn");
    if ((e = cudaMemcpyAsync(sigmas, so, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(rhos, so + n, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "download");
    return collect_device_errors(ctx, st);
}

int32_t scrust_cuda_neighbors_graph_device(scrust_context* ctx, const float* x, uint64_t n, uint64_t d, uint32_t k,
                                           const scrust_knn_options* opt, uint32_t* out_idx, float* out_dist,
                                           scrust_csr** conn, scrust_status* st) {
    int32_t rc = check_knn_args(n, d, k, st);
    if (rc) return rc;
    if ((rc = check_options(opt, st))) return rc;
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist || !conn) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    if ((rc = knn_device_impl(ctx, x, n, d, k, opt, out_idx, out_dist, st))) return rc;
    if ((rc = conn_device_impl(ctx, out_idx, out_dist, n, k, false, conn, st, true))) return rc;
    return ok_form(st, opt, (int)d);
}

int32_t scrust_cuda_neighbors_graph(scrust_context* ctx, const float* x, uint64_t n, uint64_t d, uint32_t k,
                                    const scrust_knn_options* opt, uint32_t* out_idx, float* out_dist,
                                    scrust_csr** conn, scrust_status* st) {
    int32_t rc = check_knn_args(n, d, k, st);
    if (rc) return rc;
    if ((rc = check_options(opt, st))) return rc;
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!x || !out_idx || !out_dist || !conn) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    float* dx = (float*)ws_get(ctx, SLOT_HOST_IN, sizeof(float) * n * d, &e);
    uint32_t* di = (uint32_t*)ws_get(ctx, SLOT_HOST_IDX, sizeof(uint32_t) * n * k, &e);
    float* dd = (float*)ws_get(ctx, SLOT_HOST_DIST, sizeof(float) * n * k, &e);
    if (!dx || !di || !dd) return cuda_fail(st, e, "workspace");
    if ((e = cudaMemcpyAsync(dx, x, sizeof(float) * n * d, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(st, e, "upload");
    if ((rc = knn_device_impl(ctx, dx, n, d, k, opt, di, dd, st))) return rc;
    // The neighbour lists download on the copy stream while the
    // connectivities run on the main one.
    if ((e = cudaEventRecord(ctx->copy_ev, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev, 0)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_idx, di, sizeof(uint32_t) * n * k, cudaMemcpyDeviceToHost, ctx->copy_stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out_dist, dd, sizeof(float) * n * k, cudaMemcpyDeviceToHost, ctx->copy_stream)) !=
            cudaSuccess) {
        cudaStreamSynchronize(ctx->copy_stream);
        return cuda_fail(st, e, "download");
    }
    scrust_csr* dev = nullptr;
    bool streamed = false;
    if ((rc = conn_device_impl(ctx, di, dd, n, k, false, &dev, st, true, true, &streamed))) {
        cudaStreamSynchronize(ctx->copy_stream);
        return rc;
    }
    rc = streamed ? csr_to_host_streamed(ctx, dev, conn, st) : csr_to_host(ctx, dev, conn, st);
    ctx->csr_pool.push_back(dev->buf);
    delete dev;
    if ((e = cudaStreamSynchronize(ctx->copy_stream)) != cudaSuccess) {
        if (!rc) {
            scrust_csr_free(*conn);
            *conn = nullptr;
        }
        return cuda_fail(st, e, "download");
    }
    if (rc) return rc;
    if ((rc = collect_device_errors(ctx, st))) return rc;
    return ok_form(st, opt, (int)d);
}

int32_t scrust_cuda_synchronize(scrust_context* ctx, scrust_status* st) {
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    return collect_device_errors(ctx, st);
}

uint64_t scrust_csr_n_rows(const scrust_csr* c) { return c ? c->n_rows : 0; }
uint64_t scrust_csr_n_cols(const scrust_csr* c) { return c ? c->n_cols : 0; }

uint64_t scrust_csr_nnz(const scrust_csr* c) {
    if (!c) return 0;
    if (c->nnz != UINT64_MAX) return c->nnz;
    uint32_t nnz = 0;
    scrust_csr* m = const_cast<scrust_csr*>(c);
    if (c->owner) {
        std::lock_guard<std::mutex> lock(c->owner->mu);
        DeviceGuard device_guard(c->owner->device);
        if (cudaMemcpyAsync(&nnz, c->buf.indptr + c->n_rows, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            c->owner->stream) == cudaSuccess &&
            cudaStreamSynchronize(c->owner->stream) == cudaSuccess)
            m->nnz = nnz;
        else
            cudaGetLastError();
    }
    return c->nnz == UINT64_MAX ? 0 : c->nnz;
}

int32_t scrust_csr_on_device(const scrust_csr* c) { return c ? c->on_device : 0; }
const uint32_t* scrust_csr_indptr(const scrust_csr* c) {
    return c ? (c->on_device ? c->buf.indptr : c->pinned ? c->p_indptr : c->h_indptr.data()) : nullptr;
}
const uint32_t* scrust_csr_indices(const scrust_csr* c) {
    return c ? (c->on_device ? c->buf.indices : c->pinned ? c->p_indices : c->h_indices.data()) : nullptr;
}
const float* scrust_csr_values(const scrust_csr* c) {
    return c ? (c->on_device ? c->buf.values : c->pinned ? c->p_values : c->h_values.data()) : nullptr;
}

void scrust_csr_free(scrust_csr* c) {
    if (!c) return;
    if (c->on_device && c->owner) return_csr_buffers(c->owner, c->buf);
    if (c->pinned) pinned_give(c->pinned, c->pinned_bytes);
    delete c;
}

void scrust_cuda_set_timing(scrust_context* ctx, int32_t enable) {
    if (!ctx) return;
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->timing = enable != 0;
}

int32_t scrust_cuda_phase_times(scrust_context* ctx, float* ms, int32_t max_phases) {
    if (!ctx || !ms) return 0;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int written = 0;
    int prev = PH_START;
    if (!ctx->ev_recorded[PH_START]) return 0;
    for (int p = PH_PREP; p <= PH_CONN && written < max_phases; ++p) {
        float t = 0.f;
        if (ctx->ev_recorded[p] && cudaEventElapsedTime(&t, ctx->ev[prev], ctx->ev[p]) == cudaSuccess) {
            prev = p;
        } else {
            cudaGetLastError();
            t = 0.f;
        }
        ms[written++] = t;
    }
    // Inside the candidates phase of an ordered solve: the first sweep pass,
    // the building of the second pass's tile lists, the second pass, and the
    // first collect pass (k <= 32).
    const int sub[4][2] = {{PH_PREP, PH_PASS1}, {PH_PASS1, PH_LISTS}, {PH_LISTS, PH_PASS2}, {PH_PASS2, PH_COLLECT1}};
    for (int i = 0; i < 4 && written < max_phases; ++i) {
        float t = 0.f;
        if (!(ctx->ev_recorded[sub[i][0]] && ctx->ev_recorded[sub[i][1]] &&
              cudaEventElapsedTime(&t, ctx->ev[sub[i][0]], ctx->ev[sub[i][1]]) == cudaSuccess)) {
            cudaGetLastError();
            t = 0.f;
        }
        ms[written++] = t;
    }
    return written;
}

uint64_t scrust_cuda_launch_count(const scrust_context* ctx) { return ctx ? ctx->launches : 0; }

int32_t scrust_cuda_kernel_stats(scrust_context* ctx, int32_t enable, uint64_t* out, int32_t max_words) {
    if (!ctx) return 0;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    constexpr size_t bytes = sizeof(unsigned long long) * kStatWords * kStatSlots;
    if (enable && !ctx->d_stats) {
        if (cudaMalloc(&ctx->d_stats, bytes) != cudaSuccess) {
            cudaGetLastError();
            ctx->d_stats = nullptr;
            return 0;
        }
        cudaMemsetAsync(ctx->d_stats, 0, bytes, ctx->stream);
    }
    int written = 0;
    if (ctx->d_stats && out && max_words > 0) {
        // Words 0-15: every launch together; then 16 words per slot.
        unsigned long long h[kStatWords * (kStatSlots + 1)] = {0};
        if (cudaMemcpyAsync(h + kStatWords, ctx->d_stats, bytes, cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess &&
            cudaStreamSynchronize(ctx->stream) == cudaSuccess) {
            for (int s = 1; s <= kStatSlots; s++)
                for (int i = 0; i < kStatWords; i++) h[i] += h[kStatWords * s + i];
            written = std::min(max_words, kStatWords * (kStatSlots + 1));
            for (int i = 0; i < written; i++) out[i] = h[i];
        }
        cudaMemsetAsync(ctx->d_stats, 0, bytes, ctx->stream);
    }
    if (!enable && ctx->d_stats) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->d_stats);
        ctx->d_stats = nullptr;
    }
    cudaGetLastError();
    return written;
}

const char* scrust_cuda_version(void) { return "scrust-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
