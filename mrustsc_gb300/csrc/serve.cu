// serve.cu -- a query service over a reference atlas resident in HBM.
//
// Requests (query cells) arrive from any host thread.  A scheduler thread
// admits them into batches, memory budget and free slots permitting, and runs
// each batch as one query-versus-atlas solve on a slot: its own context,
// stream and workspace.  Requests that arrive while other batches are on the
// GPU are admitted as soon as a slot and budget free up, so batches on
// different slots overlap on the device (continuous batching).  A solve is
// the tensor-form sweep of the batch's rows against the atlas, the exact
// rerank, and per-row directed connectivities (the rows of smooth_knn and exp
// weights, no symmetrisation).  For k <= 32 the atlas is ordered once when the
// service starts, and every batch is routed to its cells: threshold passes
// over the tiles of their cells and neighbouring cells and over the tiles the
// balls keep, then one collect pass, each row block's tiles split over column
// segments that share its rows' thresholds (order.cu).
// Every result is exact, so a request's output does not depend on what it was
// batched with.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace scrust {

using Clock = std::chrono::steady_clock;

struct ServeRequest {
    uint64_t id = 0;
    std::vector<float> q;
    uint64_t nq = 0;
    std::vector<uint32_t> idx;
    std::vector<float> dist;
    std::vector<uint32_t> indptr, indices;
    std::vector<float> values;
    int32_t code = SCRUST_OK;
    std::string msg;
    bool done = false;
    Clock::time_point t_submit, t_done;
};

template <class T>
struct Pinned {
    T* p = nullptr;
    size_t cap = 0;
    bool grow(size_t n) {
        if (n <= cap) return true;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaMallocHost((void**)&p, sizeof(T) * n) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cap = n;
        return true;
    }
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

struct ServeSlot {
    scrust_context* ctx = nullptr;
    bool busy = false;
    std::vector<ServeRequest*> reqs;
    uint64_t cells = 0;
    cudaEvent_t done = nullptr;
    Pinned<float> h_q, h_dist, h_val;
    Pinned<uint32_t> h_idx, h_ptr, h_ind;
    CsrBuffers csr;
    int32_t launch_code = SCRUST_OK;
    std::string launch_msg;
};

}  // namespace scrust

struct scrust_server {
    int device = 0;
    uint64_t m = 0;
    int d = 0, k = 0;
    int64_t m_pad = 0;
    scrust_knn_options opts{};
    bool bf16 = false;
    // The atlas, resident: rows, means, tensor operands (B), and the words
    // max centred norm, max quantisation radius, max |b_hat|.
    float* atlas = nullptr;
    double* means = nullptr;
    void* B16 = nullptr;
    uint32_t* words = nullptr;
    // The atlas ordered once (k <= 32): queries are routed to its cells and
    // sweep only the tiles that can hold their neighbours.
    scrust::AtlasOrder order;
    bool ordered = false;
    int64_t routed_min = 0;  // batches of at least this many rows are routed
    uint64_t budget = 0, atlas_bytes = 0, max_batch_cells = 0, bytes_per_cell = 0;
    std::vector<scrust::ServeSlot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<scrust::ServeRequest*> pending;
    std::unordered_map<uint64_t, scrust::ServeRequest*> reqs;
    uint64_t next_id = 1;
    std::thread worker;
    bool stop = false;
    uint64_t batches = 0, requests_done = 0, max_inflight = 0, cells_done = 0;
};

namespace scrust {

namespace {

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

constexpr int64_t kRoutedMinQueries = 1;

// Query rows of one batch against the atlas, on the slot's stream.
int32_t cross_enqueue(scrust_server* sv, scrust_context* ctx, const float* dq, int64_t q, uint32_t* d_idx,
                      float* d_dist, CsrBuffers* csr, scrust_status* st) {
    Reference ref;
    ref.rows = sv->atlas;
    ref.n = (int64_t)sv->m;
    ref.n_pad = sv->m_pad;
    ref.d = sv->d;
    ref.means = sv->means;
    ref.words = sv->words;
    ref.B16 = sv->B16;
    ref.bf16 = sv->bf16;
    // A routed solve visits only the tiles near the batch's rows (measured
    // at 500k atlas cells: 0.6 ms against 0.8 ms for one query, 1.3 against
    // 2.0 ms for 1000, 4.9 against 14.3 ms for 20,000); the sweep of every
    // tile stays for unordered atlases.
    const bool routed = sv->ordered && q >= sv->routed_min;
    int32_t rc = routed ? cross_ordered_enqueue(ctx, sv->order, sv->atlas, sv->means, sv->words, dq, q, sv->k, d_idx,
                                                d_dist, st)
                        : cross_knn_enqueue(ctx, ref, dq, q, sv->k, -1, d_idx, d_dist, st);
    if (rc) return rc;
    return run_query_connectivities(ctx, d_idx, d_dist, q, sv->k, csr, st);
}

bool grow_csr(CsrBuffers* b, uint64_t rows, uint64_t nnz) {
    if (b->rows_cap >= rows && b->nnz_cap >= nnz) return true;
    cudaFree(b->indptr);
    cudaFree(b->indices);
    cudaFree(b->values);
    *b = CsrBuffers{};
    if (cudaMalloc(&b->indptr, sizeof(uint32_t) * (rows + 1)) != cudaSuccess ||
        cudaMalloc(&b->indices, sizeof(uint32_t) * std::max<uint64_t>(nnz, 1)) != cudaSuccess ||
        cudaMalloc(&b->values, sizeof(float) * std::max<uint64_t>(nnz, 1)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    b->rows_cap = rows;
    b->nnz_cap = nnz;
    return true;
}

// Starts one batch on a free slot (the scheduler thread only).
void launch_batch(scrust_server* sv, ServeSlot& sl) {
    scrust_status st{};
    scrust_context* ctx = sl.ctx;
    const int d = sv->d, k = sv->k;
    const uint64_t q = sl.cells;
    sl.launch_code = SCRUST_OK;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e = cudaSuccess;
    int32_t rc = SCRUST_OK;
    if (!sl.h_q.grow(q * d) || !sl.h_idx.grow(q * k) || !sl.h_dist.grow(q * k) || !sl.h_ptr.grow(q + 1) ||
        !sl.h_ind.grow(q * k) || !sl.h_val.grow(q * k) || !grow_csr(&sl.csr, q, q * k)) {
        rc = fail(&st, SCRUST_OOM, "serve: batch buffers");
    } else {
        uint64_t o = 0;
        for (ServeRequest* r : sl.reqs) {
            memcpy(sl.h_q.p + o * d, r->q.data(), sizeof(float) * r->nq * d);
            o += r->nq;
        }
        float* dq = (float*)ws_get(ctx, SLOT_HOST_IN, sizeof(float) * q * d, &e);
        uint32_t* di = (uint32_t*)ws_get(ctx, SLOT_HOST_IDX, sizeof(uint32_t) * q * k, &e);
        float* dd = (float*)ws_get(ctx, SLOT_HOST_DIST, sizeof(float) * q * k, &e);
        if (!dq || !di || !dd) {
            rc = cuda_fail(&st, e, "serve: workspace");
        } else if ((e = cudaMemcpyAsync(dq, sl.h_q.p, sizeof(float) * q * d, cudaMemcpyHostToDevice, ctx->stream)) !=
                   cudaSuccess) {
            rc = cuda_fail(&st, e, "serve: upload");
        } else {
            rc = cross_enqueue(sv, ctx, dq, (int64_t)q, di, dd, &sl.csr, &st);
            if (rc == SCRUST_OK &&
                ((e = cudaMemcpyAsync(sl.h_idx.p, di, sizeof(uint32_t) * q * k, cudaMemcpyDeviceToHost, ctx->stream)) !=
                     cudaSuccess ||
                 (e = cudaMemcpyAsync(sl.h_dist.p, dd, sizeof(float) * q * k, cudaMemcpyDeviceToHost, ctx->stream)) !=
                     cudaSuccess ||
                 (e = cudaMemcpyAsync(sl.h_ptr.p, sl.csr.indptr, sizeof(uint32_t) * (q + 1), cudaMemcpyDeviceToHost,
                                      ctx->stream)) != cudaSuccess ||
                 (e = cudaMemcpyAsync(sl.h_ind.p, sl.csr.indices, sizeof(uint32_t) * q * k, cudaMemcpyDeviceToHost,
                                      ctx->stream)) != cudaSuccess ||
                 (e = cudaMemcpyAsync(sl.h_val.p, sl.csr.values, sizeof(float) * q * k, cudaMemcpyDeviceToHost,
                                      ctx->stream)) != cudaSuccess))
                rc = cuda_fail(&st, e, "serve: download");
        }
    }
    if (rc == SCRUST_OK && (e = cudaEventRecord(sl.done, ctx->stream)) != cudaSuccess)
        rc = cuda_fail(&st, e, "serve: event");
    if (rc != SCRUST_OK) {
        sl.launch_code = rc;
        sl.launch_msg = st.message;
    }
    sl.busy = true;
}

// Hands a finished batch's rows back to its requests (the scheduler thread).
void finish_batch(scrust_server* sv, ServeSlot& sl) {
    scrust_status st{};
    int32_t rc = sl.launch_code;
    std::string msg = sl.launch_msg;
    if (rc == SCRUST_OK) {
        std::lock_guard<std::mutex> lock(sl.ctx->mu);
        DeviceGuard device_guard(sl.ctx->device);
        rc = collect_device_errors(sl.ctx, &st);
        if (rc) msg = st.message;
    }
    const int k = sv->k;
    uint64_t o = 0;
    const auto now = Clock::now();
    std::lock_guard<std::mutex> lock(sv->mu);
    if (rc == SCRUST_OK) {
        // The rows' connectivity pointers must be a non-decreasing run
        // within the q x k entries the batch allocated.
        bool sane = sl.h_ptr.p[0] == 0;
        for (uint64_t i = 0; sane && i < sl.cells; ++i)
            sane = sl.h_ptr.p[i + 1] >= sl.h_ptr.p[i] && sl.h_ptr.p[i + 1] <= sl.cells * (uint64_t)k;
        if (!sane) {
            rc = SCRUST_KERNEL;
            msg = "serve: inconsistent connectivity rows";
        }
    }
    for (ServeRequest* r : sl.reqs) {
        if (rc == SCRUST_OK) {
            r->idx.assign(sl.h_idx.p + o * k, sl.h_idx.p + (o + r->nq) * k);
            r->dist.assign(sl.h_dist.p + o * k, sl.h_dist.p + (o + r->nq) * k);
            const uint32_t base = sl.h_ptr.p[o], end = sl.h_ptr.p[o + r->nq];
            r->indptr.resize(r->nq + 1);
            for (uint64_t i = 0; i <= r->nq; ++i) r->indptr[i] = sl.h_ptr.p[o + i] - base;
            r->indices.assign(sl.h_ind.p + base, sl.h_ind.p + end);
            r->values.assign(sl.h_val.p + base, sl.h_val.p + end);
        }
        r->code = rc;
        r->msg = msg;
        r->done = true;
        r->t_done = now;
        r->q.clear();
        r->q.shrink_to_fit();
        o += r->nq;
    }
    sv->requests_done += sl.reqs.size();
    sv->cells_done += sl.cells;
    sl.reqs.clear();
    sl.cells = 0;
    sl.busy = false;
    sv->cv_done.notify_all();
}

void scheduler(scrust_server* sv) {
    DeviceGuard device_guard(sv->device);
    for (;;) {
        bool progressed = false;
        for (ServeSlot& sl : sv->slots)
            if (sl.busy) {
                const cudaError_t q = sl.launch_code == SCRUST_OK ? cudaEventQuery(sl.done) : cudaSuccess;
                if (q == cudaSuccess) {
                    finish_batch(sv, sl);
                    progressed = true;
                } else if (q != cudaErrorNotReady) {
                    cudaGetLastError();
                    sl.launch_code = SCRUST_KERNEL;
                    sl.launch_msg = "serve: a batch failed on the device";
                    finish_batch(sv, sl);
                    progressed = true;
                }
            }
        for (ServeSlot& sl : sv->slots) {
            if (sl.busy) continue;
            {
                std::lock_guard<std::mutex> lock(sv->mu);
                uint64_t inflight = 0;
                for (const ServeSlot& o : sv->slots) inflight += o.busy ? o.cells : 0;
                // Admit in arrival order while the batch and the budget allow;
                // a request larger than a batch runs alone.
                while (!sv->pending.empty()) {
                    ServeRequest* r = sv->pending.front();
                    const bool first = sl.reqs.empty();
                    if (!first && sl.cells + r->nq > sv->max_batch_cells) break;
                    if (!first && (inflight + sl.cells + r->nq) * sv->bytes_per_cell + sv->atlas_bytes > sv->budget)
                        break;
                    if (first && inflight > 0 && (inflight + r->nq) * sv->bytes_per_cell + sv->atlas_bytes > sv->budget)
                        break;
                    sv->pending.pop_front();
                    sl.reqs.push_back(r);
                    sl.cells += r->nq;
                }
            }
            if (sl.reqs.empty()) break;
            launch_batch(sv, sl);
            progressed = true;
            std::lock_guard<std::mutex> lock(sv->mu);
            sv->batches++;
            uint64_t busy = 0;
            for (const ServeSlot& o : sv->slots) busy += o.busy ? 1 : 0;
            sv->max_inflight = std::max(sv->max_inflight, busy);
        }
        std::unique_lock<std::mutex> lock(sv->mu);
        bool any_busy = false;
        for (const ServeSlot& o : sv->slots) any_busy |= o.busy;
        if (sv->stop && sv->pending.empty() && !any_busy) break;
        if (!progressed) {
            if (any_busy)
                sv->cv_work.wait_for(lock, std::chrono::microseconds(50));
            else
                sv->cv_work.wait_for(lock, std::chrono::milliseconds(5));
        }
    }
}

void destroy_server(scrust_server* sv) {
    for (ServeSlot& sl : sv->slots) {
        if (sl.done) cudaEventDestroy(sl.done);
        cudaFree(sl.csr.indptr);
        cudaFree(sl.csr.indices);
        cudaFree(sl.csr.values);
        if (sl.ctx) scrust_cuda_context_destroy(sl.ctx);
    }
    atlas_order_free(&sv->order);
    cudaFree(sv->atlas);
    cudaFree(sv->means);
    cudaFree(sv->B16);
    cudaFree(sv->words);
    for (auto& kv : sv->reqs) delete kv.second;
    delete sv;
}

}  // namespace

}  // namespace scrust

using namespace scrust;

extern "C" {

scrust_server* scrust_serve_create(int32_t device, const float* atlas, uint64_t m, uint64_t d, uint32_t k,
                                   const scrust_knn_options* opt, uint64_t budget_bytes, uint64_t max_batch_cells,
                                   uint32_t n_slots, scrust_status* st) {
    if (!atlas || m == 0 || d == 0) {
        fail(st, SCRUST_SHAPE, "expected a non-empty atlas");
        return nullptr;
    }
    if (d > 61) {
        fail(st, SCRUST_SHAPE, "expected at most 61 dimensions for the served atlas, got %llu", (unsigned long long)d);
        return nullptr;
    }
    if (k == 0 || k > 128 || (uint64_t)k > m) {
        fail(st, SCRUST_INVALID_PARAMETER, "k must be between 1 and min(128, atlas cells), got %u", k);
        return nullptr;
    }
    if (m >= 0xffffff00ull) {
        fail(st, SCRUST_SHAPE, "expected fewer than 2^32 atlas cells");
        return nullptr;
    }
    if (opt && (opt->mode != SCRUST_MODE_EXACT || opt->metric != SCRUST_METRIC_EUCLIDEAN)) {
        fail(st, SCRUST_INVALID_PARAMETER, "the service runs exact Euclidean solves");
        return nullptr;
    }
    scrust_server* sv = new (std::nothrow) scrust_server;
    if (!sv) {
        fail(st, SCRUST_OOM, "host allocation failed");
        return nullptr;
    }
    sv->device = device;
    DeviceGuard create_guard(device);  // the slots' events and the atlas live on `device`
    sv->m = m;
    sv->d = (int)d;
    sv->k = (int)k;
    sv->m_pad = (int64_t)round_up(m, 256);
    scrust_knn_options_default(&sv->opts);
    if (opt) sv->opts = *opt;
    sv->bf16 = sv->opts.precision == SCRUST_PRECISION_BF16;
    const uint32_t ns = std::max<uint32_t>(1, std::min<uint32_t>(n_slots ? n_slots : 2, 8));
    sv->slots.resize(ns);
    for (ServeSlot& sl : sv->slots) {
        sl.ctx = scrust_cuda_context_create(device, st);
        if (!sl.ctx || cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            if (sl.ctx) cuda_fail(st, cudaGetLastError(), "serve: event");
            destroy_server(sv);
            return nullptr;
        }
    }
    // The atlas: rows, means, norms for the scale, B operands, and the maxima.
    const int dp = (int)(d + 3) / 4 * 4;
    const int mean_blocks = (int)((m + 2047) / 2048);
    cudaError_t e = cudaSuccess;
    {
        scrust_context* c0 = sv->slots[0].ctx;
        std::lock_guard<std::mutex> lock(c0->mu);
        DeviceGuard device_guard(device);
        cudaStream_t s = c0->stream;
        e = cudaMalloc(&sv->atlas, sizeof(float) * m * d);
        if (e == cudaSuccess) e = cudaMalloc(&sv->means, sizeof(double) * d * (mean_blocks + 1));
        if (e == cudaSuccess) e = cudaMalloc(&sv->B16, (size_t)sv->m_pad * 128);
        if (e == cudaSuccess) e = cudaMalloc(&sv->words, 64);
        void* A16 = nullptr;
        float* tmp = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&A16, (size_t)sv->m_pad * 128);
        if (e == cudaSuccess) e = cudaMalloc(&tmp, sizeof(float) * 4 * (size_t)sv->m_pad);
        if (e == cudaSuccess) e = cudaMemsetAsync(sv->words, 0, 64, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(sv->atlas, atlas, sizeof(float) * m * d, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_column_means(sv->atlas, (int64_t)m, (int)d, false, sv->means, sv->means + d, s);
        if (e == cudaSuccess)
            e = launch_centre_transpose(sv->atlas, (int64_t)m, sv->m_pad, (int)d, dp, sv->means, nullptr, tmp,
                                        tmp + sv->m_pad, nullptr, sv->words, s);
        if (e == cudaSuccess)
            e = launch_tensor_operands(sv->atlas, (int64_t)m, sv->m_pad, (int)d, sv->means, sv->words, false, sv->bf16,
                                       nullptr, A16, sv->B16, tmp + 2 * sv->m_pad, tmp + 3 * sv->m_pad, sv->words + 1,
                                       sv->words + 2, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaFree(A16);
        cudaFree(tmp);
        // The ordering the query solves route through (k <= 32, as the
        // threshold pass needs; an atlas of fewer than 1024 cells is swept
        // whole).
        if (e == cudaSuccess && k <= 32 && m >= 1024) {
            if (atlas_order_build(c0, sv->atlas, (int64_t)m, (int)d, sv->means, sv->words, sv->bf16, &sv->order, st)) {
                destroy_server(sv);
                return nullptr;
            }
            sv->ordered = true;
            // SCRUST_ROUTED_MIN_QUERIES moves the batch size from which
            // queries are routed (a tuning knob; every result is exact
            // either way).
            sv->routed_min = kRoutedMinQueries;
            if (const char* v = getenv("SCRUST_ROUTED_MIN_QUERIES")) {
                const long long r = atoll(v);
                if (r > 0) sv->routed_min = r;
            }
        }
    }
    if (e != cudaSuccess) {
        cuda_fail(st, e, "serve: atlas");
        cudaGetLastError();
        destroy_server(sv);
        return nullptr;
    }
    // Budget: the atlas plus, per admitted cell, its lists, operands,
    // outputs and connectivities.
    sv->atlas_bytes = sizeof(float) * m * d + (size_t)sv->m_pad * 128 + sizeof(double) * d * (mean_blocks + 1);
    if (sv->ordered)  // list-order operands and rows, the permutation, anchors and balls
        sv->atlas_bytes += (size_t)sv->m_pad * 128 + sizeof(float) * m * padded_row_floats((int)d) + 4 * m +
                           (size_t)sv->order.anchors_pad * 128 + 4 * (size_t)sv->order.anchors * (kAnchorNeighbours + 2) +
                           4 * 66 * (size_t)sv->order.segs;
    sv->bytes_per_cell = (uint64_t)(2 * 16) * (std::max(64, (2 * (int)k + 32 + 31) / 32 * 32) + 128) * 8 + 512 +
                         (uint64_t)k * 24 + (uint64_t)d * 8;
    sv->budget = budget_bytes ? budget_bytes : (uint64_t)150 << 30;
    if (sv->budget < sv->atlas_bytes + sv->bytes_per_cell * 256) {
        fail(st, SCRUST_OOM, "the memory budget does not hold the atlas and one batch");
        destroy_server(sv);
        return nullptr;
    }
    sv->max_batch_cells = max_batch_cells ? max_batch_cells : 65536;
    sv->worker = std::thread(scheduler, sv);
    ok(st);
    return sv;
}

uint64_t scrust_serve_submit(scrust_server* sv, const float* queries, uint64_t q, scrust_status* st) {
    if (!sv) {
        fail(st, SCRUST_SHAPE, "expected a server");
        return 0;
    }
    if (!queries || q == 0) {
        fail(st, SCRUST_SHAPE, "expected at least one query cell");
        return 0;
    }
    ServeRequest* r = new (std::nothrow) ServeRequest;
    if (!r) {
        fail(st, SCRUST_OOM, "host allocation failed");
        return 0;
    }
    try {
        r->q.assign(queries, queries + q * sv->d);
    } catch (...) {
        delete r;
        fail(st, SCRUST_OOM, "host allocation failed");
        return 0;
    }
    r->nq = q;
    r->t_submit = Clock::now();
    uint64_t id;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        id = r->id = sv->next_id++;
        sv->reqs[id] = r;
        sv->pending.push_back(r);
    }
    sv->cv_work.notify_one();
    ok(st);
    return id;
}

int32_t scrust_serve_wait(scrust_server* sv, uint64_t ticket, uint32_t* out_idx, float* out_dist,
                          scrust_csr** out_conn, double* latency_ms, scrust_status* st) {
    if (!sv) return fail(st, SCRUST_SHAPE, "expected a server");
    ServeRequest* r;
    {
        std::unique_lock<std::mutex> lock(sv->mu);
        auto it = sv->reqs.find(ticket);
        if (it == sv->reqs.end()) return fail(st, SCRUST_INVALID_PARAMETER, "unknown ticket %llu", (unsigned long long)ticket);
        r = it->second;
        sv->cv_done.wait(lock, [&] { return r->done; });
        sv->reqs.erase(it);
    }
    int32_t rc = r->code;
    if (rc == SCRUST_OK) {
        if (out_idx) memcpy(out_idx, r->idx.data(), sizeof(uint32_t) * r->idx.size());
        if (out_dist) memcpy(out_dist, r->dist.data(), sizeof(float) * r->dist.size());
        if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        if (out_conn) {
            scrust_csr* c = new (std::nothrow) scrust_csr;
            if (!c) {
                delete r;
                return fail(st, SCRUST_OOM, "host allocation failed");
            }
            c->n_rows = r->nq;
            c->n_cols = sv->m;
            c->nnz = r->indices.size();
            c->on_device = 0;
            c->h_indptr = std::move(r->indptr);
            c->h_indices = std::move(r->indices);
            c->h_values = std::move(r->values);
            *out_conn = c;
        }
        ok(st);
    } else {
        fail(st, rc, "%s", r->msg.c_str());
    }
    delete r;
    return rc;
}

int32_t scrust_serve_stats(scrust_server* sv, uint64_t* out, int32_t max_words) {
    if (!sv || !out) return 0;
    std::lock_guard<std::mutex> lock(sv->mu);
    const uint64_t v[7] = {sv->batches, sv->requests_done, sv->max_inflight, sv->cells_done, sv->max_batch_cells,
                           sv->bytes_per_cell, (uint64_t)sv->slots.size()};
    const int n = std::min<int>(max_words, 7);
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return n;
}

void scrust_serve_destroy(scrust_server* sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    DeviceGuard device_guard(sv->device);
    destroy_server(sv);
}

}  // extern "C"
