// internal.h -- host-side types shared by the translation units of the
// library: the context (the analogue of the reference's MetalContext,
// crates/scrust-gpu/src/context.rs:12-91), its workspace arena, and the
// launch functions each .cu file provides.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "scrust_cuda.h"

namespace scrust {

// Named workspace slots; each grows on demand and is reused across calls.
enum Slot : int {
    SLOT_MEANS = 0,
    SLOT_COORDS_T,      // centred coordinates, transposed (plain form)
    SLOT_NORM2,         // squared centred norms per row (+inf on padding)
    SLOT_MARGIN,        // per-row candidate margin (s-space)
    SLOT_CNORM,         // per-row centred norm (for bounds)
    SLOT_LIST_IDS,
    SLOT_LIST_VALS,
    SLOT_LIST_CNT,
    SLOT_OVERFLOW,
    SLOT_FALLBACK_ROWS,
    SLOT_FALLBACK_SCRATCH,
    SLOT_XWORK,         // normalised (cosine) or centred (reference-snap) rows
    SLOT_NORM64,        // FP64 norms (cosine)
    SLOT_A16,           // tensor form operands
    SLOT_B16,
    SLOT_QERR,          // per-row quantisation error norms (tensor form)
    SLOT_HOST_IN,       // staging of host inputs
    SLOT_HOST_IDX,
    SLOT_HOST_DIST,
    SLOT_CONN_A,        // connectivities scratch
    SLOT_CONN_B,
    SLOT_CONN_C,
    SLOT_CONN_D,
    SLOT_CONN_E,
    SLOT_CONN_F,
    SLOT_CONN_G,
    SLOT_CONN_H,        // merged rows of the fuzzy union before they are placed
    SLOT_SCAN,
    SLOT_MISC,
    SLOT_WORKQ,
    SLOT_ORDER,         // row ordering: anchors, permutation, priority tiles
    SLOT_PRUNE,         // tile balls and the tile lists of the second sweep pass
    SLOT_XSORTED,       // working rows in list order (ordered solves)
    SLOT_BATCH,         // batch layout maps, work order, thresholds
    SLOT_BATCH_TABLE,   // batch sample table
    SLOT_THETA,         // list thresholds of an unordered tensor-form solve
    SLOT_ROWTHETA,      // per-row shared thresholds across column segments
    SLOT_TOPK,          // a threshold pass's register top-K per list
    SLOT_RERANK_BIG,    // rows for the rerank's second sorted pass
    SLOT_QTERMS,        // per-query-row bound terms of a query-versus-reference solve
    SLOT_QSCRATCH,      // scratch operands of a query-versus-reference solve
    SLOT_XORDER,        // routing, priority tiles and pruning of a query solve against an ordered atlas
    SLOT_BATCH_GIDX,    // a batch's neighbour ids made batch-global for its connectivities
    SLOT_UMAP,          // the UMAP layout's schedules, moves, transpose and second layout
    SLOT_PCA,           // PCA: sketch, bases, CSC copy, Grams, small factors
    SLOT_COUNT
};

struct Workspace {
    void* ptr[SLOT_COUNT] = {};
    size_t bytes[SLOT_COUNT] = {};
};

// Makes `device` current for the scope of a public entry point and gives the
// calling thread its previous device back on return, so a call on a context
// never changes which device the caller's own CUDA work goes to.
class DeviceGuard {
public:
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev_) != cudaSuccess) {
            cudaGetLastError();
            prev_ = -1;
        }
        if (prev_ != device) cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int now = -1;
        if (prev_ >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev_) cudaSetDevice(prev_);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;

private:
    int prev_ = -1;
};

struct CsrBuffers {
    uint32_t* indptr = nullptr;
    uint32_t* indices = nullptr;
    float* values = nullptr;
    size_t rows_cap = 0;   // indptr holds rows_cap + 1 entries
    size_t nnz_cap = 0;
};

// A kNN graph's connectivities CSR downloaded while it is built: the fuzzy
// union, its row scan and the placing of its rows run range by range
// (kCsrRanges row ranges, each range's offsets continuing the last one's),
// and each placed range goes down on the copy stream while the later ranges
// merge.
constexpr int kCsrRanges = 8;
struct CsrStream {
    cudaEvent_t merged[kCsrRanges] = {};  // on the main stream, after each range is placed
    uint32_t* h_bounds = nullptr;         // pinned: the CSR offset past each range
};

}  // namespace scrust

struct scrust_context {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // downloads that overlap later kernels on `stream`
    cudaEvent_t copy_ev = nullptr;
    scrust::CsrStream csr_stream;        // the streamed download of kNN-graph connectivities
    std::mutex mu;
    scrust::Workspace ws;
    int* d_err = nullptr;          // scrust::DERR_COUNT ints
    uint32_t* d_counter = nullptr; // small device counters (fallback rows, work queue)
    std::vector<scrust::CsrBuffers> csr_pool;
    PFN_cuTensorMapEncodeTiled_v12000 encode_tiled = nullptr;
    uint64_t launches = 0;              // kernels enqueued so far
    // Kernel counters when statistics are on: 16 words per sweep launch of a
    // solve, for its first three launches and all later ones together.
    unsigned long long* d_stats = nullptr;
    int stats_launch = 0;               // sweep launches of the current solve so far
    bool timing = false;
    cudaEvent_t ev[9] = {};             // phase boundaries: prep | candidates | rerank | connectivities, and
    bool ev_recorded[9] = {};           // inside candidates: sweep pass 1 | tile lists | pass 2 | collect 1
    std::vector<std::pair<const void*, int>> smem_limits;  // dynamic shared memory limits already set
    std::vector<const void*> carveouts;                      // kernels whose shared-memory carveout is set
};

struct scrust_csr {
    uint64_t n_rows = 0;
    uint64_t n_cols = 0;
    uint64_t nnz = 0;
    int32_t on_device = 0;
    scrust_context* owner = nullptr;  // device CSRs return their buffers to this pool
    scrust::CsrBuffers buf;
    // Host arrays: either the vectors, or (downloads of a device graph) one
    // pinned slab from a process-wide pool holding indptr, indices, values.
    std::vector<uint32_t> h_indptr, h_indices;
    std::vector<float> h_values;
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    uint32_t* p_indptr = nullptr;
    uint32_t* p_indices = nullptr;
    float* p_values = nullptr;
};

namespace scrust {

// Phase boundary events (no-ops unless timing is enabled).
enum Phase {
    PH_START = 0, PH_PREP = 1, PH_CAND = 2, PH_RERANK = 3, PH_CONN = 4, PH_PASS1 = 5, PH_LISTS = 6, PH_PASS2 = 7,
    PH_COLLECT1 = 8, PH_COUNT = 9
};
static_assert(sizeof(scrust_context::ev) / sizeof(cudaEvent_t) == PH_COUNT, "one event per phase boundary");
void mark(scrust_context* ctx, Phase p);
unsigned long long* sweep_stats(scrust_context* ctx);

// Maps the device error block to a status, then clears it (synchronises).
int32_t collect_device_errors(scrust_context* ctx, scrust_status* st);

// Status helpers.
int32_t fail(scrust_status* st, int32_t code, const char* fmt, ...);
int32_t ok(scrust_status* st);
int32_t cuda_fail(scrust_status* st, cudaError_t e, const char* what);

// Raises a kernel's dynamic shared memory limit once per context (so that
// launches can be captured into a CUDA graph afterwards).
cudaError_t set_smem_limit(scrust_context* ctx, const void* func, int bytes);
// Preferred shared-memory carveout (percent of the unified L1/shared memory),
// set once per context and kernel.
cudaError_t set_smem_carveout(scrust_context* ctx, const void* func, int percent);

// Workspace access (may cudaMalloc; call with the context lock held).
void* ws_get(scrust_context* ctx, Slot slot, size_t bytes, cudaError_t* err);

// Parameters of one kNN solve on device-resident data.
struct KnnPlan {
    int64_t nq = 0, nr = 0;   // query rows, reference rows (equal for self-kNN)
    int d = 0, k = 0;
    bool self = true;         // query i is reference i + self_offset (exclude it)
    int64_t self_offset = 0;
    int form = SCRUST_FORM_PLAIN;
    int metric = SCRUST_METRIC_EUCLIDEAN;
    int mode = SCRUST_MODE_EXACT;
    int precision = SCRUST_PRECISION_FP16;
    int cap = 0;              // list capacity that triggers a prune
    int ctot = 0;             // list storage per (row, segment)
    int segments = 1;
    int max_ctas = 0;         // tensor sweep: CTAs at most (0: one per SM)
    // Tensor sweep, general passes: the per-row top-k kept in registers.
    // 0 = the narrowest that holds k (16 or 32; lists alone above 32), 16 or
    // 32 = that width (at least k), -1 = lists alone (warp-cooperative prunes).
    int topk_width = 0;
};

// Keys the rerank's warp path holds per row (the union of the row's lists);
// larger unions take the fallback.
constexpr int kRerankUnion = 1024;
// Lists are cut to at most max(kListFinalMin, kRerankUnion / lists per row)
// entries when a tensor-form work item ends.
constexpr int kListFinalMin = 64;

// Candidate lists as the candidate kernels write them and the rerank reads.
struct Lists {
    uint32_t* ids = nullptr;
    float* vals = nullptr;
    uint32_t* cnt = nullptr;       // [rows_pad * segments]
    uint32_t* overflow = nullptr;  // [rows_pad]
    int cap = 0, ctot = 0, segments = 1;
};

int32_t alloc_lists(scrust_context* ctx, int64_t rows_pad, Lists* lists, scrust_status* st);

// A spatial ordering of the rows of a self-kNN solve (order.cu): rows are
// grouped into cells around anchors and each 256-row work item of the tensor
// sweep gets the column tiles of its own and its anchors' neighbouring cells
// to visit first.
constexpr int kPrioMax = 64;           // priority tiles per work item
constexpr int kAnchorNeighbours = 16;  // neighbouring anchors per anchor
constexpr int64_t kMaxAnchors = 8192;
struct RowOrder {
    const uint32_t* perm = nullptr;      // sorted position -> original row
    const uint32_t* prio_order = nullptr;  // row blocks by decreasing priority-tile count
    const uint32_t* prio = nullptr;      // [items][kPrioMax] distinct column tiles, nearest cells first
    const uint32_t* prio_cnt = nullptr;  // [items], at least 1
    float* theta = nullptr;              // [n_pad * 2] list thresholds between the sweep passes
    const uint32_t* cell_of_pos = nullptr;  // [n] cell of each sorted position
    // The anchors behind the cells (a reference set ordered once keeps them
    // to route queries): their count, B operands in anchor order
    // (anchors_pad rows), walk places, the cells' first list positions in walk
    // order (anchors + 1) and each cell's neighbouring cells (anchors x
    // kAnchorNeighbours walk places).
    int64_t anchors = 0, anchors_pad = 0;
    const void* anchor_B16 = nullptr;
    const uint32_t* anchor_rank = nullptr;
    const uint32_t* cell_start = nullptr;
    const uint32_t* cell_nb = nullptr;
};
// Builds the ordering and leaves the tensor operands A16/B16 and their row
// terms bA/beps (n_pad rows each) in list order; bdelta/beps2 serve as
// scratch (the caller computes the list-order bounds afterwards).
int32_t build_row_order(scrust_context* ctx, const float* x, int64_t n, int d, const double* means,
                        uint32_t* max_bits, bool cosine, bool bf16, void* A16, void* B16, float* bA, float* beps,
                        float* bdelta, float* beps2, RowOrder* out, scrust_status* st);
struct TileLists;
// A reference set ordered once for query solves (the served atlas), device
// memory it owns: the B operands and rows in list order, the permutation, the
// anchors that route queries to cells, and the cell-segment balls of its
// column tiles.
struct AtlasOrder {
    int64_t m = 0, m_pad = 0, anchors = 0, anchors_pad = 0, segs = 0;
    int d = 0;
    bool bf16 = false;
    void* B16 = nullptr;             // m_pad rows of the B operand, list order
    uint32_t* perm = nullptr;        // list position -> atlas row
    float* rows = nullptr;           // atlas rows in list order, padded_row_floats(d) floats each
    void* anchor_B16 = nullptr;      // anchors_pad rows, anchor order
    uint32_t* anchor_rank = nullptr; // anchor -> walk place
    uint32_t* cell_start = nullptr;  // anchors + 1, by walk place
    uint32_t* cell_nb = nullptr;     // anchors x kAnchorNeighbours walk places
    float* seg_centre_t = nullptr;   // [64][segs] segment centres (zero past d)
    float* seg_radius = nullptr;     // [segs]
    uint32_t* seg_tile = nullptr;    // [segs] column tile of each segment
};
// Orders `atlas` (device rows) once: means and the maxima in `words` as the
// served atlas has them (max centred norm; the quantisation maxima are
// raised).  Synchronises the context's stream.
int32_t atlas_order_build(scrust_context* ctx, const float* atlas, int64_t m, int d, const double* means,
                          uint32_t* words, bool bf16, AtlasOrder* out, scrust_status* st);
void atlas_order_free(AtlasOrder* o);
// k <= 32 nearest atlas rows of each query row (input order outputs), exact:
// queries routed to their nearest anchor's cell and sorted by it, a threshold
// pass over priority tiles, another over the tiles the balls keep, a collect
// pass over both, the sorted rerank.  `words` are the atlas's.
int32_t cross_ordered_enqueue(scrust_context* ctx, const AtlasOrder& at, const float* atlas_rows, const double* means,
                              const uint32_t* words, const float* dq, int64_t q, int k, uint32_t* d_idx,
                              float* d_dist, scrust_status* st);
// After the priority pass: the column tiles each row block still has to
// visit, from tile bounding balls and the rows' thresholds (order.cu).
int32_t build_second_pass(scrust_context* ctx, const void* A16, bool bf16, int64_t n, int d, const RowOrder& order,
                          const float* bA, const float* bdelta, TileLists* out, scrust_status* st);
// Largest solve whose second-pass tile lists (row blocks x column tiles
// entries) the ordering accepts.
constexpr int64_t kOrderMaxRows = 8000000;

// prep.cu
cudaError_t launch_column_means(const float* x, int64_t n, int d, bool sequential, double* means,
                                double* partial, cudaStream_t s);
cudaError_t launch_normalise_rows(const float* x, int64_t n, int d, float* xn, double* norm64,
                                  int* d_err, cudaStream_t s);
// prep.cu: column means that only fix a centre (tensor form, d <= 64): f32
// block sums; `partial` as for launch_column_means.
cudaError_t launch_column_means_centre(const float* x, int64_t n, int d, double* means, double* partial,
                                       cudaStream_t s);
// prep.cu: the largest centred row norm only (tensor form, d <= 64).
cudaError_t launch_max_centred_norm(const float* x, int64_t n, int d, const double* means, uint32_t* max_norm_bits,
                                    int sm_count, cudaStream_t s);
cudaError_t launch_centre_transpose(const float* x, int64_t n, int64_t n_pad, int d, int dp,
                                    const double* means, float* coords_t, float* norm2,
                                    float* cnorm, float* xcentred, uint32_t* max_norm_bits,
                                    cudaStream_t s);
cudaError_t launch_margins(const float* cnorm, const float* norm2, int64_t n, int d, int mode,
                           int metric, int form, const uint32_t* max_norm_bits,
                           const float* qerr, const uint32_t* max_qerr_bits, float scale2,
                           float* margin, cudaStream_t s);

// knn_plain.cu
cudaError_t launch_plain_candidates(scrust_context* ctx, const KnnPlan& plan, const float* q_t,
                                    int64_t nq_pad, const float* r_t, int64_t nr_pad, int dp,
                                    const float* r_norm2, const float* margin, const Lists& lists);

// knn_tensor.cu
size_t tensor_smem_bytes();
// Row i of the operands is input row perm[i] (i when perm is null).
cudaError_t launch_tensor_operands(const float* x, int64_t n, int64_t n_pad, int d, const double* means,
                                   const uint32_t* max_norm_bits, bool cosine, bool bf16, const uint32_t* perm,
                                   void* A16, void* B16, float* bA, float* eps, uint32_t* max_eps_bits,
                                   uint32_t* max_bhat_bits, cudaStream_t s);
cudaError_t launch_tensor_bounds(int64_t n, const float* bA, const float* eps, const uint32_t* max_eps_bits,
                                 const uint32_t* max_bhat_bits, float* bdelta, float* beps2, cudaStream_t s);
// Explicit column tiles per row block of the query rows.
struct TileLists {
    const uint32_t* tiles = nullptr;
    const uint32_t* offset = nullptr;  // per row block; null: block * stride
    const uint32_t* count = nullptr;   // per row block
    int stride = 0;
    const uint32_t* order = nullptr;   // row blocks by decreasing count, or null
    // A second explicit list per row block, visited after the first
    // (`stride2` entries apart, `count2` per row block), or null.
    const uint32_t* tiles2 = nullptr;
    const uint32_t* count2 = nullptr;
    int stride2 = 0;
    // Without explicit tiles: per row block the column tile range [x, y) it
    // sweeps (a batch of independent solves laid out block-diagonally), or null.
    const uint2* range = nullptr;
    const uint32_t* row_map = nullptr;  // query row -> input row, 0xffffffff for padding; null: identity
    // Per query row, the smallest threshold of any of its lists (float_key,
    // initialised to 0xffffffff), shared by the column segments; or null.
    uint32_t* row_theta = nullptr;
};
// One pass of the tensor sweep.  `tiles` null: every column tile, outward
// from the diagonal.  `resume`: lists and thresholds continue from an earlier
// pass (counts in lists.cnt, thresholds in theta_io); theta_io, when given,
// receives each list's threshold as its row block ends.  `argmin_out` (k = 1
// only): no lists; per (row, column part) the smallest value and the 8-column
// group holding it, packed as float_key << 32 | (column / 8).
cudaError_t launch_tensor_candidates(scrust_context* ctx, const KnnPlan& plan, const void* A16, int64_t nq_pad,
                                     const void* B16, int64_t nr_pad, const float* bA, const float* bdelta,
                                     const float* beps2, const Lists& lists, bool bf16, const TileLists* tiles,
                                     bool resume, float* theta_io, int* grid_out, unsigned long long* stats,
                                     unsigned long long* argmin_out = nullptr, int pass_mode = 0,
                                     float* topk_out = nullptr);
// After a threshold pass that wrote its register top-K per list (topk_out,
// one column segment): each row's threshold from the k-th of both column
// parts' lists together, into both of its theta slots (knn_tensor.cu).
cudaError_t launch_merge_part_thresholds(const float* topk, int width, int64_t n, int64_t n_pad, int k,
                                         const float* bA, const float* bdelta, const float* beps2, float* theta,
                                         cudaStream_t s);
// Pass modes of launch_tensor_candidates (k <= 32, one column segment):
// thresholds only (register top-k, theta_io written, lists untouched), then
// collection at the fixed thresholds (appends only).
constexpr int kPassFull = 0, kPassThresholds = 1, kPassCollect = 2;
// Kernel counters: words per block, and blocks (the first three sweep
// launches of a solve, then all later ones).
constexpr int kStatWords = 16, kStatSlots = 4;

// Per-row bound of the candidate lists, as the rerank re-applies it: the
// plain form's additive margin, or the tensor form's (A, delta, eps2).
struct RowBounds {
    const float* margin = nullptr;
    const float* A = nullptr;
    const float* delta = nullptr;
    const float* eps2 = nullptr;
};

// rerank.cu.  With a permutation, list row s and list entry c stand for
// input rows perm[s] and perm[c]; outputs are written in input order.  With
// xs (the working rows in list order) and theta (each list's threshold at
// the end of the candidate pass) as well, no selection is needed.  List rows
// whose perm entry is 0xffffffff are padding and skipped.  row_lo/row_hi
// (per input row) confine a batch's solves: ids are reported relative to
// row_lo and the fallback scans [row_lo, row_hi).  xr_list: the reference
// rows by list entry when they are not xs (a query-versus-reference solve).
cudaError_t launch_rerank(scrust_context* ctx, const KnnPlan& plan, const float* qx,
                          const float* rx, const float* qnorm2, const float* rnorm2,
                          const double* qn64, const double* rn64, const float* qraw,
                          const float* rraw, const RowBounds& bounds, const Lists& lists,
                          const uint32_t* perm, const float* xs, const float* theta, uint32_t* out_idx,
                          float* out_dist, const uint32_t* row_lo = nullptr, const uint32_t* row_hi = nullptr,
                          const float* xr_list = nullptr, int xs_stride = 0, bool ids_only = false,
                          const uint32_t* qperm = nullptr);
// order.cu: row blocks sorted by decreasing count (stable) into `order`;
// `scratch` holds work_order_scratch(items) bytes.
size_t work_order_scratch(int items);
cudaError_t sort_by_work(scrust_context* ctx, const uint32_t* counts, int items, char* scratch, uint32_t* order);
// order.cu: rows of x in list order, xs[s] = x[perm[s]] (zeros where perm
// holds 0xffffffff), `stride` floats apart with zeros after the d-th.  The
// rerank reads such rows in 32-byte words: a multiple of 8 floats.
cudaError_t launch_gather_rows(const float* x, const uint32_t* perm, int64_t n, int d, int stride, float* xs,
                               cudaStream_t s);
inline int padded_row_floats(int d) { return (d + 7) / 8 * 8; }

// conn.cu
// Per-row sigma and rho.  `report_sigmas`: also compute the global mean that
// the sigma of a row with all neighbours at distance 0 takes (one more,
// latency-bound launch); without it such rows' sigmas are not the
// reference's, and nothing built from them (weights, graphs) changes.
cudaError_t launch_smooth_knn(scrust_context* ctx, const float* dist, int64_t n, int k,
                              float* sigmas, float* rhos, bool report_sigmas);
// Device CSR buffers from the context's pool (call with the context lock
// held), back to the pool, and a download into a new host CSR (pinned slab;
// synchronises the context stream).
int32_t csr_take(scrust_context* ctx, uint64_t rows, uint64_t nnz_cap, CsrBuffers* out, scrust_status* st);
void csr_give(scrust_context* ctx, const CsrBuffers& b);
int32_t csr_download(scrust_context* ctx, const CsrBuffers& b, uint64_t rows, uint64_t cols, scrust_csr** out,
                     scrust_status* st);

// The UMAP connectivities CSR of an n x k graph.  `distinct_rows`: every row's
// ids are distinct (true of every kNN graph this library builds), which
// allows the bucket transpose; graphs from callers take the stable radix sort.
// `ranges`: run the union in ctx->csr_stream's row ranges and record its
// events (the distinct-rows form only; returns whether it did through
// *streamed).
int32_t run_connectivities(scrust_context* ctx, const uint32_t* idx, const float* dist, int64_t n,
                           int k, bool validate, CsrBuffers* out, scrust_status* st, bool distinct_rows = false,
                           bool ranges = false, bool* streamed = nullptr);
// Rows of the directed fuzzy set of query rows against a reference (no
// symmetrisation, no self to drop): sigma/rho per row as smooth_knn, then
// exp weights, zero weights dropped, columns ascending, as a CSR of q rows.
int32_t run_query_connectivities(scrust_context* ctx, const uint32_t* idx, const float* dist, int64_t q, int k,
                                 CsrBuffers* out, scrust_status* st);

// Device-wide primitives (conn.cu).
cudaError_t device_exclusive_scan(scrust_context* ctx, const uint32_t* in, uint32_t* out, int64_t n,
                                  uint32_t* scratch, size_t scratch_elems);
size_t scan_scratch_elems(int64_t n);
int radix_blocks(int64_t n);
cudaError_t radix_sort_pairs(scrust_context* ctx, uint32_t* kA, unsigned long long* vA, uint32_t* kB,
                             unsigned long long* vB, int64_t n, int bits, uint32_t* hist, uint32_t* scan_scratch,
                             size_t scan_elems, uint32_t** keys_out, unsigned long long** vals_out);

// A reference set prepared for query-versus-reference solves (cross.cu):
// its rows, centring means, tensor operands B and the words max centred
// norm, max quantisation radius, max |b_hat| that fix the scale and bounds.
struct Reference {
    const float* rows = nullptr;
    int64_t n = 0, n_pad = 0;
    int d = 0;
    const double* means = nullptr;
    const uint32_t* words = nullptr;
    const void* B16 = nullptr;
    bool bf16 = false;
};
// Prepares x (n x d, device) as a reference in this context's workspace.
int32_t reference_prepare(scrust_context* ctx, const float* x, int64_t n, int d, bool bf16, Reference* out,
                          scrust_status* st);
// k nearest reference rows of q query rows (device), exact; self_offset >= 0
// marks query i as reference row i + self_offset (excluded).  Outputs q x k.
int32_t cross_knn_enqueue(scrust_context* ctx, const Reference& ref, const float* dq, int64_t q, int k,
                          int64_t self_offset, uint32_t* d_idx, float* d_dist, scrust_status* st);

// Tensor-map encoding through the driver entry point.
bool encode_2d(scrust_context* ctx, CUtensorMap* map, CUtensorMapDataType dtype, void* base,
               uint64_t inner, uint64_t outer, uint64_t row_bytes, uint32_t box_inner,
               uint32_t box_outer, CUtensorMapSwizzle swizzle);

}  // namespace scrust
