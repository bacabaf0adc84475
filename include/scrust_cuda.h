/*
 * scrust_cuda.h -- C ABI of the GB300 (sm_103a) backend for scrust's
 * `pp.neighbors` path: exact k-nearest neighbours on an embedding and the UMAP
 * fuzzy-simplicial-set connectivities.
 *
 * Plain pointers and sizes only.  Every entry point returns a scrust_code and,
 * when `status` is non-NULL, fills it with the same code and a message.  No
 * entry point aborts the process.  Host-pointer entry points block until their
 * results are in host memory; *_device entry points enqueue on the context's
 * stream and return without synchronising.
 *
 * Reference interfaces replaced (paths inside the scrust repository):
 *   scrust_cuda_knn                  scrust_core::neighbors::knn
 *                                    crates/scrust-core/src/neighbors.rs:29
 *                                    and scrust_gpu::kernels::knn::knn_metal
 *                                    crates/scrust-gpu/src/kernels/knn.rs:36
 *   scrust_cuda_connectivities       scrust_core::neighbors::connectivities
 *                                    crates/scrust-core/src/neighbors.rs:208
 *   scrust_cuda_smooth_knn_distances scrust_core::neighbors::smooth_knn_distances
 *                                    crates/scrust-core/src/neighbors.rs:239
 *   scrust_cuda_context_create/destroy  scrust_gpu::MetalContext::new / Drop
 *                                    crates/scrust-gpu/src/context.rs:12-91
 *   scrust_cuda_max_supported_k      scrust_gpu::kernels::knn::max_supported_k
 *                                    crates/scrust-gpu/src/kernels/knn.rs:27
 *   scrust_cuda_gpu_available        scrust_core::device::gpu_available
 *                                    crates/scrust-core/src/device.rs:39
 *   scrust_csr_*                     scrust_core::sparse::CsrMatrix accessors
 *                                    crates/scrust-core/src/sparse.rs:10-90
 *   scrust_cuda_neighbors_graph      the two FFI calls of python/scrust/pp/_basics.py:198,209
 *                                    fused into one device pass
 *   scrust_cuda_umap                 scrust_core::umap::umap
 *                                    crates/scrust-core/src/umap.rs:64
 *   scrust_cuda_pca                  scrust_core::pca::pca
 *                                    crates/scrust-core/src/pca.rs:74
 *   scrust_cuda_leiden               scrust_core::cluster::leiden
 *                                    crates/scrust-core/src/cluster.rs:88
 *   scrust_cuda_louvain              scrust_core::cluster::louvain
 *                                    crates/scrust-core/src/cluster.rs:125
 *   scrust_cuda_modularity           scrust_core::cluster::modularity
 *                                    crates/scrust-core/src/cluster.rs:148
 * Entry points with no reference counterpart (new semantics, parity against
 * the FP64 oracle only): scrust_cuda_knn_batched (many samples in one launch)
 * and the scrust_serve_* query service (queries against a resident atlas).
 */
#ifndef SCRUST_CUDA_H
#define SCRUST_CUDA_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SCRUST_API __attribute__((visibility("default")))
#else
#define SCRUST_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors scrust_core::Error (crates/scrust-core/src/error.rs:8-33); the
 * Python layer maps SHAPE and INVALID_PARAMETER to ValueError and the rest
 * to RuntimeError, as crates/scrust-py/src/lib.rs:26-35 does. */
typedef enum scrust_code {
    SCRUST_OK = 0,
    SCRUST_SHAPE = 1,             /* Error::Shape */
    SCRUST_INVALID_PARAMETER = 2, /* Error::InvalidParameter */
    SCRUST_NO_GPU = 3,            /* Error::NoGpu */
    SCRUST_KERNEL = 4,            /* Error::Kernel */
    SCRUST_NOT_CONVERGED = 5,     /* Error::NotConverged */
    SCRUST_OOM = 6,               /* device or host allocation failed / over budget */
    SCRUST_TIMEOUT = 7            /* a bounded device wait ran out */
} scrust_code;

typedef struct scrust_status {
    int32_t code;
    char message[256];
} scrust_status;

typedef struct scrust_context scrust_context;
typedef struct scrust_csr scrust_csr;

/* How candidates are generated before the exact rerank. */
typedef enum scrust_form {
    SCRUST_FORM_PLAIN = 0,  /* FP32 tiled expansion on CUDA cores (the drop-in) */
    SCRUST_FORM_TENSOR = 1, /* 16-bit tcgen05/TMEM candidate GEMM, FP32 accumulate */
    /* The tensor form wherever it applies (exact mode, at most 61
     * dimensions), else the plain form.  Both give the same lists; the
     * tensor form is the faster one. */
    SCRUST_FORM_AUTO = 2
} scrust_form;

typedef enum scrust_metric {
    SCRUST_METRIC_EUCLIDEAN = 0,
    SCRUST_METRIC_COSINE = 1 /* 1 - a.b/(|a||b|); no reference counterpart */
} scrust_metric;

typedef enum scrust_mode {
    /* Neighbour lists equal the FP64 exact kNN with lowest-index tie-break. */
    SCRUST_MODE_EXACT = 0,
    /* The reference's GPU semantics: centred coordinates, sequential fused
     * difference form and the sub-resolution snap of knn.rs:223-240. */
    SCRUST_MODE_REFERENCE_SNAP = 1
} scrust_mode;

typedef enum scrust_precision {
    SCRUST_PRECISION_FP16 = 0, /* 11-bit significand operands (default) */
    SCRUST_PRECISION_BF16 = 1  /* 8-bit significand operands */
} scrust_precision;

/* Whether the tensor form first orders the rows by a nearest-anchor
 * partition so each row meets its neighbours early in the sweep.  The
 * neighbour lists do not depend on it; only the speed does. */
typedef enum scrust_ordering {
    SCRUST_ORDERING_AUTO = 0, /* on for large self-kNN solves with one column segment */
    SCRUST_ORDERING_OFF = 1,
    SCRUST_ORDERING_ON = 2    /* whenever the solve has one column segment */
} scrust_ordering;

typedef struct scrust_knn_options {
    uint32_t struct_size;   /* sizeof(scrust_knn_options) */
    int32_t form;           /* scrust_form */
    int32_t metric;         /* scrust_metric */
    int32_t mode;           /* scrust_mode */
    int32_t precision;      /* scrust_precision, tensor form only */
    uint32_t list_capacity; /* candidates kept per row between prunes; 0 = automatic */
    uint32_t segments;      /* column segments per row tile; 0 = automatic */
    int32_t ordering;       /* scrust_ordering, tensor form only */
    uint32_t reserved[8];
} scrust_knn_options;

/* Fills `options` with the defaults: automatic form, Euclidean, exact, FP16,
 * automatic ordering.  A kNN call asked for the tensor form where it does not
 * apply runs the plain form (the same lists) and says so in the status
 * message while returning SCRUST_OK. */
SCRUST_API void scrust_knn_options_default(scrust_knn_options* options);

/* 1 when a CUDA device of compute capability 10.3 is usable, else 0. */
SCRUST_API int32_t scrust_cuda_gpu_available(void);

/* A per-device context: stream, workspace arena, kernel configuration. */
SCRUST_API scrust_context* scrust_cuda_context_create(int32_t device, scrust_status* status);
SCRUST_API void scrust_cuda_context_destroy(scrust_context* context);
/* The context's CUDA stream as an opaque pointer (a cudaStream_t). */
SCRUST_API void* scrust_cuda_context_stream(scrust_context* context);
/* Largest k the kernels serve; 0 for a NULL context. */
SCRUST_API uint32_t scrust_cuda_max_supported_k(const scrust_context* context);

/* Exact k nearest neighbours of every row of `embedding` (n x d, row-major
 * f32), self excluded, nearest first, ties to the smaller id.  Outputs are
 * caller-allocated n x k arrays.  Host pointers.  Errors mirror
 * neighbors.rs:41-57: n == 0 or d == 0 -> SHAPE; k == 0 or k >= n ->
 * INVALID_PARAMETER; k > scrust_cuda_max_supported_k -> INVALID_PARAMETER. */
SCRUST_API int32_t scrust_cuda_knn(scrust_context* context, const float* embedding, uint64_t n, uint64_t d,
                        uint32_t k, const scrust_knn_options* options, uint32_t* out_indices,
                        float* out_distances, scrust_status* status);

/* The same with device pointers, enqueued on the context stream. */
SCRUST_API int32_t scrust_cuda_knn_device(scrust_context* context, const float* embedding, uint64_t n,
                               uint64_t d, uint32_t k, const scrust_knn_options* options,
                               uint32_t* out_indices, float* out_distances,
                               scrust_status* status);

/* UMAP connectivities of a kNN graph (n x k ids and distances, host
 * pointers).  On success *out is a host-resident CSR (sorted columns, empty
 * diagonal, values in (0, 1]) owned by the caller: free it with
 * scrust_csr_free.  Errors mirror neighbors.rs:209-227. */
SCRUST_API int32_t scrust_cuda_connectivities(scrust_context* context, const uint32_t* indices,
                                   const float* distances, uint64_t n, uint32_t k,
                                   scrust_csr** out, scrust_status* status);

/* The same from device-resident inputs; *out is a device-resident CSR. */
SCRUST_API int32_t scrust_cuda_connectivities_device(scrust_context* context, const uint32_t* indices,
                                          const float* distances, uint64_t n, uint32_t k,
                                          scrust_csr** out, scrust_status* status);

/* Per-row sigma and rho of umap's smooth_knn_dist (host pointers), the
 * global mean summed in the reference's own f32 order. */
SCRUST_API int32_t scrust_cuda_smooth_knn_distances(scrust_context* context, const float* distances,
                                         uint64_t n, uint32_t k, float* sigmas, float* rhos,
                                         scrust_status* status);

/* pp.neighbors in one pass: kNN (out_indices / out_distances, the rows of
 * obsp["distances"]) and the connectivities CSR.  Host pointers in and out. */
SCRUST_API int32_t scrust_cuda_neighbors_graph(scrust_context* context, const float* embedding, uint64_t n,
                                    uint64_t d, uint32_t k, const scrust_knn_options* options,
                                    uint32_t* out_indices, float* out_distances,
                                    scrust_csr** connectivities, scrust_status* status);

/* The same with device pointers; the CSR is device-resident. */
SCRUST_API int32_t scrust_cuda_neighbors_graph_device(scrust_context* context, const float* embedding,
                                           uint64_t n, uint64_t d, uint32_t k,
                                           const scrust_knn_options* options,
                                           uint32_t* out_indices, float* out_distances,
                                           scrust_csr** connectivities, scrust_status* status);

/* CSR accessors.  Arrays live on the host or the device as the producing call
 * says (scrust_csr_on_device).  nnz of a device CSR is final once the
 * context stream has been synchronised (scrust_cuda_synchronize). */
SCRUST_API uint64_t scrust_csr_n_rows(const scrust_csr* csr);
SCRUST_API uint64_t scrust_csr_n_cols(const scrust_csr* csr);
SCRUST_API uint64_t scrust_csr_nnz(const scrust_csr* csr);
SCRUST_API int32_t scrust_csr_on_device(const scrust_csr* csr);
SCRUST_API const uint32_t* scrust_csr_indptr(const scrust_csr* csr);
SCRUST_API const uint32_t* scrust_csr_indices(const scrust_csr* csr);
SCRUST_API const float* scrust_csr_values(const scrust_csr* csr);
SCRUST_API void scrust_csr_free(scrust_csr* csr);

/* Blocks until the context stream is idle; reports a pending kernel error. */
SCRUST_API int32_t scrust_cuda_synchronize(scrust_context* context, scrust_status* status);

/* No counterpart in the reference.  scrust_cuda_smooth_knn_distances for
 * callers that cannot let a library allocate device memory -- processes whose
 * own pool allocator owns the GPU's memory, or services that reserve their
 * HBM budget up front -- on device pointers they own: `distances` (n x k),
 * `sigmas` and `rhos` (n).  The computation's only scratch is a fixed 33 KB
 * array compiled into the library (held by every GPU that loads it until the
 * process exits), so n * k is limited to 16,777,216; larger inputs return
 * SCRUST_INVALID_PARAMETER.  The work runs on the GPU that holds the three
 * buffers (buffers on different GPUs, or in host memory, return
 * SCRUST_INVALID_PARAMETER), enqueued on `stream` (a cudaStream_t of that
 * GPU; NULL is its legacy default stream) without synchronising; the calling
 * thread's current device is left as it was.  The first call on each device
 * looks up the array's device address and keeps it for the process's life,
 * so make that call before any stream capture and do not use the entry point
 * across a cudaDeviceReset.  All calls on a device share the array: calls
 * that overlap on the GPU race on it and must be ordered by the caller.  The
 * global mean (the sigma floor of rows whose neighbours all sit at distance
 * 0) is an FP64 sum here, within a few 1e-6 relative of the reference's f32
 * sum that scrust_cuda_smooth_knn_distances reproduces. */
SCRUST_API int32_t scrust_cuda_smooth_knn_distances_noalloc(const float* distances, uint64_t n, uint32_t k,
                                                            float* sigmas, float* rhos, void* stream,
                                                            scrust_status* status);

/* Row-range solve for a sharded graph build: the k nearest rows of x (n x d,
 * device) for each row in [row_begin, row_end), self excluded, ids global.
 * Outputs are (row_end - row_begin) x k.  Tensor form, exact Euclidean, d at
 * most 61.  The rows' union over shards equals scrust_cuda_knn_device. */
SCRUST_API int32_t scrust_cuda_knn_rows_device(scrust_context* context, const float* embedding, uint64_t n,
                                               uint64_t d, uint32_t k, uint64_t row_begin, uint64_t row_end,
                                               const scrust_knn_options* options, uint32_t* out_indices,
                                               float* out_distances, scrust_status* status);

/* ---- Batches of independent samples (no reference counterpart) ----
 *
 * `n_samples` independent self-kNN solves in one tensor-form sweep.  The
 * samples' rows are concatenated in `embedding` (device pointer, sum(n_s) x
 * d f32); `row_offsets` (host, n_samples + 1 entries, starting at 0) gives
 * each sample's rows.  Outputs are sum(n_s) x k, in the same row order, with
 * neighbour ids relative to the sample's first row.  Each sample's result
 * is bit-identical to a solve of that sample alone.  Exact mode only; d at
 * most 61; every sample needs more than k cells. */
typedef struct scrust_batch_plan scrust_batch_plan;
/* Host pointers: uploads, solves, downloads and reports device errors. */
SCRUST_API int32_t scrust_cuda_knn_batch(scrust_context* context, const float* embedding, const uint64_t* row_offsets,
                                         uint32_t n_samples, uint64_t d, uint32_t k,
                                         const scrust_knn_options* options, uint32_t* out_indices,
                                         float* out_distances, scrust_status* status);
SCRUST_API int32_t scrust_cuda_knn_batch_device(scrust_context* context, const float* embedding,
                                                const uint64_t* row_offsets, uint32_t n_samples, uint64_t d,
                                                uint32_t k, const scrust_knn_options* options,
                                                uint32_t* out_indices, float* out_distances, scrust_status* status);
/* A plan fixes the layout and the device buffers, autotunes the candidate
 * over-provisioning (the list capacity, when options->list_capacity is 0),
 * the sweep's register top-k width and the operand precision on this batch,
 * and captures the whole solve in a CUDA graph.  Each launch is one graph
 * launch on the context stream. */
SCRUST_API scrust_batch_plan* scrust_cuda_batch_plan_create(scrust_context* context, const uint64_t* row_offsets,
                                                            uint32_t n_samples, uint64_t d, uint32_t k,
                                                            const scrust_knn_options* options,
                                                            const float* embedding, uint32_t* out_indices,
                                                            float* out_distances, scrust_status* status);
SCRUST_API int32_t scrust_cuda_batch_plan_launch(scrust_batch_plan* plan, scrust_status* status);
/* The autotuner's choice and its time for one batch; returns 0 for NULL. */
SCRUST_API int32_t scrust_cuda_batch_plan_choice(const scrust_batch_plan* plan, uint32_t* list_capacity,
                                                 int32_t* precision, float* tuned_ms);
/* The register top-k width the autotuner chose for the sweep: 16 or 32, or 0
 * for candidate lists alone (warp-cooperative prunes); -1 for NULL. */
SCRUST_API int32_t scrust_cuda_batch_plan_topk_width(const scrust_batch_plan* plan);

/* Graphs of many samples.  A plan made by scrust_cuda_batch_plan_create_graphs
 * also builds every sample's UMAP connectivities inside the same captured
 * launch: smooth_knn, exp weights and the fuzzy union of that sample's rows
 * alone (crates/scrust-core/src/neighbors.rs:208-372 applied per sample),
 * into one device CSR of sum(n_s) rows in input order whose column ids are
 * relative to each sample's first row.  Sample s's own CSR is rows
 * [row_offsets[s], row_offsets[s+1]): indptr over those rows less
 * indptr[row_offsets[s]], and the entries between.  The arrays belong to the
 * plan and hold the last launch's graph once the context stream has
 * synchronised; nnz is indptr[sum(n_s)].  At most 2^31 graph entries. */
SCRUST_API scrust_batch_plan* scrust_cuda_batch_plan_create_graphs(scrust_context* context, const uint64_t* row_offsets,
                                                                   uint32_t n_samples, uint64_t d, uint32_t k,
                                                                   const scrust_knn_options* options,
                                                                   const float* embedding, uint32_t* out_indices,
                                                                   float* out_distances, scrust_status* status);
/* The device arrays of a graph plan's connectivities; returns 0 (and writes
 * nothing) for a kNN-only plan. */
SCRUST_API int32_t scrust_cuda_batch_plan_graph(const scrust_batch_plan* plan, const uint32_t** indptr,
                                                const uint32_t** indices, const float** values);
/* Host pointers, no plan: kNN of every sample (as scrust_cuda_knn_batch) and
 * the batch's connectivities as a host CSR laid out as above (free it with
 * scrust_csr_free). */
SCRUST_API int32_t scrust_cuda_neighbors_graph_batch(scrust_context* context, const float* embedding,
                                                     const uint64_t* row_offsets, uint32_t n_samples, uint64_t d,
                                                     uint32_t k, const scrust_knn_options* options,
                                                     uint32_t* out_indices, float* out_distances,
                                                     scrust_csr** connectivities, scrust_status* status);
SCRUST_API void scrust_cuda_batch_plan_destroy(scrust_batch_plan* plan);

/* ---- Query service over a resident atlas (no reference counterpart) ----
 *
 * The atlas (host pointer, m x d f32, d <= 61) is uploaded once and stays in
 * HBM.  Requests of any number of query cells are submitted from any thread
 * and answered by a scheduler thread that admits them into batches (at most
 * `max_batch_cells` cells, 0 = 65536) while one of `n_slots` slots (0 = 2)
 * and the memory budget (`budget_bytes`, 0 = 150 GiB, atlas included) allow;
 * batches on different slots overlap on the GPU.  Each request gets its k
 * nearest atlas cells (exact, FP64-equal lists, no self-exclusion) and the
 * rows of its directed connectivities (smooth_knn sigma/rho and exp weights
 * per row, columns ascending, no symmetrisation) as a host CSR of q rows by
 * m columns.  A request's result does not depend on its batch.  Exact
 * Euclidean only. */
typedef struct scrust_server scrust_server;
SCRUST_API scrust_server* scrust_serve_create(int32_t device, const float* atlas, uint64_t m, uint64_t d, uint32_t k,
                                              const scrust_knn_options* options, uint64_t budget_bytes,
                                              uint64_t max_batch_cells, uint32_t n_slots, scrust_status* status);
/* Copies the q x d queries and returns a ticket (0 on error). */
SCRUST_API uint64_t scrust_serve_submit(scrust_server* server, const float* queries, uint64_t q,
                                        scrust_status* status);
/* Blocks until the request is answered; writes q x k ids and distances,
 * optionally the connectivities CSR (free with scrust_csr_free) and the
 * submit-to-answer latency.  A ticket is waited for once. */
SCRUST_API int32_t scrust_serve_wait(scrust_server* server, uint64_t ticket, uint32_t* out_indices,
                                     float* out_distances, scrust_csr** out_connectivities, double* latency_ms,
                                     scrust_status* status);
/* batches, requests answered, most batches on the GPU at once, cells
 * answered, max batch cells, budget bytes per cell, slots; returns the count
 * written. */
SCRUST_API int32_t scrust_serve_stats(scrust_server* server, uint64_t* out, int32_t max_words);
/* Answers what is pending, then stops the scheduler and frees everything. */
SCRUST_API void scrust_serve_destroy(scrust_server* server);

/* ---- UMAP layout of a connectivities graph ----
 *
 * Replaces scrust_core::umap::umap (crates/scrust-core/src/umap.rs:64) with
 * its parameters (UmapParams, umap.rs:9-33).  The layout is umap-learn's SGD
 * as the reference runs it -- the same curve fit, firing schedule, per-cell
 * negative-sample streams, attraction, repulsion and clip -- but every epoch
 * computes all moves from the layout as it stood when the epoch began and
 * sums them per cell in a fixed order, so it is deterministic (the same bits
 * on every run) where the reference's sequential sweep has no parallel form;
 * and the random initial layout draws one stream per cell.  Errors mirror
 * umap.rs:86-110: n_components or n_epochs of 0 and min_dist outside
 * [0, 3 spread] -> INVALID_PARAMETER; an empty or non-square graph, or one
 * with no edge strong enough to fire -> SHAPE.  n_components at most 16. */
typedef struct scrust_umap_params {
    uint32_t struct_size;          /* sizeof(scrust_umap_params) */
    uint32_t n_components;         /* 2 */
    uint32_t n_epochs;             /* 200 */
    float min_dist;                /* 0.5 */
    float spread;                  /* 1.0 */
    float learning_rate;           /* 1.0 */
    uint32_t negative_sample_rate; /* 5; 0 switches repulsion off */
    uint32_t reserved0;
    uint64_t seed;                 /* 0 */
    uint32_t reserved[8];
} scrust_umap_params;
SCRUST_API void scrust_umap_params_default(scrust_umap_params* params);
/* Host pointers: a CSR graph (n_rows + 1 indptr, indices and values of
 * indptr[n_rows] entries) in, the (n_rows, n_components) f32 layout out. */
SCRUST_API int32_t scrust_cuda_umap(scrust_context* context, const uint32_t* indptr, const uint32_t* indices,
                                    const float* values, uint64_t n_rows, uint64_t n_cols,
                                    const scrust_umap_params* params, float* out_embedding, scrust_status* status);
/* Device pointers (nnz given), enqueued on the context stream after one
 * synchronisation that checks the graph has an edge to fire. */
SCRUST_API int32_t scrust_cuda_umap_device(scrust_context* context, const uint32_t* indptr, const uint32_t* indices,
                                           const float* values, uint64_t n_rows, uint64_t n_cols, uint64_t nnz,
                                           const scrust_umap_params* params, float* out_embedding,
                                           scrust_status* status);

/* ---- PCA, the step before the neighbours path ----
 *
 * Replaces scrust_core::pca::pca (crates/scrust-core/src/pca.rs:74): truncated
 * PCA of a cells x genes CSR matrix by the reference's randomised SVD
 * (sketch of n_components + 24 columns, 7 or 4 power iterations, the
 * largest-loading sign fix, scanpy's explained variance and ratios for
 * zero_center on and off).  Deterministic: the same inputs and seed give the
 * same bits; the Gaussian sketch is this library's counter-based one, so the
 * results agree with the reference's subspace, not its bits.  Outputs: the
 * embedding (n_cells x n_components, obsm["X_pca"]), the components
 * (n_components x n_genes, varm["PCs"] transposed), the explained variance
 * and its ratio (n_components each).  Errors mirror pca.rs:81-94:
 * n_components of 0 or above min(n_cells, n_genes), or fewer than 2 cells ->
 * INVALID_PARAMETER.  n_components at most 104. */
SCRUST_API int32_t scrust_cuda_pca(scrust_context* context, const uint32_t* indptr, const uint32_t* indices,
                                   const float* values, uint64_t n_cells, uint64_t n_genes, uint32_t n_components,
                                   int32_t zero_center, uint64_t seed, float* out_embedding, float* out_components,
                                   float* out_variance, float* out_variance_ratio, scrust_status* status);
/* Device pointers (nnz given): the embedding stays in HBM, ready for
 * scrust_cuda_neighbors_graph_device.  Synchronises once at the end. */
SCRUST_API int32_t scrust_cuda_pca_device(scrust_context* context, const uint32_t* indptr, const uint32_t* indices,
                                          const float* values, uint64_t n_cells, uint64_t n_genes, uint64_t nnz,
                                          uint32_t n_components, int32_t zero_center, uint64_t seed,
                                          float* out_embedding, float* out_components, float* out_variance,
                                          float* out_variance_ratio, scrust_status* status);

/* ---- Community detection on the connectivities, the step after it ----
 *
 * Replace scrust_core::cluster::{leiden, louvain, modularity}
 * (crates/scrust-core/src/cluster.rs:88,125,148): RBConfiguration modularity
 * with a resolution on the graph (A + A^T) / 2 of a square CSR matrix.
 * Leiden runs up to n_iterations passes of local moving, refinement into
 * well-connected subcommunities and aggregation, stopping at a pass that
 * returns its own input; Louvain one pass without refinement.  Labels are
 * numbered by descending community size, ties to the smaller id; the
 * modularity of the labels and the community count are written beside them.
 * The moves run in parallel rounds, so the partition is this library's own:
 * deterministic for the same graph and seed, not the reference's label for
 * label (its moves are sequential from a ChaCha12 stream).  Errors mirror
 * cluster.rs:95-97,170-180,214-290: resolution not finite and > 0 or
 * n_iterations of 0 -> INVALID_PARAMETER; an empty or non-square graph ->
 * SHAPE; weights negative or not finite, or none positive ->
 * INVALID_PARAMETER.  Host pointers; synchronises. */
SCRUST_API int32_t scrust_cuda_leiden(scrust_context* context, const uint32_t* indptr, const uint32_t* indices,
                                      const float* values, uint64_t n_rows, uint64_t n_cols, double resolution,
                                      uint32_t n_iterations, uint64_t seed, uint32_t* out_labels,
                                      double* out_modularity, uint64_t* out_n_communities, scrust_status* status);
SCRUST_API int32_t scrust_cuda_louvain(scrust_context* context, const uint32_t* indptr, const uint32_t* indices,
                                       const float* values, uint64_t n_rows, uint64_t n_cols, double resolution,
                                       uint64_t seed, uint32_t* out_labels, double* out_modularity,
                                       uint64_t* out_n_communities, scrust_status* status);
/* Modularity of given labels: n_labels must equal n_rows (else SHAPE) and
 * every label must be below n_rows (else INVALID_PARAMETER). */
SCRUST_API int32_t scrust_cuda_modularity(scrust_context* context, const uint32_t* indptr, const uint32_t* indices,
                                          const float* values, uint64_t n_rows, uint64_t n_cols,
                                          const uint32_t* labels, uint64_t n_labels, double resolution,
                                          double* out_modularity, scrust_status* status);

/* Phase timing.  When enabled, each kNN / connectivities call records CUDA
 * events on the context stream around its phases; scrust_cuda_phase_times
 * writes the last call's milliseconds (after a synchronise) in the order
 * prep, candidates, rerank, connectivities, then four parts of candidates in
 * an ordered tensor-form solve (its first sweep pass, the building of the
 * second tile lists, the second sweep pass when k > 32, and the collect pass
 * over both tile lists when k <= 32; 0 where absent), and returns how many it
 * wrote. */
SCRUST_API void scrust_cuda_set_timing(scrust_context* context, int32_t enable);
SCRUST_API int32_t scrust_cuda_phase_times(scrust_context* context, float* ms, int32_t max_phases);

/* Kernel counters (observability).  enable = 1 turns collection on (later
 * calls accumulate), enable = 0 turns it off.  Writes up to max_words
 * counters accumulated since the previous read and resets them; returns how
 * many it wrote.  For the tensor form, by index: 0 appends, 1 prunes,
 * 2 overflow rows, 3 epilogue wait cycles, 5/6 MMA wait cycles (B tiles,
 * accumulators), 7 producer wait cycles, 8 tiles, 9 prune cycles, and for the
 * register top-k 12 chunks with an entrant, 13 bulk merges, 14 insertion
 * rounds, 15 entrants; 4, 10 and 11 are unused.  Words 0-15 hold every sweep
 * launch together; with max_words up to 80, words 16-31, 32-47 and 48-63 hold
 * the first, second and third sweep launch of each solve on their own and
 * 64-79 every later launch (an ordered solve with k <= 32 runs a threshold
 * pass over its priority tiles, then one collect pass over those and the tiles
 * the tile balls keep). */
SCRUST_API int32_t scrust_cuda_kernel_stats(scrust_context* context, int32_t enable, uint64_t* out,
                                            int32_t max_words);

/* Self-test of the bounded device waits (no counterpart in the reference:
 * the Metal backend has no device-side waits).  Runs one kernel that waits
 * on an mbarrier nothing arrives on, with the wall-clock limit every sweep
 * kernel's waits use replaced by limit_ns (at most 100 ms, else
 * INVALID_PARAMETER).  Returns SCRUST_TIMEOUT when the wait ran out and was
 * reported, as a sweep kernel's would be; the context stays usable. */
SCRUST_API int32_t scrust_cuda_selftest_bounded_wait(scrust_context* context, uint64_t limit_ns,
                                                     scrust_status* status);

/* Number of kernels this context has launched since it was created. */
SCRUST_API uint64_t scrust_cuda_launch_count(const scrust_context* context);

/* Library version string. */
SCRUST_API const char* scrust_cuda_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SCRUST_CUDA_H */
