/*
 * neighbors_oracle.c -- the ORACLE for the pp.neighbors path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke entry
 * point and the CPU-baseline leg of bench.py call it; the shipped CUDA library
 * never links, loads or calls it.
 *
 * It restates, in plain C, the reference's CPU implementation of
 * `scrust_core::neighbors` (crates/scrust-core/src/neighbors.rs) and the CPU
 * twin of its Metal kernel (crates/scrust-gpu/src/kernels/knn.rs), plus the
 * FP64 exact kNN of tests/test_neighbors_audit.py:52-61.  Every function cites
 * the reference lines it follows.
 *
 * Parity of this restatement is pinned by the reference's own known answers
 * (neighbors.rs:408-437 line/grid/tiling, :498-590 scanpy golden neighbour
 * sets, connectivity rows, nnz and sums; knn.rs:339-415 Metal cases).  See
 * tests/test_oracle_golden.py.
 *
 * Third-party arithmetic that the reference takes from crates that are not
 * vendored (restated from their published algorithms):
 *   - ndarray 0.16.1 `ArrayBase::sum` on contiguous data is
 *     `numeric_util::unrolled_fold`: eight strided partial sums combined as
 *     ((p0+p4), (p1+p5), (p2+p6), (p3+p7)) into the accumulator, then the
 *     tail added sequentially (unrolled_sum_f32 below).
 *   - candle-core 0.9.2 -> gemm 0.19.0 computes the tile matmul of
 *     neighbors.rs:74; its f32 summation order is not published.  It is
 *     restated as a sequential fused multiply-add over the dimensions, so the
 *     expansion-form path is pinned only where ulp-level order does not decide
 *     a neighbour.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (oracle/build.py).
 * -ffp-contract=off matters: the reference's Rust arithmetic is never
 * contracted, so every fused multiply-add below is an explicit fmaf().
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum {
    ORACLE_OK = 0,
    ORACLE_SHAPE = 1,
    ORACLE_INVALID_PARAMETER = 2,
    ORACLE_OOM = 6,
};

/* f32::EPSILON, neighbors.rs:128 and knn.rs:174. */
static const float F32_EPS = 1.1920928955078125e-07f;

typedef struct {
    float d;
    uint32_t id;
} pair_f32;

typedef struct {
    double d;
    uint32_t id;
} pair_f64;

/* (d, id) ascending: neighbors.rs:181-182 (`total_cmp` then id) and
 * knn.rs:179-182 (`closer`).  Inputs are never NaN here, so total_cmp and
 * the numeric order agree for the non-negative values compared. */
static int cmp_pair_f32(const void* a, const void* b) {
    const pair_f32* x = (const pair_f32*)a;
    const pair_f32* y = (const pair_f32*)b;
    if (x->d < y->d) return -1;
    if (x->d > y->d) return 1;
    return (x->id > y->id) - (x->id < y->id);
}

static int cmp_pair_f64(const void* a, const void* b) {
    const pair_f64* x = (const pair_f64*)a;
    const pair_f64* y = (const pair_f64*)b;
    if (x->d < y->d) return -1;
    if (x->d > y->d) return 1;
    return (x->id > y->id) - (x->id < y->id);
}

/* ndarray 0.16.1 numeric_util::unrolled_fold with f32 addition. */
float oracle_unrolled_sum_f32(const float* xs, int64_t len) {
    float acc = 0.0f;
    float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f, p3 = 0.0f;
    float p4 = 0.0f, p5 = 0.0f, p6 = 0.0f, p7 = 0.0f;
    while (len >= 8) {
        p0 = p0 + xs[0];
        p1 = p1 + xs[1];
        p2 = p2 + xs[2];
        p3 = p3 + xs[3];
        p4 = p4 + xs[4];
        p5 = p5 + xs[5];
        p6 = p6 + xs[6];
        p7 = p7 + xs[7];
        xs += 8;
        len -= 8;
    }
    acc = acc + (p0 + p4);
    acc = acc + (p1 + p5);
    acc = acc + (p2 + p6);
    acc = acc + (p3 + p7);
    for (int64_t i = 0; i < len; i++) acc = acc + xs[i];
    return acc;
}

/* Argument checks of neighbors.rs:41-57. */
static int check_knn_args(int64_t n, int64_t d, int64_t k) {
    if (n <= 0 || d <= 0) return ORACLE_SHAPE;
    if (k <= 0) return ORACLE_INVALID_PARAMETER;
    if (k >= n) return ORACLE_INVALID_PARAMETER;
    return ORACLE_OK;
}

/* Column means accumulated row by row in f64, neighbors.rs:144-154. */
static void column_means(const float* x, int64_t n, int64_t d, double* means) {
    for (int64_t c = 0; c < d; c++) means[c] = 0.0;
    for (int64_t r = 0; r < n; r++)
        for (int64_t c = 0; c < d; c++) means[c] += (double)x[r * d + c];
    for (int64_t c = 0; c < d; c++) means[c] /= (double)n;
}

/* neighbors.rs:144-162: subtract in f64, round once to f32. */
int oracle_centred(const float* x, int64_t n, int64_t d, float* out) {
    double* means = (double*)malloc(sizeof(double) * (size_t)d);
    if (!means) return ORACLE_OOM;
    column_means(x, n, d, means);
    for (int64_t r = 0; r < n; r++)
        for (int64_t c = 0; c < d; c++)
            out[r * d + c] = (float)((double)x[r * d + c] - means[c]);
    free(means);
    return ORACLE_OK;
}

/* The k smallest of one row of squared distances, self excluded, ties to the
 * smaller id, then sqrt: neighbors.rs:171-191.  `buf` holds n pairs. */
static void select_nearest(const float* sq, int64_t n, int64_t cell, int64_t k,
                           pair_f32* buf, uint32_t* idx, float* dist) {
    int64_t m = 0;
    for (int64_t j = 0; j < n; j++) {
        if (j == cell) continue;
        float v = sq[j];
        buf[m].d = v > 0.0f ? v : 0.0f; /* square.max(0.0), :178 */
        buf[m].id = (uint32_t)j;
        m++;
    }
    /* A bounded insertion keeps the k best seen so far: identical result to
     * select_nth_unstable_by + sort_unstable_by under the total order. */
    pair_f32* top = buf; /* reuse the head of buf as the sorted top-k */
    int64_t have = 0;
    for (int64_t t = 0; t < m; t++) {
        pair_f32 c = buf[t];
        if (have == k) {
            pair_f32 w = top[k - 1];
            if (!(c.d < w.d || (c.d == w.d && c.id < w.id))) continue;
            have--;
        }
        int64_t s = have;
        while (s > 0 && (c.d < top[s - 1].d || (c.d == top[s - 1].d && c.id < top[s - 1].id))) {
            top[s] = top[s - 1];
            s--;
        }
        top[s] = c;
        have++;
    }
    for (int64_t t = 0; t < k; t++) {
        idx[t] = top[t].id;
        dist[t] = sqrtf(top[t].d); /* :189 */
    }
}

/*
 * The reference CPU kNN, neighbors.rs:29-101.
 *   centring (f64 means), squared norms, tiles of `tile_rows` rows, the
 *   expansion raw = (-2 * (T . P^T)) + (|a|^2 + |b|^2) (:73-74), the snap
 *   raw < (|a|^2+|b|^2) * ((D+2) * eps) -> 0 (:78-82, :127-129), and
 *   select_nearest per row (:84-96).  tile_rows <= 0 means 64Mi / n (:30).
 * Squared norms: candle's sqr().sum_keepdim(1) (:62), restated as a
 * sequential f32 sum of rounded squares.  The dot: sequential fmaf (gemm 0.19
 * order unpublished).  The result does not depend on tile_rows (:430-437).
 */
int oracle_knn_reference_cpu(const float* x, int64_t n, int64_t d, int64_t k,
                             int64_t tile_rows, uint32_t* idx, float* dist) {
    int rc = check_knn_args(n, d, k);
    if (rc) return rc;
    if (tile_rows <= 0) {
        tile_rows = (64LL * 1024 * 1024) / n;
        if (tile_rows < 1) tile_rows = 1;
    }
    float* c = (float*)malloc(sizeof(float) * (size_t)(n * d));
    float* sq = (float*)malloc(sizeof(float) * (size_t)n);
    if (!c || !sq) {
        free(c);
        free(sq);
        return ORACLE_OOM;
    }
    oracle_centred(x, n, d, c);
    for (int64_t r = 0; r < n; r++) {
        float s = 0.0f;
        for (int64_t t = 0; t < d; t++) {
            float v = c[r * d + t] * c[r * d + t];
            s = s + v;
        }
        sq[r] = s;
    }
    const float resolution = ((float)d + 2.0f) * F32_EPS;

    /* Column blocks transposed for a vectorisable inner loop over columns; the
     * per-element order stays sequential over dimensions. */
    const int64_t CB = 64;
    int64_t nblocks = (n + CB - 1) / CB;
    float* ct = (float*)malloc(sizeof(float) * (size_t)(nblocks * CB * d));
    if (!ct) {
        free(c);
        free(sq);
        return ORACLE_OOM;
    }
    for (int64_t b = 0; b < nblocks; b++)
        for (int64_t t = 0; t < d; t++)
            for (int64_t j = 0; j < CB; j++) {
                int64_t col = b * CB + j;
                ct[(b * d + t) * CB + j] = col < n ? c[col * d + t] : 0.0f;
            }

    int failed = 0;
    for (int64_t start = 0; start < n; start += tile_rows) {
        int64_t height = tile_rows < n - start ? tile_rows : n - start;
#pragma omp parallel
        {
            float* row = (float*)malloc(sizeof(float) * (size_t)n);
            pair_f32* buf = (pair_f32*)malloc(sizeof(pair_f32) * (size_t)n);
            float acc[CB];
            if (!row || !buf) {
#pragma omp atomic write
                failed = 1;
            } else {
#pragma omp for schedule(dynamic, 1)
                for (int64_t off = 0; off < height; off++) {
                    int64_t i = start + off;
                    const float* a = c + i * d;
                    for (int64_t b = 0; b < nblocks; b++) {
                        for (int64_t j = 0; j < CB; j++) acc[j] = 0.0f;
                        const float* blk = ct + b * d * CB;
                        for (int64_t t = 0; t < d; t++) {
                            float av = a[t];
                            const float* bt = blk + t * CB;
                            for (int64_t j = 0; j < CB; j++) acc[j] = fmaf(av, bt[j], acc[j]);
                        }
                        int64_t jmax = (b + 1) * CB <= n ? CB : n - b * CB;
                        for (int64_t j = 0; j < jmax; j++) {
                            int64_t col = b * CB + j;
                            float sums = sq[i] + sq[col];
                            float raw = (-2.0f * acc[j]) + sums;
                            float floor_ = sums * resolution;
                            row[col] = raw < floor_ ? 0.0f : raw;
                        }
                    }
                    select_nearest(row, n, i, k, buf, idx + i * k, dist + i * k);
                }
            }
            free(row);
            free(buf);
        }
    }
    free(ct);
    free(c);
    free(sq);
    return failed ? ORACLE_OOM : ORACLE_OK;
}

/*
 * The same computation restricted to the query rows `rows[0..nrows)`, each
 * against all n cells.  Used to time a bounded sample of a large workload on
 * the host; output row r corresponds to cell rows[r].
 */
int oracle_knn_reference_cpu_rows(const float* x, int64_t n, int64_t d, int64_t k,
                                  const int64_t* rows, int64_t nrows, uint32_t* idx,
                                  float* dist) {
    int rc = check_knn_args(n, d, k);
    if (rc) return rc;
    float* c = (float*)malloc(sizeof(float) * (size_t)(n * d));
    float* sq = (float*)malloc(sizeof(float) * (size_t)n);
    const int64_t CB = 64;
    int64_t nblocks = (n + CB - 1) / CB;
    float* ct = (float*)malloc(sizeof(float) * (size_t)(nblocks * CB * d));
    if (!c || !sq || !ct) {
        free(c);
        free(sq);
        free(ct);
        return ORACLE_OOM;
    }
    oracle_centred(x, n, d, c);
    for (int64_t r = 0; r < n; r++) {
        float s = 0.0f;
        for (int64_t t = 0; t < d; t++) {
            float v = c[r * d + t] * c[r * d + t];
            s = s + v;
        }
        sq[r] = s;
    }
    const float resolution = ((float)d + 2.0f) * F32_EPS;
    for (int64_t b = 0; b < nblocks; b++)
        for (int64_t t = 0; t < d; t++)
            for (int64_t j = 0; j < CB; j++) {
                int64_t col = b * CB + j;
                ct[(b * d + t) * CB + j] = col < n ? c[col * d + t] : 0.0f;
            }
    int failed = 0;
#pragma omp parallel
    {
        float* row = (float*)malloc(sizeof(float) * (size_t)n);
        pair_f32* buf = (pair_f32*)malloc(sizeof(pair_f32) * (size_t)n);
        float acc[CB];
        if (!row || !buf) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 1)
            for (int64_t r = 0; r < nrows; r++) {
                int64_t i = rows[r];
                const float* a = c + i * d;
                for (int64_t b = 0; b < nblocks; b++) {
                    for (int64_t j = 0; j < CB; j++) acc[j] = 0.0f;
                    const float* blk = ct + b * d * CB;
                    for (int64_t t = 0; t < d; t++) {
                        float av = a[t];
                        const float* bt = blk + t * CB;
                        for (int64_t j = 0; j < CB; j++) acc[j] = fmaf(av, bt[j], acc[j]);
                    }
                    int64_t jmax = (b + 1) * CB <= n ? CB : n - b * CB;
                    for (int64_t j = 0; j < jmax; j++) {
                        int64_t col = b * CB + j;
                        float sums = sq[i] + sq[col];
                        float raw = (-2.0f * acc[j]) + sums;
                        float floor_ = sums * resolution;
                        row[col] = raw < floor_ ? 0.0f : raw;
                    }
                }
                select_nearest(row, n, i, k, buf, idx + r * k, dist + r * k);
            }
        }
        free(row);
        free(buf);
    }
    free(ct);
    free(c);
    free(sq);
    return failed ? ORACLE_OOM : ORACLE_OK;
}

/*
 * The reference CPU path split where a BLAS takes over, for timing it on the
 * host the way it runs (candle hands the tile product of neighbors.rs:74 to
 * gemm's SGEMM microkernels):
 *   oracle_centred_norms   centred coordinates (neighbors.rs:144-162) and
 *                          squared norms (:62, sequential f32 sums);
 *   oracle_expansion_select  given G = T . P^T for a tile of query rows (the
 *                          caller's SGEMM), raw = (-2 G) + (|a|^2 + |b|^2),
 *                          the snap below (D+2) eps (|a|^2 + |b|^2) (:75-82)
 *                          and select_nearest (:171-191), rows in parallel.
 */
int oracle_centred_norms(const float* x, int64_t n, int64_t d, float* c, float* sq) {
    int rc = check_knn_args(n, d, 1 < n ? 1 : 0);
    if (rc) return rc;
    rc = oracle_centred(x, n, d, c);
    if (rc) return rc;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; r++) {
        float s = 0.0f;
        for (int64_t t = 0; t < d; t++) {
            float v = c[r * d + t] * c[r * d + t];
            s = s + v;
        }
        sq[r] = s;
    }
    return ORACLE_OK;
}

int oracle_expansion_select(const float* g, int64_t h, int64_t n, int64_t d, const int64_t* rows,
                            const float* sq, int64_t k, uint32_t* idx, float* dist) {
    int rc = check_knn_args(n, d, k);
    if (rc) return rc;
    const float resolution = ((float)d + 2.0f) * F32_EPS;
    int failed = 0;
#pragma omp parallel
    {
        float* row = (float*)malloc(sizeof(float) * (size_t)n);
        pair_f32* buf = (pair_f32*)malloc(sizeof(pair_f32) * (size_t)n);
        if (!row || !buf) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 1)
            for (int64_t r = 0; r < h; r++) {
                const int64_t i = rows[r];
                const float* gr = g + r * n;
                for (int64_t col = 0; col < n; col++) {
                    float sums = sq[i] + sq[col];
                    float raw = (-2.0f * gr[col]) + sums;
                    float floor_ = sums * resolution;
                    row[col] = raw < floor_ ? 0.0f : raw;
                }
                select_nearest(row, n, i, k, buf, idx + r * k, dist + r * k);
            }
        }
        free(row);
        free(buf);
    }
    return failed ? ORACLE_OOM : ORACLE_OK;
}

/*
 * CPU twin of the reference's Metal kernel, knn.rs:282-313 with
 * centre_and_norms (:135-158): centred coordinates, norms by an fmaf chain,
 * the difference form sum fma(a-b, a-b) in dimension order (:223-232), the
 * snap below ((D+2) * eps) * (|q|^2 + |c|^2) (:237-240), order by (d^2, id),
 * sqrt of the k survivors.
 */
int oracle_knn_metal_twin(const float* x, int64_t n, int64_t d, int64_t k, uint32_t* idx,
                          float* dist) {
    int rc = check_knn_args(n, d, k);
    if (rc) return rc;
    double* means = (double*)malloc(sizeof(double) * (size_t)d);
    float* c = (float*)malloc(sizeof(float) * (size_t)(n * d));
    float* nsq = (float*)malloc(sizeof(float) * (size_t)n);
    if (!means || !c || !nsq) {
        free(means);
        free(c);
        free(nsq);
        return ORACLE_OOM;
    }
    column_means(x, n, d, means);
    for (int64_t r = 0; r < n; r++) {
        float norm = 0.0f;
        for (int64_t t = 0; t < d; t++) {
            float coord = (float)((double)x[r * d + t] - means[t]);
            c[r * d + t] = coord;
            norm = fmaf(coord, coord, norm);
        }
        nsq[r] = norm;
    }
    int failed = 0;
#pragma omp parallel
    {
        pair_f32* buf = (pair_f32*)malloc(sizeof(pair_f32) * (size_t)n);
        if (!buf) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 16)
            for (int64_t q = 0; q < n; q++) {
                int64_t m = 0;
                for (int64_t j = 0; j < n; j++) {
                    if (j == q) continue;
                    float s = 0.0f;
                    for (int64_t t = 0; t < d; t++) {
                        float delta = c[q * d + t] - c[j * d + t];
                        s = fmaf(delta, delta, s);
                    }
                    float threshold = ((float)d + 2.0f) * F32_EPS * (nsq[q] + nsq[j]);
                    if (s < threshold) s = 0.0f;
                    buf[m].d = s;
                    buf[m].id = (uint32_t)j;
                    m++;
                }
                qsort(buf, (size_t)m, sizeof(pair_f32), cmp_pair_f32);
                for (int64_t t = 0; t < k; t++) {
                    idx[q * k + t] = buf[t].id;
                    dist[q * k + t] = sqrtf(buf[t].d);
                }
            }
        }
        free(buf);
    }
    free(means);
    free(c);
    free(nsq);
    return failed ? ORACLE_OOM : ORACLE_OK;
}

/* FP64 squared distance in dimension order, no fused operations. */
static double sq_dist_f64(const float* a, const float* b, int64_t d) {
    double s = 0.0;
    for (int64_t t = 0; t < d; t++) {
        double diff = (double)a[t] - (double)b[t];
        double p = diff * diff;
        s = s + p;
    }
    return s;
}

/* The same sum, abandoned once a partial sum exceeds `limit`: the terms are
 * non-negative and round-to-nearest addition of a non-negative term never
 * decreases the sum, so the full sum would exceed `limit` too.  Returns the
 * full sum when it is at most `limit` (then bit-equal to sq_dist_f64). */
static double sq_dist_f64_below(const float* a, const float* b, int64_t d, double limit) {
    double s = 0.0;
    int64_t t = 0;
    for (; t + 8 <= d; t += 8) {
        for (int64_t u = t; u < t + 8; u++) {
            double diff = (double)a[u] - (double)b[u];
            double p = diff * diff;
            s = s + p;
        }
        if (s > limit) return s;
    }
    for (; t < d; t++) {
        double diff = (double)a[t] - (double)b[t];
        double p = diff * diff;
        s = s + p;
    }
    return s;
}

/*
 * The FP64 ground truth of tests/test_neighbors_audit.py:52-61:
 * d = sqrt(max(sum (x_i - x_j)^2, 0)) in float64, k non-self neighbours
 * ordered by (d, j).  The sum runs in dimension order with no fused
 * operations, which fixes its rounding; the GPU adjudication uses the same
 * order.  Rows `rows[0..nrows)` (all rows when rows == NULL).
 * Outputs: idx (nrows, k), d64 (nrows, k) FP64 distances, dist (nrows, k)
 * those distances rounded to f32.
 */
int oracle_knn_fp64_rows(const float* x, int64_t n, int64_t d, int64_t k, const int64_t* rows,
                         int64_t nrows, uint32_t* idx, double* d64, float* dist) {
    int rc = check_knn_args(n, d, k);
    if (rc) return rc;
    if (rows == NULL) nrows = n;
    int failed = 0;
#pragma omp parallel
    {
        pair_f64* top = (pair_f64*)malloc(sizeof(pair_f64) * (size_t)(k + 1));
        if (!top) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 4)
            for (int64_t r = 0; r < nrows; r++) {
                int64_t q = rows ? rows[r] : r;
                int64_t have = 0;
                /* Once k are held, a column whose squared distance exceeds
                 * the k-th's by a relative 1e-12 has a strictly larger square
                 * root (its relative gap, ~5e-13, is far above the double
                 * rounding of sqrt), so it can neither enter nor tie: such
                 * columns are dropped early.  The result is unchanged. */
                double limit = INFINITY;
                for (int64_t j = 0; j < n; j++) {
                    if (j == q) continue;
                    double s = sq_dist_f64_below(x + q * d, x + j * d, d, limit);
                    if (s > limit) continue;
                    double v = sqrt(s > 0.0 ? s : 0.0);
                    pair_f64 cnd = {v, (uint32_t)j};
                    if (have == k) {
                        pair_f64 w = top[k - 1];
                        if (!(v < w.d || (v == w.d && cnd.id < w.id))) continue;
                        have--;
                    }
                    int64_t s2 = have;
                    while (s2 > 0 &&
                           (v < top[s2 - 1].d || (v == top[s2 - 1].d && cnd.id < top[s2 - 1].id))) {
                        top[s2] = top[s2 - 1];
                        s2--;
                    }
                    top[s2] = cnd;
                    have++;
                    if (have == k) {
                        double kth = top[k - 1].d;
                        limit = kth * kth * (1.0 + 1e-12);
                    }
                }
                for (int64_t t = 0; t < k; t++) {
                    idx[r * k + t] = top[t].id;
                    if (d64) d64[r * k + t] = top[t].d;
                    if (dist) dist[r * k + t] = (float)top[t].d;
                }
            }
        }
        free(top);
    }
    return failed ? ORACLE_OOM : ORACLE_OK;
}

/*
 * FP64 exact kNN of query rows against reference rows (the serving form's
 * semantics: no self-exclusion, ids index the reference): the same
 * dimension-order FP64 sum, sqrt, (d, id) order and exact early exit as
 * oracle_knn_fp64_rows.  Outputs (nq, k).
 */
int oracle_knn_fp64_cross(const float* q, int64_t nq, const float* ref, int64_t nr, int64_t d, int64_t k,
                          uint32_t* idx, double* d64, float* dist) {
    if (nq <= 0 || nr <= 0 || d <= 0) return ORACLE_SHAPE;
    if (k <= 0 || k > nr) return ORACLE_INVALID_PARAMETER;
    int failed = 0;
#pragma omp parallel
    {
        pair_f64* top = (pair_f64*)malloc(sizeof(pair_f64) * (size_t)(k + 1));
        if (!top) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 4)
            for (int64_t r = 0; r < nq; r++) {
                int64_t have = 0;
                double limit = INFINITY;
                for (int64_t j = 0; j < nr; j++) {
                    double s = sq_dist_f64_below(q + r * d, ref + j * d, d, limit);
                    if (s > limit) continue;
                    double v = sqrt(s > 0.0 ? s : 0.0);
                    pair_f64 cnd = {v, (uint32_t)j};
                    if (have == k) {
                        pair_f64 w = top[k - 1];
                        if (!(v < w.d || (v == w.d && cnd.id < w.id))) continue;
                        have--;
                    }
                    int64_t s2 = have;
                    while (s2 > 0 &&
                           (v < top[s2 - 1].d || (v == top[s2 - 1].d && cnd.id < top[s2 - 1].id))) {
                        top[s2] = top[s2 - 1];
                        s2--;
                    }
                    top[s2] = cnd;
                    have++;
                    if (have == k) {
                        double kth = top[k - 1].d;
                        limit = kth * kth * (1.0 + 1e-12);
                    }
                }
                for (int64_t t = 0; t < k; t++) {
                    idx[r * k + t] = top[t].id;
                    if (d64) d64[r * k + t] = top[t].d;
                    if (dist) dist[r * k + t] = (float)top[t].d;
                }
            }
        }
        free(top);
    }
    return failed ? ORACLE_OOM : ORACLE_OK;
}

/*
 * FP64 cosine kNN, the definition scanpy/sklearn use (the reference has no
 * cosine metric): d = 1 - a.b / (|a| |b|), all in float64 with dimension-order
 * sums and no fused operations; k non-self neighbours ordered by (d, j).
 * Zero rows are rejected (ORACLE_SHAPE).
 */
int oracle_knn_cosine_fp64_rows(const float* x, int64_t n, int64_t d, int64_t k,
                                const int64_t* rows, int64_t nrows, uint32_t* idx, double* d64,
                                float* dist) {
    int rc = check_knn_args(n, d, k);
    if (rc) return rc;
    if (rows == NULL) nrows = n;
    double* norms = (double*)malloc(sizeof(double) * (size_t)n);
    if (!norms) return ORACLE_OOM;
    for (int64_t i = 0; i < n; i++) {
        double s = 0.0;
        for (int64_t t = 0; t < d; t++) {
            double v = (double)x[i * d + t];
            double p = v * v;
            s = s + p;
        }
        norms[i] = sqrt(s);
        if (!(norms[i] > 0.0)) {
            free(norms);
            return ORACLE_SHAPE;
        }
    }
    int failed = 0;
#pragma omp parallel
    {
        pair_f64* top = (pair_f64*)malloc(sizeof(pair_f64) * (size_t)(k + 1));
        if (!top) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 4)
            for (int64_t r = 0; r < nrows; r++) {
                int64_t q = rows ? rows[r] : r;
                int64_t have = 0;
                for (int64_t j = 0; j < n; j++) {
                    if (j == q) continue;
                    double dot = 0.0;
                    for (int64_t t = 0; t < d; t++) {
                        double p = (double)x[q * d + t] * (double)x[j * d + t];
                        dot = dot + p;
                    }
                    double den = norms[q] * norms[j];
                    double v = 1.0 - dot / den;
                    pair_f64 cnd = {v, (uint32_t)j};
                    if (have == k) {
                        pair_f64 w = top[k - 1];
                        if (!(v < w.d || (v == w.d && cnd.id < w.id))) continue;
                        have--;
                    }
                    int64_t s2 = have;
                    while (s2 > 0 &&
                           (v < top[s2 - 1].d || (v == top[s2 - 1].d && cnd.id < top[s2 - 1].id))) {
                        top[s2] = top[s2 - 1];
                        s2--;
                    }
                    top[s2] = cnd;
                    have++;
                }
                for (int64_t t = 0; t < k; t++) {
                    idx[r * k + t] = top[t].id;
                    if (d64) d64[r * k + t] = top[t].d;
                    if (dist) dist[r * k + t] = (float)top[t].d;
                }
            }
        }
        free(top);
    }
    free(norms);
    return failed ? ORACLE_OOM : ORACLE_OK;
}

/*
 * smooth_knn_distances, neighbors.rs:239-298 (umap-learn semantics):
 * row width k+1 with the implied self entry, target log2(k+1) in f64, the
 * global mean by ndarray's unrolled sum, rho = first d > 0, 64 f32 bisection
 * steps with the doubling branch, f64 tolerance test, and the sigma floor
 * 1e-3 * (row mean if rho > 0 else global mean).
 */
int oracle_smooth_knn(const float* dist, int64_t n, int64_t k, float* sigmas, float* rhos) {
    if (n <= 0 || k <= 0) return ORACLE_SHAPE;
    const int64_t width = k + 1;
    const double target = log2((double)width);
    const float mean_distance = oracle_unrolled_sum_f32(dist, n * k) / (float)(n * k);
    /* Rows are independent: threads split them, the arithmetic per row is
     * the sequential one below. */
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; r++) {
        const float* row = dist + r * k;
        float rho = 0.0f;
        for (int64_t j = 0; j < k; j++)
            if (row[j] > 0.0f) {
                rho = row[j];
                break;
            }
        float low = 0.0f, high = FLT_MAX, mid = 1.0f;
        for (int it = 0; it < 64; it++) {
            float card = 0.0f;
            for (int64_t j = 0; j < k; j++) {
                float offset = row[j] - rho;
                float term = offset > 0.0f ? expf(-offset / mid) : 1.0f;
                card = card + term;
            }
            double c64 = (double)card;
            if (fabs(c64 - target) < 1e-5) break;
            if (c64 > target) {
                high = mid;
                mid = (low + high) / 2.0f;
            } else {
                low = mid;
                mid = high >= FLT_MAX ? mid * 2.0f : (low + high) / 2.0f;
            }
        }
        float reference = rho > 0.0f ? oracle_unrolled_sum_f32(row, k) / (float)width : mean_distance;
        float floor_ = 1e-3f * reference;
        sigmas[r] = fmaxf(mid, floor_);
        rhos[r] = rho;
    }
    return ORACLE_OK;
}

typedef struct {
    uint32_t col;
    uint32_t pos;
    float w;
} edge_t;

static int cmp_edge(const void* a, const void* b) {
    const edge_t* x = (const edge_t*)a;
    const edge_t* y = (const edge_t*)b;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return (x->pos > y->pos) - (x->pos < y->pos);
}

/*
 * connectivities, neighbors.rs:208-231 with directed_weights (:300-327) and
 * symmetrise (:329-372).  Outputs a CSR (indptr n+1, indices/values up to
 * 2nk entries) and its nnz.  Validation: shape/empty/out-of-range ids give
 * ORACLE_SHAPE (:209-227).
 */
int oracle_connectivities(const uint32_t* idx, const float* dist, int64_t n, int64_t k,
                          uint32_t* indptr, uint32_t* indices, float* values, int64_t* nnz_out) {
    if (n <= 0 || k <= 0) return ORACLE_SHAPE;
    for (int64_t i = 0; i < n * k; i++)
        if ((int64_t)idx[i] >= n) return ORACLE_SHAPE;
    float* sigmas = (float*)malloc(sizeof(float) * (size_t)n);
    float* rhos = (float*)malloc(sizeof(float) * (size_t)n);
    edge_t* fwd = (edge_t*)malloc(sizeof(edge_t) * (size_t)(n * k));
    int64_t* fcount = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int64_t* tcount = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    edge_t* bwd = (edge_t*)malloc(sizeof(edge_t) * (size_t)(n * k));
    int64_t* tfill = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    if (!sigmas || !rhos || !fwd || !fcount || !tcount || !bwd || !tfill) {
        free(sigmas); free(rhos); free(fwd); free(fcount); free(tcount); free(bwd); free(tfill);
        return ORACLE_OOM;
    }
    oracle_smooth_knn(dist, n, k, sigmas, rhos);
    /* directed_weights: skip self, w = 1 when offset <= 0 or sigma == 0,
     * else exp(-offset / sigma); drop w == 0; sort each row by column. */
    for (int64_t r = 0; r < n; r++) {
        edge_t* row = fwd + r * k;
        int64_t m = 0;
        for (int64_t j = 0; j < k; j++) {
            uint32_t nb = idx[r * k + j];
            if ((int64_t)nb == r) continue;
            float offset = dist[r * k + j] - rhos[r];
            float w = (offset <= 0.0f || sigmas[r] == 0.0f) ? 1.0f : expf(-offset / sigmas[r]);
            if (w != 0.0f) {
                row[m].col = nb;
                row[m].pos = (uint32_t)j;
                row[m].w = w;
                m++;
            }
        }
        qsort(row, (size_t)m, sizeof(edge_t), cmp_edge);
        fcount[r] = m;
        for (int64_t t = 0; t < m; t++) tcount[row[t].col + 1]++;
    }
    /* symmetrise: transpose lists sorted by source row, then a sorted merge
     * with value (w + r) - (w * r). */
    for (int64_t r = 0; r < n; r++) tcount[r + 1] += tcount[r];
    for (int64_t r = 0; r < n; r++) {
        const edge_t* row = fwd + r * k;
        for (int64_t t = 0; t < fcount[r]; t++) {
            uint32_t c = row[t].col;
            edge_t e = {(uint32_t)r, 0, row[t].w};
            bwd[tcount[c] + tfill[c]] = e;
            tfill[c]++;
        }
    }
    /* Rows were visited in increasing order, so each transpose list is
     * already sorted by source row. */
    int64_t nnz = 0;
    indptr[0] = 0;
    for (int64_t r = 0; r < n; r++) {
        const edge_t* f = fwd + r * k;
        const edge_t* b = bwd + tcount[r];
        int64_t nf = fcount[r], nbk = tcount[r + 1] - tcount[r];
        int64_t fi = 0, bi = 0;
        while (fi < nf || bi < nbk) {
            uint32_t col;
            if (fi < nf && bi < nbk)
                col = f[fi].col < b[bi].col ? f[fi].col : b[bi].col;
            else if (fi < nf)
                col = f[fi].col;
            else
                col = b[bi].col;
            float w = 0.0f, rv = 0.0f;
            if (fi < nf && f[fi].col == col) {
                w = f[fi].w;
                fi++;
            }
            if (bi < nbk && b[bi].col == col) {
                rv = b[bi].w;
                bi++;
            }
            indices[nnz] = col;
            float sum = w + rv;
            float prod = w * rv;
            values[nnz] = sum - prod;
            nnz++;
        }
        indptr[r + 1] = (uint32_t)nnz;
    }
    *nnz_out = nnz;
    free(sigmas); free(rhos); free(fwd); free(fcount); free(tcount); free(bwd); free(tfill);
    return ORACLE_OK;
}

/* Directed weights alone (neighbors.rs:300-327), as a dense (n, k) array in
 * the input's column order (0 where an entry is skipped or dropped). */
int oracle_directed_weights(const uint32_t* idx, const float* dist, int64_t n, int64_t k,
                            float* weights) {
    if (n <= 0 || k <= 0) return ORACLE_SHAPE;
    float* sigmas = (float*)malloc(sizeof(float) * (size_t)n);
    float* rhos = (float*)malloc(sizeof(float) * (size_t)n);
    if (!sigmas || !rhos) {
        free(sigmas);
        free(rhos);
        return ORACLE_OOM;
    }
    oracle_smooth_knn(dist, n, k, sigmas, rhos);
    for (int64_t r = 0; r < n; r++)
        for (int64_t j = 0; j < k; j++) {
            uint32_t nb = idx[r * k + j];
            float w = 0.0f;
            if ((int64_t)nb != r) {
                float offset = dist[r * k + j] - rhos[r];
                w = (offset <= 0.0f || sigmas[r] == 0.0f) ? 1.0f : expf(-offset / sigmas[r]);
            }
            weights[r * k + j] = w;
        }
    free(sigmas);
    free(rhos);
    return ORACLE_OK;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
