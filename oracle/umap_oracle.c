/*
 * umap_oracle.c -- the ORACLE for the UMAP layout on the connectivities.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests and the smoke entry point call it as
 * the checker; the shipped CUDA library never links, loads or calls it.
 *
 * A C restatement of crates/scrust-core/src/umap.rs (the reference's CPU
 * layout, a transcription of umap-learn's sequential SGD):
 *   oracle_tau_*             TauRng (umap.rs:174-229): splitmix64 seeding of
 *                            the three tau88 words, umap-learn's recurrence
 *   oracle_fit_ab_params     fit_ab_params (:272-391): damped Gauss-Newton on
 *                            300 points of the offset exponential
 *   oracle_umap              umap (:64-84): validation (:86-110), the edge
 *                            list with its firing intervals (:113-170), the
 *                            random layout and its rescale (:232-257), and
 *                            optimize_layout (:393-452) with attraction,
 *                            repulsion and the +-4 clip (:454-509)
 * Every f32 operation is written out as the reference performs it (built with
 * -ffp-contract=off, so nothing is fused); powf is the host libm's, as Rust's
 * f32::powf is.
 *
 * Parity of this restatement is pinned by the reference's own tests of
 * umap.rs (:1092-1254): the umap-learn fitted-curve table, two-cluster
 * separation, the zero-negative-rate collapse, seed reproducibility, and the
 * scanpy neighbourhood check on its 80-cell golden graph and layout
 * (tests/golden/umap_reference_80_cells.json, parsed from the source text).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { U_OK = 0, U_SHAPE = 1, U_INVALID_PARAMETER = 2, U_OOM = 6 };

static const float REPULSION_STRENGTH = 1.0f;
static const float GRADIENT_CLIP = 4.0f;
static const float REPULSION_EPSILON = 0.001f;
static const float INIT_RANGE = 10.0f;

typedef struct {
    uint32_t s[3];
} tau_rng;

static uint64_t splitmix_next(uint64_t* state) {
    *state += 0x9E3779B97F4A7C15ull;
    uint64_t z = *state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static tau_rng tau_new(uint64_t seed) {
    tau_rng r;
    uint64_t sm = seed;
    r.s[0] = (uint32_t)splitmix_next(&sm) | 0x2u;
    r.s[1] = (uint32_t)splitmix_next(&sm) | 0x8u;
    r.s[2] = (uint32_t)splitmix_next(&sm) | 0x10u;
    return r;
}

static uint32_t tau_next(tau_rng* r) {
    uint32_t* s = r->s;
    s[0] = ((s[0] & 4294967294u) << 12) ^ (((s[0] << 13) ^ s[0]) >> 19);
    s[1] = ((s[1] & 4294967288u) << 4) ^ (((s[1] << 2) ^ s[1]) >> 25);
    s[2] = ((s[2] & 4294967280u) << 17) ^ (((s[2] << 3) ^ s[2]) >> 11);
    return s[0] ^ s[1] ^ s[2];
}

static float tau_unit(tau_rng* r) { return (float)tau_next(r) / (float)UINT32_MAX; }

/* The first `count` words of TauRng::new(seed), for checking the device's
 * generator word for word. */
void oracle_tau_words(uint64_t seed, int64_t count, uint32_t* out) {
    tau_rng r = tau_new(seed);
    for (int64_t i = 0; i < count; i++) out[i] = tau_next(&r);
}

/* ---- fit_ab_params ------------------------------------------------------- */

static void power_term(double x, double b, double* term, double* log_factor) {
    if (x <= 0.0) {
        *term = 0.0;
        *log_factor = 0.0;
    } else {
        *term = pow(x, 2.0 * b);
        *log_factor = 2.0 * log(x);
    }
}

static double model_value(double x, double a, double b) {
    double t, l;
    power_term(x, b, &t, &l);
    return 1.0 / (1.0 + a * t);
}

static double sum_squares(const double* xs, const double* ys, int n, double a, double b) {
    double s = 0.0;
    for (int i = 0; i < n; i++) {
        double r = model_value(xs[i], a, b) - ys[i];
        s += r * r;
    }
    return s;
}

int oracle_fit_ab_params(float min_dist_f, float spread_f, float* a_out, float* b_out) {
    if (!(spread_f > 0.0f)) return U_INVALID_PARAMETER;
    if (!(min_dist_f >= 0.0f && min_dist_f <= spread_f * 3.0f)) return U_INVALID_PARAMETER;
    enum { SAMPLES = 300 };
    double xs[SAMPLES], ys[SAMPLES];
    const double min_dist = (double)min_dist_f, spread = (double)spread_f;
    for (int i = 0; i < SAMPLES; i++) {
        double x = 3.0 * spread * (double)i / (double)(SAMPLES - 1);
        xs[i] = x;
        ys[i] = x < min_dist ? 1.0 : exp(-(x - min_dist) / spread);
    }
    double a = 1.0, b = 1.0, damping = 1e-3;
    double cost = sum_squares(xs, ys, SAMPLES, a, b);
    for (int it = 0; it < 200; it++) {
        double jaa = 0, jab = 0, jbb = 0, ga = 0, gb = 0;
        for (int i = 0; i < SAMPLES; i++) {
            double term, lf;
            power_term(xs[i], b, &term, &lf);
            double den = 1.0 + a * term;
            double sq = den * den;
            double residual = 1.0 / den - ys[i];
            double da = -term / sq;
            double db = -a * term * lf / sq;
            jaa += da * da;
            jab += da * db;
            jbb += db * db;
            ga += da * residual;
            gb += db * residual;
        }
        double daa = jaa * (1.0 + damping), dbb = jbb * (1.0 + damping);
        double det = daa * dbb - jab * jab;
        if (fabs(det) < DBL_EPSILON) break;
        double step_a = -(dbb * ga - jab * gb) / det;
        double step_b = -(daa * gb - jab * ga) / det;
        double ta = a + step_a, tb = b + step_b;
        if (ta <= 0.0 || tb <= 0.0) {
            damping *= 10.0;
            continue;
        }
        double tc = sum_squares(xs, ys, SAMPLES, ta, tb);
        if (tc < cost) {
            double improvement = cost - tc;
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
    return U_OK;
}

/* ---- the layout ------------------------------------------------------------ */

static float clipf(float v) { return v < -GRADIENT_CLIP ? -GRADIENT_CLIP : (v > GRADIENT_CLIP ? GRADIENT_CLIP : v); }

static float sq_dist(const float* y, int64_t l, int64_t r, int64_t dim) {
    float s = 0.0f;
    for (int64_t d = 0; d < dim; d++) {
        float diff = y[l + d] - y[r + d];
        float p = diff * diff;
        s = s + p;
    }
    return s;
}

/*
 * The whole reference layout.  Inputs: a square CSR graph (n rows, indptr
 * n+1, indices/values nnz).  Output: out (n, n_components) row-major.
 * Errors as umap.rs:86-110 (and fit_ab_params's parameter checks).
 */
int oracle_umap(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n, int64_t n_cols,
                int64_t n_components, int64_t n_epochs, float min_dist, float spread, float learning_rate,
                int64_t negative_sample_rate, uint64_t seed, float* out) {
    if (n_components <= 0 || n_epochs <= 0) return U_INVALID_PARAMETER;
    if (n <= 0 || indptr[n] == 0) return U_SHAPE;
    if (n_cols != n) return U_SHAPE;
    float a, b;
    int rc = oracle_fit_ab_params(min_dist, spread, &a, &b);
    if (rc) return rc;
    const int64_t nnz = indptr[n];
    /* EdgeList::from_graph */
    float max_weight = -INFINITY;
    for (int64_t e = 0; e < nnz; e++) max_weight = values[e] > max_weight ? values[e] : max_weight;
    const float threshold = max_weight / (float)n_epochs;
    uint32_t* head = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nnz);
    uint32_t* tail = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nnz);
    double* eps = (double*)malloc(sizeof(double) * (size_t)nnz);
    double* eps_neg = (double*)malloc(sizeof(double) * (size_t)nnz);
    double* next = (double*)malloc(sizeof(double) * (size_t)nnz);
    double* next_neg = (double*)malloc(sizeof(double) * (size_t)nnz);
    tau_rng* rngs = (tau_rng*)malloc(sizeof(tau_rng) * (size_t)n);
    if (!head || !tail || !eps || !eps_neg || !next || !next_neg || !rngs) {
        free(head); free(tail); free(eps); free(eps_neg); free(next); free(next_neg); free(rngs);
        return U_OOM;
    }
    int64_t m = 0;
    for (int64_t row = 0; row < n; row++)
        for (int64_t e = indptr[row]; e < indptr[row + 1]; e++) {
            float w = values[e];
            if (w <= 0.0f || w < threshold) continue;
            head[m] = (uint32_t)row;
            tail[m] = indices[e];
            eps[m] = (double)max_weight / (double)w;
            m++;
        }
    if (m == 0) {
        free(head); free(tail); free(eps); free(eps_neg); free(next); free(next_neg); free(rngs);
        return U_SHAPE;
    }
    const int64_t dim = n_components;
    /* random_layout + rescale_to_init_range */
    tau_rng init = tau_new(seed);
    for (int64_t i = 0; i < n * dim; i++) out[i] = (tau_unit(&init) * 2.0f - 1.0f) * INIT_RANGE;
    for (int64_t c = 0; c < dim; c++) {
        float lo = INFINITY, hi = -INFINITY;
        for (int64_t i = 0; i < n; i++) {
            float v = out[i * dim + c];
            lo = v < lo ? v : lo;
            hi = v > hi ? v : hi;
        }
        float range = hi - lo;
        for (int64_t i = 0; i < n; i++) {
            float v = out[i * dim + c];
            out[i * dim + c] = range > 0.0f ? INIT_RANGE * (v - lo) / range : 0.0f;
        }
    }
    /* optimize_layout */
    for (int64_t v = 0; v < n; v++) rngs[v] = tau_new(seed ^ ((uint64_t)v * 0x9E3779B97F4A7C15ull));
    for (int64_t e = 0; e < m; e++) {
        eps_neg[e] = negative_sample_rate ? eps[e] / (double)negative_sample_rate : INFINITY;
        next_neg[e] = eps_neg[e];
        next[e] = eps[e];
    }
    float alpha = learning_rate;
    for (int64_t epoch = 0; epoch < n_epochs; epoch++) {
        const double now = (double)epoch;
        for (int64_t e = 0; e < m; e++) {
            if (next[e] > now) continue;
            const int64_t cur = (int64_t)head[e] * dim, oth = (int64_t)tail[e] * dim;
            {
                float dist = sq_dist(out, cur, oth, dim);
                float coef = 0.0f;
                if (dist > 0.0f) {
                    float num = -2.0f * a * b * powf(dist, b - 1.0f);
                    float den = a * powf(dist, b) + 1.0f;
                    coef = num / den;
                }
                for (int64_t d = 0; d < dim; d++) {
                    float g = clipf(coef * (out[cur + d] - out[oth + d]));
                    out[cur + d] += g * alpha;
                    out[oth + d] -= g * alpha;
                }
            }
            next[e] += eps[e];
            if (negative_sample_rate == 0) continue;
            int64_t n_neg = (int64_t)((now - next_neg[e]) / eps_neg[e]);
            if (n_neg < 0) n_neg = 0;
            tau_rng* rng = &rngs[head[e]];
            for (int64_t t = 0; t < n_neg; t++) {
                const int64_t smp = (int64_t)(tau_next(rng) % (uint32_t)n) * dim;
                if (smp == cur) continue;
                float dist = sq_dist(out, cur, smp, dim);
                if (dist <= 0.0f) continue;
                float coef = 2.0f * REPULSION_STRENGTH * b / ((REPULSION_EPSILON + dist) * (a * powf(dist, b) + 1.0f));
                for (int64_t d = 0; d < dim; d++) {
                    float g = clipf(coef * (out[cur + d] - out[smp + d]));
                    out[cur + d] += g * alpha;
                }
            }
            next_neg[e] += (double)n_neg * eps_neg[e];
        }
        alpha = learning_rate * (1.0f - (float)epoch / (float)n_epochs);
    }
    free(head); free(tail); free(eps); free(eps_neg); free(next); free(next_neg); free(rngs);
    return U_OK;
}
