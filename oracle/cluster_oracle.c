/*
 * cluster_oracle.c -- the ORACLE for community detection on the graph.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests call it as the checker; the shipped
 * CUDA library never links, loads or calls it.
 *
 * A C restatement of crates/scrust-core/src/cluster.rs (Leiden and Louvain
 * maximising RBConfiguration modularity):
 *   graph_from_csr      Graph::from_csr (:214-290): (A + A^T) / 2 as flat
 *                       neighbour lists, f64 strengths and total
 *   score               score (:311-332): Q community by community
 *   move_nodes          move_nodes (:386-496): queue-based local moving,
 *                       best gain with ties to the smaller id, leaving for an
 *                       empty community on a negative best gain
 *   refine              refine (:517-641) with sample_merge (:650-675): the
 *                       well-connected singleton merges inside each community
 *   aggregate, optimise, compact, by_descending_size (:681-850)
 *   oracle_leiden / oracle_louvain / oracle_modularity  (:88-168)
 * One substitution: the reference draws its visit orders and merge samples
 * from rand's StdRng (ChaCha12), which is not restated here; this oracle
 * draws them from a splitmix64 stream (Fisher-Yates shuffles, f64 uniforms
 * from the top 53 bits).  Partitions therefore match the reference's in
 * distribution, not label for label; the reference's own cluster tests
 * (:882-1100: hand-computed modularity, clique recovery, Leiden >= Louvain,
 * seeds, resolution, label order, symmetrisation, errors, connectedness) pin
 * it -- tests/test_cluster_oracle.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { C_OK = 0, C_SHAPE = 1, C_INVALID_PARAMETER = 2, C_OOM = 6 };

static const double REFINEMENT_RANDOMNESS = 0.01;

typedef struct {
    uint64_t s;
} srng;

static uint64_t rng_u64(srng* r) {
    r->s += 0x9E3779B97F4A7C15ull;
    uint64_t z = r->s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double rng_f64(srng* r) { return (double)(rng_u64(r) >> 11) * 1.1102230246251565e-16; }
static void shuffle(uint32_t* a, int64_t n, srng* r) {
    for (int64_t i = n - 1; i > 0; i--) {
        int64_t j = (int64_t)(((unsigned __int128)rng_u64(r) * (uint64_t)(i + 1)) >> 64);
        uint32_t t = a[i];
        a[i] = a[j];
        a[j] = t;
    }
}

typedef struct {
    int64_t n;
    int64_t* indptr;
    uint32_t* nb;
    double* w;
    double* strength;
    double total;
} graph_t;

static void graph_free(graph_t* g) {
    free(g->indptr);
    free(g->nb);
    free(g->w);
    free(g->strength);
    memset(g, 0, sizeof(*g));
}

static int graph_from_csr(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n,
                          int64_t n_cols, graph_t* g) {
    memset(g, 0, sizeof(*g));
    if (n <= 0 || n_cols != n) return C_SHAPE;
    const int64_t nnz = indptr[n];
    for (int64_t e = 0; e < nnz; e++)
        if (!isfinite(values[e]) || values[e] < 0.0f) return C_INVALID_PARAMETER;
    g->n = n;
    g->indptr = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    g->nb = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(2 * nnz + 1));
    g->w = (double*)malloc(sizeof(double) * (size_t)(2 * nnz + 1));
    g->strength = (double*)calloc((size_t)n, sizeof(double));
    int64_t* cursor = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    if (!g->indptr || !g->nb || !g->w || !g->strength || !cursor) {
        free(cursor);
        graph_free(g);
        return C_OOM;
    }
    for (int64_t r = 0; r < n; r++)
        for (int64_t e = indptr[r]; e < indptr[r + 1]; e++) {
            g->indptr[r + 1]++;
            g->indptr[indices[e] + 1]++;
        }
    for (int64_t v = 0; v < n; v++) g->indptr[v + 1] += g->indptr[v];
    for (int64_t v = 0; v < n; v++) cursor[v] = g->indptr[v];
    for (int64_t r = 0; r < n; r++)
        for (int64_t e = indptr[r]; e < indptr[r + 1]; e++) {
            const uint32_t c = indices[e];
            const double half = (double)values[e] / 2.0;
            g->nb[cursor[r]] = c;
            g->w[cursor[r]++] = half;
            g->nb[cursor[c]] = (uint32_t)r;
            g->w[cursor[c]++] = half;
        }
    free(cursor);
    double total = 0.0;
    for (int64_t v = 0; v < n; v++) {
        double s = 0.0;
        for (int64_t e = g->indptr[v]; e < g->indptr[v + 1]; e++) s += g->w[e];
        g->strength[v] = s;
        total += s;
    }
    g->total = total;
    if (!(total > 0.0)) {
        graph_free(g);
        return C_INVALID_PARAMETER;
    }
    return C_OK;
}

static double score(const graph_t* g, const uint32_t* labels, int64_t nc, double res) {
    double* internal = (double*)calloc((size_t)nc, sizeof(double));
    double* strength = (double*)calloc((size_t)nc, sizeof(double));
    for (int64_t v = 0; v < g->n; v++) {
        const uint32_t c = labels[v];
        strength[c] += g->strength[v];
        for (int64_t e = g->indptr[v]; e < g->indptr[v + 1]; e++)
            if (labels[g->nb[e]] == c) internal[c] += g->w[e];
    }
    double q = 0.0;
    for (int64_t c = 0; c < nc; c++)
        q += internal[c] / g->total - res * (strength[c] / g->total) * (strength[c] / g->total);
    free(internal);
    free(strength);
    return q;
}

/* Communities with a free list of unused ids (:340-381). */
typedef struct {
    uint32_t* of;
    double* strength;
    int64_t* size;
    uint32_t* free_ids;
    int64_t n_free;
} comms_t;

static int cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return (x > y) - (x < y);
}

static int move_nodes(const graph_t* g, comms_t* cm, double res, srng* rng) {
    const int64_t n = g->n;
    uint32_t* queue = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    char* queued = (char*)malloc((size_t)n);
    double* edge_to = (double*)calloc((size_t)n, sizeof(double));
    char* seen = (char*)calloc((size_t)n, 1);
    uint32_t* touched = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        queue[i] = (uint32_t)i;
        queued[i] = 1;
    }
    shuffle(queue, n, rng);
    /* A ring buffer: at most n nodes are queued at a time. */
    int64_t head = 0, count = n;
    int moved_any = 0;
    while (count > 0) {
        const int64_t node = queue[head];
        head = (head + 1) % n;
        count--;
        queued[node] = 0;
        const double ks = g->strength[node];
        const uint32_t prev = cm->of[node];
        cm->strength[prev] -= ks;
        if (--cm->size[prev] == 0) cm->free_ids[cm->n_free++] = prev;
        int64_t nt = 0;
        for (int64_t e = g->indptr[node]; e < g->indptr[node + 1]; e++) {
            if ((int64_t)g->nb[e] == node) continue;
            const uint32_t c = cm->of[g->nb[e]];
            if (!seen[c]) {
                seen[c] = 1;
                touched[nt++] = c;
            }
            edge_to[c] += g->w[e];
        }
        qsort(touched, (size_t)nt, sizeof(uint32_t), cmp_u32);
#define GAIN(c) (edge_to[(c)] - res * cm->strength[(c)] * ks / g->total)
        uint32_t best = prev;
        double best_gain = GAIN(prev);
        for (int64_t t = 0; t < nt; t++) {
            const double cand = GAIN(touched[t]);
            if (cand > best_gain) {
                best_gain = cand;
                best = touched[t];
            }
        }
#undef GAIN
        const int has_empty = cm->n_free > 0;
        const uint32_t empty = has_empty ? cm->free_ids[cm->n_free - 1] : 0;
        if (has_empty && best_gain < 0.0) best = empty;
        if (best != prev) {
            if (has_empty && best == empty) cm->n_free--;
            cm->of[node] = best;
            cm->strength[best] += ks;
            cm->size[best]++;
            moved_any = 1;
            for (int64_t e = g->indptr[node]; e < g->indptr[node + 1]; e++) {
                const uint32_t v = g->nb[e];
                if ((int64_t)v != node && !queued[v] && cm->of[v] != best) {
                    queued[v] = 1;
                    queue[(head + count) % n] = v;
                    count++;
                }
            }
        } else {
            if (cm->size[prev] == 0) cm->n_free--;
            cm->of[node] = prev;
            cm->strength[prev] += ks;
            cm->size[prev]++;
        }
        for (int64_t t = 0; t < nt; t++) {
            edge_to[touched[t]] = 0.0;
            seen[touched[t]] = 0;
        }
    }
    free(queue);
    free(queued);
    free(edge_to);
    free(seen);
    free(touched);
    return moved_any;
}

/* compact (:807-826): the ids in use renumbered 0.. in ascending order. */
static int64_t compact(const uint32_t* labels, int64_t n, uint32_t* out) {
    uint32_t width = 0;
    for (int64_t i = 0; i < n; i++) width = labels[i] + 1 > width ? labels[i] + 1 : width;
    uint32_t* map = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(width + 1));
    for (uint32_t i = 0; i < width; i++) map[i] = UINT32_MAX;
    for (int64_t i = 0; i < n; i++) map[labels[i]] = 0;
    int64_t next = 0;
    for (uint32_t id = 0; id < width; id++)
        if (map[id] == 0) map[id] = (uint32_t)next++;
    for (int64_t i = 0; i < n; i++) out[i] = map[labels[i]];
    free(map);
    return next;
}

static void group_by(const uint32_t* labels, int64_t n, int64_t nl, int64_t* offsets, uint32_t* members) {
    memset(offsets, 0, sizeof(int64_t) * (size_t)(nl + 1));
    for (int64_t i = 0; i < n; i++) offsets[labels[i] + 1]++;
    for (int64_t l = 0; l < nl; l++) offsets[l + 1] += offsets[l];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nl + 1));
    memcpy(cur, offsets, sizeof(int64_t) * (size_t)(nl + 1));
    for (int64_t i = 0; i < n; i++) members[cur[labels[i]]++] = (uint32_t)i;
    free(cur);
}

static int well_connected(double cut, double part, double subset, double res, double total) {
    return cut >= res * part * (subset - part) / total;
}

static int sample_merge(const uint32_t* ct, const double* cg, int64_t nch, srng* rng, uint32_t* out) {
    if (nch == 0) return 0;
    int64_t bi = 0;
    for (int64_t i = 1; i < nch; i++)
        if (cg[i] >= cg[bi]) bi = i; /* max_by keeps the last of equal maxima */
    const double largest = cg[bi];
    double total = 0.0;
    double* wts = (double*)malloc(sizeof(double) * (size_t)nch);
    for (int64_t i = 0; i < nch; i++) {
        wts[i] = exp((cg[i] - largest) / REFINEMENT_RANDOMNESS);
        total += wts[i];
    }
    if (!isfinite(total) || total <= 0.0) {
        free(wts);
        *out = ct[bi];
        return 1;
    }
    double draw = rng_f64(rng) * total;
    for (int64_t i = 0; i < nch; i++) {
        draw -= wts[i];
        if (draw <= 0.0) {
            free(wts);
            *out = ct[i];
            return 1;
        }
    }
    free(wts);
    *out = ct[bi];
    return 1;
}

static void refine(const graph_t* g, const uint32_t* part, int64_t nc, double res, srng* rng, uint32_t* of) {
    const int64_t n = g->n;
    int64_t* offsets = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nc + 1));
    uint32_t* members = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    group_by(part, n, nc, offsets, members);
    double* sub_strength = (double*)malloc(sizeof(double) * (size_t)n);
    int64_t* sub_size = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    double* sub_boundary = (double*)calloc((size_t)n, sizeof(double));
    double* sub_internal = (double*)calloc((size_t)n, sizeof(double));
    char* in_subset = (char*)calloc((size_t)n, 1);
    double* to_subset = (double*)calloc((size_t)n, sizeof(double));
    double* edge_to = (double*)calloc((size_t)n, sizeof(double));
    char* seen = (char*)calloc((size_t)n, 1);
    uint32_t* targets = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    uint32_t* ct = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    double* cg = (double*)malloc(sizeof(double) * (size_t)n);
    uint32_t* visit = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    for (int64_t v = 0; v < n; v++) {
        of[v] = (uint32_t)v;
        sub_strength[v] = g->strength[v];
        sub_size[v] = 1;
    }
    for (int64_t c = 0; c < nc; c++) {
        const uint32_t* subset = members + offsets[c];
        const int64_t len = offsets[c + 1] - offsets[c];
        if (len < 2) continue;
        for (int64_t i = 0; i < len; i++) in_subset[subset[i]] = 1;
        double subset_strength = 0.0;
        for (int64_t i = 0; i < len; i++) {
            const uint32_t v = subset[i];
            double inside = 0.0;
            for (int64_t e = g->indptr[v]; e < g->indptr[v + 1]; e++)
                if (g->nb[e] != v && in_subset[g->nb[e]]) inside += g->w[e];
            to_subset[v] = inside;
            sub_boundary[v] = inside;
            sub_internal[v] = 0.0;
            subset_strength += g->strength[v];
        }
        int64_t nv = 0;
        for (int64_t i = 0; i < len; i++)
            if (well_connected(to_subset[subset[i]], g->strength[subset[i]], subset_strength, res, g->total))
                visit[nv++] = subset[i];
        shuffle(visit, nv, rng);
        for (int64_t vi = 0; vi < nv; vi++) {
            const uint32_t node = visit[vi];
            if (sub_size[node] != 1) continue;
            int64_t nt = 0;
            for (int64_t e = g->indptr[node]; e < g->indptr[node + 1]; e++) {
                const uint32_t nb = g->nb[e];
                if (nb == node || !in_subset[nb]) continue;
                const uint32_t t = of[nb];
                if (!seen[t]) {
                    seen[t] = 1;
                    targets[nt++] = t;
                }
                edge_to[t] += g->w[e];
            }
            qsort(targets, (size_t)nt, sizeof(uint32_t), cmp_u32);
            int64_t nch = 0;
            for (int64_t i = 0; i < nt; i++) {
                const uint32_t t = targets[i];
                const double gain = edge_to[t] - res * sub_strength[t] * g->strength[node] / g->total;
                const double cut = sub_boundary[t] - sub_internal[t];
                if (gain >= 0.0 && well_connected(cut, sub_strength[t], subset_strength, res, g->total)) {
                    ct[nch] = t;
                    cg[nch++] = gain;
                }
            }
            uint32_t target;
            if (sample_merge(ct, cg, nch, rng, &target)) {
                sub_internal[target] += 2.0 * edge_to[target];
                sub_boundary[target] += to_subset[node];
                sub_strength[target] += g->strength[node];
                sub_size[target] += 1;
                sub_size[node] = 0;
                of[node] = target;
            }
            for (int64_t i = 0; i < nt; i++) {
                edge_to[targets[i]] = 0.0;
                seen[targets[i]] = 0;
            }
        }
        for (int64_t i = 0; i < len; i++) in_subset[subset[i]] = 0;
    }
    free(offsets); free(members); free(sub_strength); free(sub_size); free(sub_boundary); free(sub_internal);
    free(in_subset); free(to_subset); free(edge_to); free(seen); free(targets); free(ct); free(cg); free(visit);
}

static void aggregate(const graph_t* g, const uint32_t* labels, int64_t nc, graph_t* out) {
    int64_t* offsets = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nc + 1));
    uint32_t* members = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)g->n);
    group_by(labels, g->n, nc, offsets, members);
    const int64_t cap = g->indptr[g->n] + 1;
    out->n = nc;
    out->indptr = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nc + 1));
    out->nb = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)cap);
    out->w = (double*)malloc(sizeof(double) * (size_t)cap);
    out->strength = (double*)malloc(sizeof(double) * (size_t)nc);
    double* edge_to = (double*)calloc((size_t)nc, sizeof(double));
    char* seen = (char*)calloc((size_t)nc, 1);
    uint32_t* touched = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nc);
    int64_t m = 0;
    out->indptr[0] = 0;
    for (int64_t c = 0; c < nc; c++) {
        int64_t nt = 0;
        for (int64_t i = offsets[c]; i < offsets[c + 1]; i++) {
            const uint32_t v = members[i];
            for (int64_t e = g->indptr[v]; e < g->indptr[v + 1]; e++) {
                const uint32_t t = labels[g->nb[e]];
                if (!seen[t]) {
                    seen[t] = 1;
                    touched[nt++] = t;
                }
                edge_to[t] += g->w[e];
            }
        }
        qsort(touched, (size_t)nt, sizeof(uint32_t), cmp_u32);
        for (int64_t i = 0; i < nt; i++) {
            out->nb[m] = touched[i];
            out->w[m++] = edge_to[touched[i]];
            edge_to[touched[i]] = 0.0;
            seen[touched[i]] = 0;
        }
        out->indptr[c + 1] = m;
    }
    for (int64_t c = 0; c < nc; c++) {
        double s = 0.0;
        for (int64_t e = out->indptr[c]; e < out->indptr[c + 1]; e++) s += out->w[e];
        out->strength[c] = s;
    }
    out->total = g->total;
    free(offsets); free(members); free(edge_to); free(seen); free(touched);
}

/* optimise (:732-784). Returns n_communities; labels written to out. */
static int64_t optimise(const graph_t* g0, const uint32_t* initial, int64_t n_initial, double res, int refinement,
                        srng* rng, uint32_t* out) {
    graph_t level = *g0;
    int owned = 0;
    const int64_t n0 = g0->n;
    uint32_t* fold = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n0);
    for (int64_t i = 0; i < n0; i++) fold[i] = (uint32_t)i;
    uint32_t* level_labels = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n0);
    memcpy(level_labels, initial, sizeof(uint32_t) * (size_t)n0);
    int64_t level_comms = n_initial;
    for (;;) {
        const int64_t n = level.n;
        comms_t cm;
        cm.of = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
        cm.strength = (double*)calloc((size_t)n, sizeof(double));
        cm.size = (int64_t*)calloc((size_t)n, sizeof(int64_t));
        cm.free_ids = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
        cm.n_free = 0;
        for (int64_t id = n - 1; id >= level_comms; id--) cm.free_ids[cm.n_free++] = (uint32_t)id;
        for (int64_t v = 0; v < n; v++) {
            cm.of[v] = level_labels[v];
            cm.strength[level_labels[v]] += level.strength[v];
            cm.size[level_labels[v]]++;
        }
        const int moved = move_nodes(&level, &cm, res, rng);
        uint32_t* partition = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
        const int64_t ncomm = compact(cm.of, n, partition);
        free(cm.of); free(cm.strength); free(cm.size); free(cm.free_ids);
        if (!moved || ncomm == n) {
            for (int64_t i = 0; i < n0; i++) out[i] = partition[fold[i]];
            free(partition); free(fold); free(level_labels);
            if (owned) graph_free(&level);
            return ncomm;
        }
        uint32_t* collapse = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
        int64_t ncol;
        if (refinement) {
            uint32_t* sub = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
            refine(&level, partition, ncomm, res, rng, sub);
            ncol = compact(sub, n, collapse);
            free(sub);
        } else {
            memcpy(collapse, partition, sizeof(uint32_t) * (size_t)n);
            ncol = ncomm;
        }
        graph_t next;
        aggregate(&level, collapse, ncol, &next);
        uint32_t* next_labels = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)ncol);
        for (int64_t v = 0; v < n; v++) next_labels[collapse[v]] = partition[v];
        for (int64_t i = 0; i < n0; i++) fold[i] = collapse[fold[i]];
        if (owned) graph_free(&level);
        level = next;
        owned = 1;
        free(level_labels);
        level_labels = next_labels;
        level_comms = ncomm;
        free(partition);
        free(collapse);
    }
}

/* by_descending_size (:828-850): largest community 0, ties by smaller id. */
static void by_descending_size(uint32_t* labels, int64_t n, int64_t nc) {
    int64_t* size = (int64_t*)calloc((size_t)nc, sizeof(int64_t));
    uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nc);
    uint32_t* rank = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)nc);
    for (int64_t i = 0; i < n; i++) size[labels[i]]++;
    for (int64_t c = 0; c < nc; c++) order[c] = (uint32_t)c;
    /* stable insertion sort by descending size */
    for (int64_t i = 1; i < nc; i++) {
        uint32_t v = order[i];
        int64_t j = i;
        while (j > 0 && size[order[j - 1]] < size[v]) {
            order[j] = order[j - 1];
            j--;
        }
        order[j] = v;
    }
    for (int64_t c = 0; c < nc; c++) rank[order[c]] = (uint32_t)c;
    for (int64_t i = 0; i < n; i++) labels[i] = rank[labels[i]];
    free(size);
    free(order);
    free(rank);
}

static int run(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n, int64_t n_cols,
               double res, int64_t n_iterations, uint64_t seed, int leiden, uint32_t* labels, double* modularity,
               int64_t* n_communities) {
    if (!isfinite(res) || res <= 0.0) return C_INVALID_PARAMETER;
    if (leiden && n_iterations <= 0) return C_INVALID_PARAMETER;
    graph_t g;
    int rc = graph_from_csr(indptr, indices, values, n, n_cols, &g);
    if (rc) return rc;
    srng rng = {seed};
    uint32_t* cur = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    uint32_t* found = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    for (int64_t i = 0; i < n; i++) cur[i] = (uint32_t)i;
    int64_t nc = n;
    const int64_t passes = leiden ? n_iterations : 1;
    for (int64_t it = 0; it < passes; it++) {
        const int64_t fnc = optimise(&g, cur, nc, res, leiden, &rng, found);
        if (leiden && memcmp(found, cur, sizeof(uint32_t) * (size_t)n) == 0) break;
        memcpy(cur, found, sizeof(uint32_t) * (size_t)n);
        nc = fnc;
    }
    by_descending_size(cur, n, nc);
    memcpy(labels, cur, sizeof(uint32_t) * (size_t)n);
    *modularity = score(&g, labels, nc, res);
    *n_communities = nc;
    free(cur);
    free(found);
    graph_free(&g);
    return C_OK;
}

int oracle_leiden(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n, int64_t n_cols,
                  double resolution, int64_t n_iterations, uint64_t seed, uint32_t* labels, double* modularity,
                  int64_t* n_communities) {
    return run(indptr, indices, values, n, n_cols, resolution, n_iterations, seed, 1, labels, modularity,
               n_communities);
}

int oracle_louvain(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n, int64_t n_cols,
                   double resolution, uint64_t seed, uint32_t* labels, double* modularity, int64_t* n_communities) {
    return run(indptr, indices, values, n, n_cols, resolution, 1, seed, 0, labels, modularity, n_communities);
}

int oracle_modularity(const uint32_t* indptr, const uint32_t* indices, const float* values, int64_t n, int64_t n_cols,
                      const uint32_t* labels, int64_t n_labels, double resolution, double* out) {
    if (!isfinite(resolution) || resolution <= 0.0) return C_INVALID_PARAMETER;
    graph_t g;
    int rc = graph_from_csr(indptr, indices, values, n, n_cols, &g);
    if (rc) return rc;
    if (n_labels != n) {
        graph_free(&g);
        return C_SHAPE;
    }
    uint32_t mx = 0;
    for (int64_t i = 0; i < n; i++) mx = labels[i] > mx ? labels[i] : mx;
    if ((int64_t)mx + 1 > n) {
        graph_free(&g);
        return C_INVALID_PARAMETER;
    }
    *out = score(&g, labels, (int64_t)mx + 1, resolution);
    graph_free(&g);
    return C_OK;
}
