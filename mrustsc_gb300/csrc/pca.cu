// pca.cu -- truncated PCA of a cells x genes CSR matrix on the GPU, the step
// before the neighbours path (crates/scrust-core/src/pca.rs:74): its
// embedding can stay in HBM and go straight into the kNN graph build.
//
// The algorithm is the reference's randomised SVD (pca.rs:74-216): per-gene
// means and total variance (ddof 1 centred, 0 uncentred), a Gaussian sketch
// of n_components + 24 columns, power iterations (7 when fewer than a tenth
// of the spectrum is asked for, else 4) with an orthonormalisation after
// every product, then the eigendecomposition of (X^T Q)^T (X^T Q), singular
// values from its eigenvalues, the largest-loading sign fix (pca.rs:497-519)
// and scanpy's explained variance (S^2 / (n - 1) centred, the score columns'
// population variance uncentred).  Centring is a rank-one correction of
// every product, so the centred matrix is never formed.
//
// Device layout and order:
//   - X @ V: one warp per cell row, the row's entries in CSR order;
//     X^T @ U: one warp per gene over a stable CSC copy (made once by the
//     library's radix sort), entries in row order.  No atomics: the same
//     inputs give the same bits.
//   - Grams: each block sums its rows' products in f32 groups of 32 rows into
//     f64, the blocks' partial Grams then add up in block order.
//   - Orthonormalisation: shifted CholeskyQR, twice (the shift, 1e-7 of the
//     largest diagonal entry, keeps a numerically rank-deficient sketch
//     factorable, as the reference's eigenvalue floor does).  Any orthonormal
//     basis of the sketch gives the same components; the reference whitens
//     by the Gram's eigenvectors instead.
//   - The final small eigenproblem: cyclic Jacobi in f64 in one block.
// The Gaussian sketch comes from a counter-based generator (splitmix64 of
// the seed and the entry's index, Box-Muller in f64) instead of the
// reference's StdRng stream, so results agree with the reference's
// subspace, not its bits.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace scrust {

namespace {

constexpr int kOversampling = 24;
constexpr int kPcaMaxWidth = 128;  // sketch columns (n_components + 24) at most
constexpr double kShift = 1e-7;
constexpr int kJacobiSweeps = 60;
constexpr int kGramRows = 32;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Omega (g x w, row-major): standard normals by Box-Muller from two uniforms
// in (0, 1] drawn from the seed and the pair's index.
__global__ void pca_gaussian_kernel(int64_t count, uint64_t seed, float* __restrict__ omega) {
    const int64_t pair = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (2 * pair >= count) return;
    const uint64_t h1 = mix64(seed ^ mix64((uint64_t)pair * 2 + 1));
    const uint64_t h2 = mix64(seed ^ mix64((uint64_t)pair * 2 + 2));
    const double u1 = ((double)(h1 >> 11) + 1.0) * 1.1102230246251565e-16;  // (0, 1]
    const double u2 = (double)(h2 >> 11) * 1.1102230246251565e-16;          // [0, 1)
    const double r = sqrt(-2.0 * log(u1));
    const double t = 6.283185307179586 * u2;
    omega[2 * pair] = (float)(r * cos(t));
    if (2 * pair + 1 < count) omega[2 * pair + 1] = (float)(r * sin(t));
}

__global__ void pca_csc_keys_kernel(const uint32_t* __restrict__ indptr, const uint32_t* __restrict__ indices,
                                    const float* __restrict__ values, int64_t n, uint32_t* __restrict__ keys,
                                    unsigned long long* __restrict__ vals) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (uint32_t e = indptr[r], e1 = indptr[r + 1]; e < e1; ++e) {
        keys[e] = indices[e];
        vals[e] = ((unsigned long long)(uint32_t)r << 32) | __float_as_uint(values[e]);
    }
}

// start[c] = number of sorted keys below c, c in [0, g].
__global__ void pca_starts_kernel(const uint32_t* __restrict__ keys, int64_t nnz, int64_t g,
                                  uint32_t* __restrict__ start) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p > nnz) return;
    const int64_t lo = p == 0 ? 0 : (int64_t)keys[p - 1] + 1;
    const int64_t hi = p == nnz ? g : (int64_t)keys[p];
    for (int64_t c = lo; c <= hi && c <= g; ++c) start[c] = (uint32_t)p;
}

// Per gene: f64 sum and sum of squares over its entries in row order, the
// f32 mean, and the gene's variance term (pca.rs:227-255).
__global__ void pca_column_stats_kernel(const uint32_t* __restrict__ cstart, const unsigned long long* __restrict__ cv,
                                        int64_t g, int64_t n, double ddof, float* __restrict__ mean,
                                        double* __restrict__ var_term) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g) return;
    double s = 0.0, q = 0.0;
    for (uint32_t p = cstart[c], p1 = cstart[c + 1]; p < p1; ++p) {
        const double v = (double)__uint_as_float((uint32_t)cv[p]);
        s += v;
        q += v * v;
    }
    const double dn = (double)n;
    mean[c] = (float)(s / dn);
    var_term[c] = fmax(q - s * s / dn, 0.0) / (dn - ddof);
}

// Sum of `count` doubles in index order by one block (fixed tree per block of
// 256, blocks in order), into out[0].
__global__ void pca_sum_kernel(const double* __restrict__ x, int64_t count, double* __restrict__ out) {
    __shared__ double part[256];
    double total = 0.0;
    for (int64_t base = 0; base < count; base += 256) {
        const int64_t i = base + threadIdx.x;
        part[threadIdx.x] = i < count ? x[i] : 0.0;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) total += part[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = total;
}

// m[j] = sum_g mean[g] * B[g, j] (genes in order), one thread per column.
__global__ void pca_mean_row_kernel(const float* __restrict__ mean, const float* __restrict__ B, int64_t g, int w,
                                    float* __restrict__ m) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= w) return;
    double s = 0.0;
    for (int64_t c = 0; c < g; ++c) s += (double)mean[c] * (double)B[c * w + j];
    m[j] = (float)s;
}

// Column sums of U (n x w) in two fixed-order levels: per block of rows, then
// over the blocks.
constexpr int kColRows = 4096;
__global__ void pca_colsum_part_kernel(const float* __restrict__ U, int64_t n, int w, double* __restrict__ part) {
    const int64_t r0 = (int64_t)blockIdx.x * kColRows;
    const int64_t r1 = min(n, r0 + kColRows);
    for (int j = threadIdx.x; j < w; j += blockDim.x) {
        double s = 0.0;
        for (int64_t r = r0; r < r1; ++r) s += (double)U[r * w + j];
        part[(int64_t)blockIdx.x * w + j] = s;
    }
}
__global__ void pca_colsum_final_kernel(const double* __restrict__ part, int blocks, int w, float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= w) return;
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += part[(int64_t)b * w + j];
    out[j] = (float)s;
}

// Y (rows x w) = A (rows, sparse) @ B (cols x w) - ones * m (when m is given);
// one warp per sparse row, lanes over the w columns.  The rows are CSR rows
// of X (A = X) or CSC columns of X (A = X^T, entries as row << 32 | value).
template <bool PACKED>
__global__ void __launch_bounds__(256) pca_spmm_kernel(const uint32_t* __restrict__ start,
                                                       const uint32_t* __restrict__ idx,
                                                       const float* __restrict__ val,
                                                       const unsigned long long* __restrict__ packed, int64_t rows,
                                                       const float* __restrict__ B, int w,
                                                       const float* __restrict__ m, const float* __restrict__ scale,
                                                       const float* __restrict__ mvec, float* __restrict__ Y) {
    const int lane = threadIdx.x & 31;
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= rows) return;
    float acc[kPcaMaxWidth / 32];
#pragma unroll
    for (int t = 0; t < kPcaMaxWidth / 32; ++t) acc[t] = 0.f;
    for (uint32_t e = start[r], e1 = start[r + 1]; e < e1; ++e) {
        uint32_t c;
        float v;
        if (PACKED) {
            const unsigned long long pv = packed[e];
            c = (uint32_t)(pv >> 32);
            v = __uint_as_float((uint32_t)pv);
        } else {
            c = idx[e];
            v = val[e];
        }
        const float* brow = B + (int64_t)c * w;
#pragma unroll
        for (int t = 0; t < kPcaMaxWidth / 32; ++t) {
            const int j = t * 32 + lane;
            if (j < w) acc[t] = fmaf(v, brow[j], acc[t]);
        }
    }
#pragma unroll
    for (int t = 0; t < kPcaMaxWidth / 32; ++t) {
        const int j = t * 32 + lane;
        if (j < w) {
            float y = acc[t];
            // Centring: X_c B = X B - 1 (mean^T B); X_c^T U = X^T U - mean (1^T U).
            if (m) y -= m[j];
            if (scale) y -= scale[r] * mvec[j];
            Y[r * w + j] = y;
        }
    }
}

// Partial Grams: block b sums, over its rows, groups of kGramRows rows' f32
// products added into f64 accumulators; entries (i, j), i <= j, row by row
// of the upper triangle.  Shared memory: the f64 accumulators, each entry's
// (i, j), and the group of rows.
size_t gram_smem_bytes(int w) {
    const size_t entries = (size_t)w * (w + 1) / 2;
    return entries * sizeof(double) + entries * sizeof(uint32_t) + sizeof(float) * kGramRows * w;
}

__global__ void pca_gram_part_kernel(const float* __restrict__ Y, int64_t n, int w, int64_t rows_per_block,
                                     double* __restrict__ part) {
    extern __shared__ double gsm[];
    const int entries = w * (w + 1) / 2;
    double* acc = gsm;
    uint32_t* ij = reinterpret_cast<uint32_t*>(acc + entries);
    float* tile = reinterpret_cast<float*>(ij + entries);
    for (int t = threadIdx.x; t < entries; t += blockDim.x) {
        int i = 0, rem = t;
        while (i < w && rem >= w - i) {
            rem -= w - i;
            ++i;
        }
        ij[t] = ((uint32_t)i << 16) | (uint32_t)(i + rem);
        acc[t] = 0.0;
    }
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t r1 = min(n, r0 + rows_per_block);
    __syncthreads();
    for (int64_t base = r0; base < r1; base += kGramRows) {
        const int rows = (int)min((int64_t)kGramRows, r1 - base);
        for (int t = threadIdx.x; t < rows * w; t += blockDim.x) tile[t] = Y[base * w + t];
        __syncthreads();
        for (int t = threadIdx.x; t < entries; t += blockDim.x) {
            const int i = (int)(ij[t] >> 16), j = (int)(ij[t] & 0xffffu);
            float s = 0.f;
            for (int r = 0; r < rows; ++r) s = fmaf(tile[r * w + i], tile[r * w + j], s);
            acc[t] += (double)s;
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < entries; t += blockDim.x) part[(int64_t)blockIdx.x * entries + t] = acc[t];
}

__global__ void pca_gram_final_kernel(const double* __restrict__ part, int blocks, int w, double* __restrict__ G) {
    const int entries = w * (w + 1) / 2;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= entries) return;
    int i = 0, rem = t;
    while (i < w && rem >= w - i) {
        rem -= w - i;
        ++i;
    }
    const int j = i + rem;
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += part[(int64_t)b * entries + t];
    G[i * w + j] = s;
    G[j * w + i] = s;
}

// T = L^-T of the shifted Cholesky factor of G (w x w, f64), as f32; one block.
__global__ void pca_cholesky_kernel(const double* __restrict__ G, int w, double* __restrict__ L,
                                    float* __restrict__ T, int* __restrict__ err) {
    __shared__ double shift, diag;
    if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int i = 0; i < w; ++i) mx = fmax(mx, G[i * w + i]);
        shift = mx > 0.0 ? kShift * mx : 1.0;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < w * w; t += blockDim.x) L[t] = 0.0;
    __syncthreads();
    for (int j = 0; j < w; ++j) {
        if (threadIdx.x == 0) {
            double d = G[j * w + j] + shift;
            for (int k = 0; k < j; ++k) d -= L[j * w + k] * L[j * w + k];
            if (!(d > 0.0)) {
                d = shift;
                atomicExch(err, 1);
            }
            diag = sqrt(d);
            L[j * w + j] = diag;
        }
        __syncthreads();
        for (int i = j + 1 + threadIdx.x; i < w; i += blockDim.x) {
            double v = G[i * w + j];
            for (int k = 0; k < j; ++k) v -= L[i * w + k] * L[j * w + k];
            L[i * w + j] = v / diag;
        }
        __syncthreads();
    }
    // Column c of L^-1 by forward substitution.
    for (int c = threadIdx.x; c < w; c += blockDim.x) {
        double x[kPcaMaxWidth];
        for (int r = 0; r < w; ++r) {
            double v = r == c ? 1.0 : 0.0;
            for (int k = 0; k < r; ++k) v -= L[r * w + k] * x[k];
            x[r] = v / L[r * w + r];
        }
        // x is column c of L^-1, i.e. row c of L^-T (zero before c).
        for (int r = 0; r < w; ++r) T[c * w + r] = (float)x[r];
    }
}

// Y (n x w) <- Y @ T (w x w, upper triangular), one warp per row.
__global__ void __launch_bounds__(256) pca_rmul_kernel(float* __restrict__ Y, int64_t n, int w,
                                                       const float* __restrict__ T) {
    const int lane = threadIdx.x & 31;
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= n) return;
    float y[kPcaMaxWidth / 32], out[kPcaMaxWidth / 32];
#pragma unroll
    for (int t = 0; t < kPcaMaxWidth / 32; ++t) {
        const int j = t * 32 + lane;
        y[t] = j < w ? Y[r * w + j] : 0.f;
        out[t] = 0.f;
    }
    // y_i is held by lane i % 32 in slot i / 32: broadcast it slot by slot.
#pragma unroll
    for (int t = 0; t < kPcaMaxWidth / 32; ++t) {
        for (int l = 0; l < 32; ++l) {
            const int i = t * 32 + l;
            if (i >= w) break;
            const float yi = __shfl_sync(0xffffffffu, y[t], l);
#pragma unroll
            for (int u = 0; u < kPcaMaxWidth / 32; ++u) {
                const int j = u * 32 + lane;
                if (j < w) out[u] = fmaf(yi, T[i * w + j], out[u]);
            }
        }
    }
#pragma unroll
    for (int t = 0; t < kPcaMaxWidth / 32; ++t) {
        const int j = t * 32 + lane;
        if (j < w) Y[r * w + j] = out[t];
    }
}

// Eigenvalues (diagonal of A on return) and eigenvectors (columns of V) of a
// symmetric w x w f64 matrix by cyclic Jacobi rotations (pca.rs:388-447), one
// block: thread 0 forms each rotation, the block applies it.
__global__ void pca_jacobi_kernel(double* __restrict__ A, int w, double* __restrict__ V, int* __restrict__ err) {
    __shared__ double c_s, s_s, off_s, tol_s;
    __shared__ int skip_s;
    for (int t = threadIdx.x; t < w * w; t += blockDim.x) V[t] = (t / w == t % w) ? 1.0 : 0.0;
    if (threadIdx.x == 0) {
        double scale = 0.0;
        for (int t = 0; t < w * w; ++t) scale += A[t] * A[t];
        tol_s = 2.220446049250313e-16 * 2.220446049250313e-16 * fmax(scale, 2.2250738585072014e-308);
    }
    __syncthreads();
    for (int sweep = 0; sweep < kJacobiSweeps; ++sweep) {
        if (threadIdx.x == 0) {
            double off = 0.0;
            for (int r = 0; r < w; ++r)
                for (int c = 0; c < w; ++c)
                    if (r != c) off += A[r * w + c] * A[r * w + c];
            off_s = off;
        }
        __syncthreads();
        if (off_s <= tol_s) return;
        for (int p = 0; p < w; ++p)
            for (int q = p + 1; q < w; ++q) {
                if (threadIdx.x == 0) {
                    const double pivot = A[p * w + q];
                    skip_s = pivot == 0.0;
                    if (!skip_s) {
                        const double theta = (A[q * w + q] - A[p * w + p]) / (2.0 * pivot);
                        const double sgn = theta > 0.0 ? 1.0 : (theta < 0.0 ? -1.0 : 0.0);
                        const double tangent = sgn / fmax(fabs(theta) + sqrt(theta * theta + 1.0), 2.220446049250313e-16);
                        const double cs = 1.0 / sqrt(tangent * tangent + 1.0);
                        c_s = cs;
                        s_s = tangent * cs;
                    }
                }
                __syncthreads();
                if (!skip_s) {
                    const double cs = c_s, sn = s_s;
                    for (int k = threadIdx.x; k < w; k += blockDim.x) {
                        const double l = A[k * w + p], r = A[k * w + q];
                        A[k * w + p] = cs * l - sn * r;
                        A[k * w + q] = sn * l + cs * r;
                    }
                    __syncthreads();
                    for (int k = threadIdx.x; k < w; k += blockDim.x) {
                        const double l = A[p * w + k], r = A[q * w + k];
                        A[p * w + k] = cs * l - sn * r;
                        A[q * w + k] = sn * l + cs * r;
                    }
                    __syncthreads();
                    if (threadIdx.x == 0) {
                        A[p * w + q] = 0.0;
                        A[q * w + p] = 0.0;
                    }
                    for (int k = threadIdx.x; k < w; k += blockDim.x) {
                        const double l = V[k * w + p], r = V[k * w + q];
                        V[k * w + p] = cs * l - sn * r;
                        V[k * w + q] = sn * l + cs * r;
                    }
                }
                __syncthreads();
            }
    }
    if (threadIdx.x == 0) atomicExch(err, 2);
}

// From the eigenpairs of H = B B^T (w x w): the n_components largest, their
// singular values, and the two small matrices the outputs are built from:
// basis[:, j] = v_j * s_j (embedding = Q @ basis), scaled[:, j] = v_j / s_j
// (components^T = B^T @ scaled).  One thread.
__global__ void pca_select_kernel(const double* __restrict__ A, const double* __restrict__ V, int w, int nc,
                                  float* __restrict__ basis, float* __restrict__ scaled, double* __restrict__ sing) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int order[kPcaMaxWidth];
    for (int i = 0; i < w; ++i) order[i] = i;
    // Stable descending order of the eigenvalues (insertion sort).
    for (int i = 1; i < w; ++i) {
        const int v = order[i];
        int j = i;
        while (j > 0 && A[order[j - 1] * w + order[j - 1]] < A[v * w + v]) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = v;
    }
    for (int c = 0; c < nc; ++c) {
        const int idx = order[c];
        const double s = sqrt(fmax(A[idx * w + idx], 0.0));
        sing[c] = s;
        const double inv = s > 0.0 ? 1.0 / s : 0.0;
        for (int r = 0; r < w; ++r) {
            const double e = V[r * w + idx];
            basis[r * nc + c] = (float)(e * s);
            scaled[r * nc + c] = (float)(e * inv);
        }
    }
}

// Out (rows x nc) = A (rows x w) @ M (w x nc), one thread per output row.
__global__ void pca_small_mul_kernel(const float* __restrict__ A, int64_t rows, int w, const float* __restrict__ M,
                                     int nc, float* __restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    for (int c = 0; c < nc; ++c) {
        float s = 0.f;
        for (int i = 0; i < w; ++i) s = fmaf(A[r * w + i], M[i * nc + c], s);
        out[r * nc + c] = s;
    }
}

// components (nc x g) from components^T (g x nc); the sign fix of
// pca.rs:497-519: the first largest-magnitude loading of each component is
// made positive (and its embedding column flipped with it).
__global__ void pca_signs_kernel(const float* __restrict__ ct, int64_t g, int nc, int* __restrict__ flip) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    float extreme = 0.f;
    for (int64_t k = 0; k < g; ++k) {
        const float v = ct[k * nc + c];
        if (fabsf(v) > fabsf(extreme)) extreme = v;
    }
    flip[c] = extreme < 0.f ? 1 : 0;
}

__global__ void pca_finish_kernel(const float* __restrict__ ct, int64_t g, int nc, const int* __restrict__ flip,
                                  float* __restrict__ components, float* __restrict__ emb, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < g * nc) {
        const int64_t k = t / nc;
        const int c = (int)(t % nc);
        const float v = ct[t];
        components[(int64_t)c * g + k] = flip[c] ? -v : v;
    }
    if (t < n * nc) {
        const int c = (int)(t % nc);
        if (flip[c]) emb[t] = -emb[t];
    }
}

// Explained variance: S^2 / (n - 1) centred, else each score column's
// population variance (f64, rows in order); ratios over the total variance.
__global__ void pca_variance_kernel(const double* __restrict__ sing, const float* __restrict__ emb, int64_t n, int nc,
                                    int centred, const double* __restrict__ total, float* __restrict__ var,
                                    float* __restrict__ ratio) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    float v;
    if (centred) {
        v = (float)(sing[c] * sing[c] / (double)(n - 1));
    } else {
        double m = 0.0;
        for (int64_t r = 0; r < n; ++r) m += (double)emb[r * nc + c];
        m /= (double)n;
        double s = 0.0;
        for (int64_t r = 0; r < n; ++r) {
            const double d = (double)emb[r * nc + c] - m;
            s += d * d;
        }
        v = (float)(s / (double)n);
    }
    var[c] = v;
    ratio[c] = total[0] > 0.0 ? (float)((double)v / total[0]) : 0.f;
}

size_t al(size_t v) { return (v + 255) & ~(size_t)255; }

struct PcaWork {
    float *omega, *Y, *Z, *mvec, *colsum, *mean, *T, *basis, *scaled, *ct;
    double *var_term, *total, *gram_part, *G, *L, *V, *sing, *colpart;
    uint32_t *kA, *kB, *cstart;
    unsigned long long *vA, *vB;
    uint32_t *hist, *scan;
    size_t scan_elems;
    int* flip;
    const uint32_t* ckeys;
    const unsigned long long* cvals;
};

}  // namespace

int32_t pca_device_impl(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                        int64_t n, int64_t g, int64_t nnz, int nc, bool zero_center, uint64_t seed, float* emb,
                        float* components, float* variance, float* ratio, scrust_status* st) {
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    const int64_t maxc = std::min(n, g);
    const int w = (int)std::min<int64_t>(nc + kOversampling, maxc);
    const int entries = w * (w + 1) / 2;
    // A Gram over `rows` rows runs ceil(rows / max(32, ceil(rows / 4S))) <= 4S
    // blocks (S = SMs).
    const int gram_blocks = 4 * ctx->sm_count;
    const int col_blocks = (int)((n + kColRows - 1) / kColRows);
    const int nb = radix_blocks(std::max<int64_t>(nnz, 1));
    PcaWork wk;
    wk.scan_elems = scan_scratch_elems((int64_t)256 * nb);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t r = off;
        off = al(off + bytes);
        return r;
    };
    const size_t o_om = take(4 * (size_t)g * w), o_y = take(4 * (size_t)n * w), o_z = take(4 * (size_t)g * w),
                 o_mv = take(4 * (size_t)w), o_cs = take(4 * (size_t)w), o_mean = take(4 * (size_t)g),
                 o_t = take(4 * (size_t)w * w), o_basis = take(4 * (size_t)w * nc), o_sc = take(4 * (size_t)w * nc),
                 o_ct = take(4 * (size_t)g * nc), o_vt = take(8 * (size_t)g), o_tot = take(8),
                 o_gp = take(8 * (size_t)gram_blocks * entries), o_g = take(8 * (size_t)w * w),
                 o_l = take(8 * (size_t)w * w), o_v = take(8 * (size_t)w * w), o_sing = take(8 * (size_t)nc),
                 o_cp = take(8 * (size_t)col_blocks * w), o_ka = take(4 * (size_t)nnz), o_kb = take(4 * (size_t)nnz),
                 o_cst = take(4 * (size_t)(g + 1)), o_va = take(8 * (size_t)nnz), o_vb = take(8 * (size_t)nnz),
                 o_hist = take(4 * ((size_t)256 * nb + 16)), o_scan = take(4 * wk.scan_elems), o_flip = take(4 * ((size_t)nc + 1));
    char* base = (char*)ws_get(ctx, SLOT_PCA, off, &e);
    if (!base) return cuda_fail(st, e, "pca: workspace");
    wk.omega = (float*)(base + o_om);
    wk.Y = (float*)(base + o_y);
    wk.Z = (float*)(base + o_z);
    wk.mvec = (float*)(base + o_mv);
    wk.colsum = (float*)(base + o_cs);
    wk.mean = (float*)(base + o_mean);
    wk.T = (float*)(base + o_t);
    wk.basis = (float*)(base + o_basis);
    wk.scaled = (float*)(base + o_sc);
    wk.ct = (float*)(base + o_ct);
    wk.var_term = (double*)(base + o_vt);
    wk.total = (double*)(base + o_tot);
    wk.gram_part = (double*)(base + o_gp);
    wk.G = (double*)(base + o_g);
    wk.L = (double*)(base + o_l);
    wk.V = (double*)(base + o_v);
    wk.sing = (double*)(base + o_sing);
    wk.colpart = (double*)(base + o_cp);
    wk.kA = (uint32_t*)(base + o_ka);
    wk.kB = (uint32_t*)(base + o_kb);
    wk.cstart = (uint32_t*)(base + o_cst);
    wk.vA = (unsigned long long*)(base + o_va);
    wk.vB = (unsigned long long*)(base + o_vb);
    wk.hist = (uint32_t*)(base + o_hist);
    wk.scan = (uint32_t*)(base + o_scan);
    wk.flip = (int*)(base + o_flip);
    int* err = wk.flip + nc;  // after the nc sign flags
    if ((e = cudaMemsetAsync(err, 0, sizeof(int), s)) != cudaSuccess) return cuda_fail(st, e, "pca: memset");
    uint64_t launches = 0;
    // The CSC copy: entries sorted by gene, rows ascending within a gene.
    pca_csc_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(indptr, indices, values, n, wk.kA, wk.vA);
    int bits = 1;
    while (((int64_t)1 << bits) <= g) bits++;
    uint32_t* ckeys = nullptr;
    unsigned long long* cvals = nullptr;
    if ((e = radix_sort_pairs(ctx, wk.kA, wk.vA, wk.kB, wk.vB, nnz, bits, wk.hist, wk.scan, wk.scan_elems, &ckeys,
                              &cvals)) != cudaSuccess)
        return cuda_fail(st, e, "pca: transpose");
    pca_starts_kernel<<<(unsigned)((nnz + 1 + 255) / 256), 256, 0, s>>>(ckeys, nnz, g, wk.cstart);
    pca_column_stats_kernel<<<(unsigned)((g + 255) / 256), 256, 0, s>>>(wk.cstart, cvals, g, n,
                                                                        zero_center ? 1.0 : 0.0, wk.mean, wk.var_term);
    pca_sum_kernel<<<1, 256, 0, s>>>(wk.var_term, g, wk.total);
    launches += 5;
    const unsigned cell_warps = (unsigned)((n * 32 + 255) / 256), gene_warps = (unsigned)((g * 32 + 255) / 256);
    const float* mean = zero_center ? wk.mean : nullptr;
    // X_c @ B into Y
    auto times = [&](const float* B, float* Y) -> cudaError_t {
        if (mean) {
            pca_mean_row_kernel<<<(w + 127) / 128, 128, 0, s>>>(wk.mean, B, g, w, wk.mvec);
            launches += 1;
        }
        pca_spmm_kernel<false><<<cell_warps, 256, 0, s>>>(indptr, indices, values, nullptr, n, B, w,
                                                         mean ? wk.mvec : nullptr, nullptr, nullptr, Y);
        launches += 1;
        return cudaGetLastError();
    };
    // X_c^T @ U into Z
    auto transpose_times = [&](const float* U, float* Z) -> cudaError_t {
        if (mean) {
            pca_colsum_part_kernel<<<col_blocks, 128, 0, s>>>(U, n, w, wk.colpart);
            pca_colsum_final_kernel<<<(w + 127) / 128, 128, 0, s>>>(wk.colpart, col_blocks, w, wk.colsum);
            launches += 2;
        }
        pca_spmm_kernel<true><<<gene_warps, 256, 0, s>>>(wk.cstart, nullptr, nullptr, cvals, g, U, w, nullptr,
                                                        mean ? wk.mean : nullptr, mean ? wk.colsum : nullptr, Z);
        launches += 1;
        return cudaGetLastError();
    };
    auto gram = [&](const float* Y, int64_t rows) -> cudaError_t {
        const int64_t rpb = std::max<int64_t>(kGramRows, (rows + 4 * ctx->sm_count - 1) / (4 * ctx->sm_count));
        const int blocks = (int)((rows + rpb - 1) / rpb);
        const size_t smem = gram_smem_bytes(w);
        cudaError_t e3 = set_smem_limit(ctx, (const void*)pca_gram_part_kernel, (int)smem);
        if (e3 != cudaSuccess) return e3;
        pca_gram_part_kernel<<<blocks, 512, smem, s>>>(Y, rows, w, rpb, wk.gram_part);
        pca_gram_final_kernel<<<(entries + 255) / 256, 256, 0, s>>>(wk.gram_part, blocks, w, wk.G);
        launches += 2;
        return cudaGetLastError();
    };
    auto orthonormalize = [&](float* Y, int64_t rows) -> cudaError_t {
        for (int pass = 0; pass < 2; ++pass) {
            cudaError_t e2 = gram(Y, rows);
            if (e2 != cudaSuccess) return e2;
            pca_cholesky_kernel<<<1, 128, 0, s>>>(wk.G, w, wk.L, wk.T, err);
            pca_rmul_kernel<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, s>>>(Y, rows, w, wk.T);
            launches += 2;
            if ((e2 = cudaGetLastError()) != cudaSuccess) return e2;
        }
        return cudaSuccess;
    };
    pca_gaussian_kernel<<<(unsigned)(((g * w + 1) / 2 + 255) / 256), 256, 0, s>>>(g * w, seed, wk.omega);
    launches += 1;
    if ((e = times(wk.omega, wk.Y)) != cudaSuccess || (e = orthonormalize(wk.Y, n)) != cudaSuccess)
        return cuda_fail(st, e, "pca: sketch");
    const int power = (double)nc < 0.1 * (double)maxc ? 7 : 4;
    for (int it = 0; it < power; ++it) {
        if ((e = transpose_times(wk.Y, wk.Z)) != cudaSuccess || (e = orthonormalize(wk.Z, g)) != cudaSuccess ||
            (e = times(wk.Z, wk.Y)) != cudaSuccess || (e = orthonormalize(wk.Y, n)) != cudaSuccess)
            return cuda_fail(st, e, "pca: power iteration");
    }
    // B^T = X_c^T Q (g x w), its Gram, the eigenpairs, the outputs.
    if ((e = transpose_times(wk.Y, wk.Z)) != cudaSuccess || (e = gram(wk.Z, g)) != cudaSuccess)
        return cuda_fail(st, e, "pca: projection");
    pca_jacobi_kernel<<<1, 128, 0, s>>>(wk.G, w, wk.V, err);
    pca_select_kernel<<<1, 32, 0, s>>>(wk.G, wk.V, w, nc, wk.basis, wk.scaled, wk.sing);
    pca_small_mul_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(wk.Y, n, w, wk.basis, nc, emb);
    pca_small_mul_kernel<<<(unsigned)((g + 127) / 128), 128, 0, s>>>(wk.Z, g, w, wk.scaled, nc, wk.ct);
    pca_signs_kernel<<<(nc + 63) / 64, 64, 0, s>>>(wk.ct, g, nc, wk.flip);
    const int64_t span = std::max(g, n) * nc;
    pca_finish_kernel<<<(unsigned)((span + 255) / 256), 256, 0, s>>>(wk.ct, g, nc, wk.flip, components, emb, n);
    pca_variance_kernel<<<(nc + 63) / 64, 64, 0, s>>>(wk.sing, emb, n, nc, zero_center ? 1 : 0, wk.total, variance,
                                                     ratio);
    launches += 7;
    ctx->launches += launches;
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(st, e, "pca");
    int herr = 0;
    if ((e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(st, e, "pca: synchronise");
    if (herr == 2)
        return fail(st, SCRUST_NOT_CONVERGED, "Jacobi eigenvalue iteration did not converge in %d sweeps", kJacobiSweeps);
    return ok(st);
}

}  // namespace scrust

using namespace scrust;

namespace {

int32_t check_pca(uint64_t n, uint64_t g, uint32_t nc, scrust_status* st) {
    const uint64_t maxc = std::min(n, g);
    if (nc == 0) return fail(st, SCRUST_INVALID_PARAMETER, "n_components must be at least 1, got 0");
    if (nc > maxc)
        return fail(st, SCRUST_INVALID_PARAMETER, "n_components must be at most min(n_cells, n_genes), got %u", nc);
    if (n < 2) return fail(st, SCRUST_INVALID_PARAMETER, "n_cells must be at least 2, got %llu", (unsigned long long)n);
    if (nc + kOversampling > (uint32_t)kPcaMaxWidth && nc > (uint32_t)(kPcaMaxWidth - kOversampling))
        return fail(st, SCRUST_INVALID_PARAMETER, "n_components must be at most %d, got %u", kPcaMaxWidth - kOversampling,
                    nc);
    if (n >= 0xffffff00ull || g >= 0xffffff00ull) return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 cells and genes");
    return SCRUST_OK;
}

}  // namespace

extern "C" {

int32_t scrust_cuda_pca_device(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices,
                               const float* values, uint64_t n_cells, uint64_t n_genes, uint64_t nnz,
                               uint32_t n_components, int32_t zero_center, uint64_t seed, float* out_embedding,
                               float* out_components, float* out_variance, float* out_variance_ratio,
                               scrust_status* st) {
    int32_t rc = check_pca(n_cells, n_genes, n_components, st);
    if (rc) return rc;
    if (nnz >= 0xffffff00ull) return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 stored entries");
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    if (!indptr || (nnz && (!indices || !values)) || !out_embedding || !out_components || !out_variance ||
        !out_variance_ratio)
        return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    return pca_device_impl(ctx, indptr, indices, values, (int64_t)n_cells, (int64_t)n_genes, (int64_t)nnz,
                           (int)n_components, zero_center != 0, seed, out_embedding, out_components, out_variance,
                           out_variance_ratio, st);
}

int32_t scrust_cuda_pca(scrust_context* ctx, const uint32_t* indptr, const uint32_t* indices, const float* values,
                        uint64_t n_cells, uint64_t n_genes, uint32_t n_components, int32_t zero_center, uint64_t seed,
                        float* out_embedding, float* out_components, float* out_variance, float* out_variance_ratio,
                        scrust_status* st) {
    int32_t rc = check_pca(n_cells, n_genes, n_components, st);
    if (rc) return rc;
    if (!indptr || !out_embedding || !out_components || !out_variance || !out_variance_ratio)
        return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    const uint64_t nnz = indptr[n_cells];
    if (nnz && (!indices || !values)) return fail(st, SCRUST_SHAPE, "expected non-null pointers");
    // CsrMatrix::new's structural checks (crates/scrust-core/src/sparse.rs:18-90).
    if (indptr[0] != 0) return fail(st, SCRUST_SHAPE, "expected indptr to start at 0");
    for (uint64_t r = 0; r < n_cells; ++r)
        if (indptr[r + 1] < indptr[r]) return fail(st, SCRUST_SHAPE, "expected a non-decreasing indptr");
    for (uint64_t i = 0; i < nnz; ++i)
        if (indices[i] >= n_genes)
            return fail(st, SCRUST_SHAPE, "expected column indices below %llu", (unsigned long long)n_genes);
    if (nnz >= 0xffffff00ull) return fail(st, SCRUST_SHAPE, "expected fewer than 2^32 stored entries");
    if (!ctx) return fail(st, SCRUST_NO_GPU, "no CUDA context (no usable GPU)");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e;
    const uint32_t nc = n_components;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t r = off;
        off = (off + bytes + 255) & ~(size_t)255;
        return r;
    };
    const size_t o_ip = take(4 * (n_cells + 1)), o_ix = take(4 * std::max<uint64_t>(nnz, 1)),
                 o_vl = take(4 * std::max<uint64_t>(nnz, 1)), o_emb = take(4 * n_cells * nc),
                 o_cmp = take(4 * n_genes * nc), o_var = take(4 * nc), o_rat = take(4 * nc);
    char* buf = (char*)ws_get(ctx, SLOT_HOST_IN, off, &e);
    if (!buf) return cuda_fail(st, e, "workspace");
    if ((e = cudaMemcpyAsync(buf + o_ip, indptr, 4 * (n_cells + 1), cudaMemcpyHostToDevice, ctx->stream)) !=
            cudaSuccess ||
        (nnz && (e = cudaMemcpyAsync(buf + o_ix, indices, 4 * nnz, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess) ||
        (nnz && (e = cudaMemcpyAsync(buf + o_vl, values, 4 * nnz, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess))
        return cuda_fail(st, e, "upload");
    if ((rc = pca_device_impl(ctx, (const uint32_t*)(buf + o_ip), (const uint32_t*)(buf + o_ix),
                              (const float*)(buf + o_vl), (int64_t)n_cells, (int64_t)n_genes, (int64_t)nnz, (int)nc,
                              zero_center != 0, seed, (float*)(buf + o_emb), (float*)(buf + o_cmp),
                              (float*)(buf + o_var), (float*)(buf + o_rat), st)))
        return rc;
    if ((e = cudaMemcpyAsync(out_embedding, buf + o_emb, 4 * n_cells * nc, cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out_components, buf + o_cmp, 4 * n_genes * nc, cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out_variance, buf + o_var, 4 * nc, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_variance_ratio, buf + o_rat, 4 * nc, cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess)
        return cuda_fail(st, e, "download");
    return collect_device_errors(ctx, st);
}

}  // extern "C"
