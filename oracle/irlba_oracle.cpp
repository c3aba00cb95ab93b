// ORACLE — test infrastructure only. Nothing in the product path links, loads or
// calls this file; it gives the CPU results that the GPU engine is compared with,
// and the CPU baseline that bench.py times beside it.
//
// A plain-C++ restatement of CppIrlba's augmented implicitly restarted Lanczos
// bidiagonalization (IRLBA) on column-major double arrays. Every function cites
// the reference file:line it follows (paths relative to the CppIrlba project).
//
// The reference cannot be built here: it needs Eigen 5.0.0, aarand, subpar and
// sanisizer, none of which is available offline. Three pieces therefore differ
// from the reference by construction and are restated from published methods:
//   * Eigen::JacobiSVD (compute.hpp:27-28) of the square B in the restart loop
//     (compute.hpp:225) -> a restatement of Eigen's two-sided Jacobi SVD for real
//     square input (the published Kogbetliantz / Brent-Luk-Van Loan scheme as
//     Eigen 5.0.0 orders and terminates it; jacobi_svd_square below), so the
//     restart SVD stops where the reference's does; for the exact SVD of a
//     rectangular matrix (compute.hpp:30-46) -> one-sided Jacobi SVD (Hestenes
//     1958; Demmel & Veselic 1992), columns sorted by decreasing singular value,
//     with an orthonormal completion of U for zero singular values.
//   * aarand::standard_normal (utils.hpp:27,34) -> Box-Muller on two 53-bit uniforms
//     drawn from std::mt19937_64 (u = (x >> 11) * 2^-53, mapped to (0, 1]).
//   * subpar::parallelize_simple (parallel.hpp:36) -> OpenMP parallel region with
//     one task per thread.
// Dense GEMV/GEMM follow Eigen's mathematical definitions; summation order differs.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>
#include <omp.h>

namespace oracle {

typedef int64_t Index;

// ---------------------------------------------------------------------------
// Options (Options.hpp:19-83). Field names and defaults as the reference.
// ---------------------------------------------------------------------------
struct Options {
    double invariant_subspace_tolerance = -1;
    double convergence_tolerance = 1e-5;
    double singular_value_ratio_tolerance = -1;
    int extra_work = 7;
    int max_iterations = 1000;
    bool exact_for_small_matrix = true;
    bool exact_for_large_number = true;
    bool cap_number = false;
    uint64_t seed = std::mt19937_64::default_seed;
    const double* initial = nullptr;  // std::optional<EigenVector_> in the reference
    Index initial_size = 0;
};

// ---------------------------------------------------------------------------
// Random normals (utils.hpp:16-53). Box-Muller pairs; odd lengths use the first
// value of one extra pair (utils.hpp:31-35).
// ---------------------------------------------------------------------------
inline double uniform01(std::mt19937_64& eng) {
    return (static_cast<double>(eng() >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

inline std::pair<double, double> standard_normal(std::mt19937_64& eng) {
    const double u1 = uniform01(eng);
    const double u2 = uniform01(eng);
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double theta = 6.283185307179586476925286766559 * u2;
    return {r * std::cos(theta), r * std::sin(theta)};
}

void fill_with_random_normals(double* vec, Index n, std::mt19937_64& eng) {
    Index total = n;
    const bool odd = total % 2;
    if (odd) --total;
    for (Index i = 0; i < total; i += 2) {
        auto p = standard_normal(eng);
        vec[i] = p.first;
        vec[i + 1] = p.second;
    }
    if (odd) {
        auto p = standard_normal(eng);
        vec[total] = p.first;
    }
}

// ---------------------------------------------------------------------------
// Matrix plug-in surface (Matrix/interface.hpp:141-223), collapsed to one class
// per wrapper with multiply / adjoint_multiply / realize.
// ---------------------------------------------------------------------------
struct Matrix {
    virtual ~Matrix() {}
    virtual Index rows() const = 0;
    virtual Index cols() const = 0;
    // out = A * right (Workspace::multiply, interface.hpp:49). out fully overwritten.
    virtual void multiply(const double* right, double* out) const = 0;
    // out = A^T * right (AdjointWorkspace::multiply, interface.hpp:87).
    virtual void adjoint_multiply(const double* right, double* out) const = 0;
    // Column-major realization (RealizeWorkspace::realize_copy, interface.hpp:125-130).
    virtual void realize(double* buffer) const = 0;
};

// SimpleMatrix over a dense matrix (Matrix/simple.hpp:27-73). `ld` is the
// leading dimension; row_major selects the storage order of the input.
struct DenseMatrix : public Matrix {
    Index nr, nc, ld;
    const double* data;
    bool row_major;
    DenseMatrix(Index r, Index c, const double* d, Index lead, bool rm) : nr(r), nc(c), ld(lead), data(d), row_major(rm) {}
    Index rows() const override { return nr; }
    Index cols() const override { return nc; }
    double at(Index r, Index c) const { return row_major ? data[r * ld + c] : data[c * ld + r]; }
    void multiply(const double* x, double* out) const override {  // simple.hpp:42-44
        for (Index r = 0; r < nr; ++r) out[r] = 0;
        for (Index c = 0; c < nc; ++c) {
            const double xc = x[c];
            for (Index r = 0; r < nr; ++r) out[r] += at(r, c) * xc;
        }
    }
    void adjoint_multiply(const double* y, double* out) const override {  // simple.hpp:70-72
        for (Index c = 0; c < nc; ++c) {
            double s = 0;
            for (Index r = 0; r < nr; ++r) s += at(r, c) * y[r];
            out[c] = s;
        }
    }
    void realize(double* buf) const override {
        for (Index c = 0; c < nc; ++c)
            for (Index r = 0; r < nr; ++r) buf[c * nr + r] = at(r, c);
    }
};

// ParallelSparseMatrix (Matrix/sparse.hpp:29-589): compressed sparse row/column
// with nnz-balanced thread partitions computed at construction.
struct SparseMatrix : public Matrix {
    Index primary_dim, secondary_dim;
    int num_threads;
    const double* values;      // FP64 values, or
    const float* values32;     // FP32 values (the reference's ValueArray may hold float)
    const int32_t* indices;
    const int64_t* ptrs;
    bool column_major;
    std::vector<Index> primary_boundaries, secondary_boundaries;
    std::vector<std::vector<int64_t>> secondary_nonzero_boundaries;

    // ParallelSparseMatrixCore constructor, sparse.hpp:35-115.
    SparseMatrix(Index nrow, Index ncol, const double* x, const int32_t* i, const int64_t* p, bool cm, int nt,
                 const float* x32 = nullptr)
        : primary_dim(cm ? ncol : nrow), secondary_dim(cm ? nrow : ncol), num_threads(nt),
          values(x), values32(x32), indices(i), ptrs(p), column_major(cm) {
        if (num_threads > 1) {
            const int64_t total = ptrs[primary_dim];
            const int64_t per_thread_floor = total / num_threads;
            const int per_thread_extra = static_cast<int>(total % num_threads);

            // sparse.hpp:62-74: primary boundaries balanced by nnz.
            primary_boundaries.assign(num_threads + 1, 0);
            {
                Index counter = 0;
                int64_t sofar = 0;
                for (int t = 0; t < num_threads; ++t) {
                    sofar += per_thread_floor + (t < per_thread_extra);
                    while (counter < primary_dim && ptrs[counter + 1] <= sofar) ++counter;
                    primary_boundaries[t + 1] = counter;
                }
            }

            // sparse.hpp:77-94: secondary boundaries balanced by nnz.
            std::vector<int64_t> secondary_nonzeros(secondary_dim, 0);
            for (int64_t s = 0; s < total; ++s) ++secondary_nonzeros[indices[s]];
            secondary_boundaries.assign(num_threads + 1, 0);
            {
                Index counter = 0;
                int64_t sofar = 0, cum = 0;
                for (int t = 0; t < num_threads; ++t) {
                    sofar += per_thread_floor + (t < per_thread_extra);
                    while (counter < secondary_dim && cum <= sofar) {
                        cum += secondary_nonzeros[counter];
                        ++counter;
                    }
                    secondary_boundaries[t + 1] = counter;
                }
            }

            // sparse.hpp:96-112: per-primary split points of each thread's secondary range.
            secondary_nonzero_boundaries.assign(num_threads + 1, std::vector<int64_t>(primary_dim));
            for (Index c = 0; c < primary_dim; ++c) {
                const int64_t start = ptrs[c], end = ptrs[c + 1];
                secondary_nonzero_boundaries[0][c] = start;
                int64_t s = start;
                for (int t = 0; t < num_threads; ++t) {
                    const Index limit = secondary_boundaries[t + 1];
                    while (s < end && static_cast<Index>(indices[s]) < limit) ++s;
                    secondary_nonzero_boundaries[t + 1][c] = s;
                }
            }
        }
    }

    Index rows() const override { return column_major ? secondary_dim : primary_dim; }
    Index cols() const override { return column_major ? primary_dim : secondary_dim; }

    // Calls f with the stored value array (double or float); products promote to double.
    template <class F>
    void with_values(F f) const {
        if (values32) f(values32);
        else f(values);
    }
    double value(int64_t s) const { return values32 ? static_cast<double>(values32[s]) : values[s]; }

    // indirect_multiply, sparse.hpp:185-235 (scatter along the secondary dimension).
    void indirect_multiply(const double* rhs, double* out) const {
        with_values([&](const auto* vals) { indirect_impl(vals, rhs, out); });
    }
    template <class V>
    void indirect_impl(const V* vals, const double* rhs, double* out) const {
        if (num_threads == 1) {
            std::fill(out, out + secondary_dim, 0.0);
            for (Index c = 0; c < primary_dim; ++c) {
                const double val = rhs[c];
                for (int64_t s = ptrs[c]; s < ptrs[c + 1]; ++s) out[indices[s]] += static_cast<double>(vals[s]) * val;
            }
            return;
        }
#pragma omp parallel num_threads(num_threads)
        {
            const int t = omp_get_thread_num();
            const Index sstart = secondary_boundaries[t], send = secondary_boundaries[t + 1];
            // Private buffer per thread (sparse.hpp:205-216); thread 0 writes in place.
            std::vector<double> buffer;
            double* optr;
            if (t != 0) {
                buffer.assign(send - sstart, 0.0);
                optr = buffer.data();
            } else {
                optr = out + sstart;
                std::fill(optr, optr + (send - sstart), 0.0);
            }
            const auto& nz_starts = secondary_nonzero_boundaries[t];
            const auto& nz_ends = secondary_nonzero_boundaries[t + 1];
            for (Index c = 0; c < primary_dim; ++c) {
                const double val = rhs[c];
                for (int64_t s = nz_starts[c]; s < nz_ends[c]; ++s)
                    optr[indices[s] - sstart] += static_cast<double>(vals[s]) * val;
            }
            if (t != 0) std::copy(optr, optr + (send - sstart), out + sstart);
        }
    }

    // column_dot_product, sparse.hpp:259-267.
    template <class V>
    double primary_dot(const V* vals, Index p, const double* rhs) const {
        double dot = 0;
        for (int64_t s = ptrs[p]; s < ptrs[p + 1]; ++s) dot += static_cast<double>(vals[s]) * rhs[indices[s]];
        return dot;
    }

    // direct_multiply, sparse.hpp:238-256 (gather along the primary dimension).
    void direct_multiply(const double* rhs, double* out) const {
        with_values([&](const auto* vals) {
            if (num_threads == 1) {
                for (Index c = 0; c < primary_dim; ++c) out[c] = primary_dot(vals, c, rhs);
                return;
            }
#pragma omp parallel num_threads(num_threads)
            {
                const int t = omp_get_thread_num();
                for (Index c = primary_boundaries[t]; c < primary_boundaries[t + 1]; ++c)
                    out[c] = primary_dot(vals, c, rhs);
            }
        });
    }

    // Layout dispatch, sparse.hpp:305-311 and :346-352.
    void multiply(const double* x, double* out) const override {
        if (column_major) indirect_multiply(x, out); else direct_multiply(x, out);
    }
    void adjoint_multiply(const double* y, double* out) const override {
        if (column_major) direct_multiply(y, out); else indirect_multiply(y, out);
    }
    // ParallelSparseRealizeWorkspace::realize, sparse.hpp:382-409.
    void realize(double* buf) const override {
        const Index nr = rows(), nc = cols();
        std::fill(buf, buf + nr * nc, 0.0);
        for (Index p = 0; p < primary_dim; ++p) {
            for (int64_t s = ptrs[p]; s < ptrs[p + 1]; ++s) {
                if (column_major) buf[p * nr + indices[s]] = value(s);
                else buf[static_cast<Index>(indices[s]) * nr + p] = value(s);
            }
        }
    }
};

// CenteredMatrix (Matrix/centered.hpp:27-204): column centring as a rank-1 correction.
struct CenteredMatrix : public Matrix {
    const Matrix* inner;
    const double* center;  // length cols()
    CenteredMatrix(const Matrix* m, const double* c) : inner(m), center(c) {}
    Index rows() const override { return inner->rows(); }
    Index cols() const override { return inner->cols(); }
    void multiply(const double* x, double* out) const override {  // centered.hpp:46-52
        inner->multiply(x, out);
        double beta = 0;
        for (Index c = 0; c < cols(); ++c) beta += x[c] * center[c];
        for (Index r = 0; r < rows(); ++r) out[r] -= beta;
    }
    void adjoint_multiply(const double* y, double* out) const override {  // centered.hpp:83-87
        inner->adjoint_multiply(y, out);
        double beta = 0;
        for (Index r = 0; r < rows(); ++r) beta += y[r];
        for (Index c = 0; c < cols(); ++c) out[c] -= beta * center[c];
    }
    void realize(double* buf) const override {  // centered.hpp:118-122
        inner->realize(buf);
        const Index nr = rows();
        for (Index c = 0; c < cols(); ++c)
            for (Index r = 0; r < nr; ++r) buf[c * nr + r] -= center[c];
    }
};

// ScaledMatrix (Matrix/scaled.hpp:235-476): row/column multiply or divide.
struct ScaledMatrix : public Matrix {
    const Matrix* inner;
    const double* scale;
    bool column, divide;
    ScaledMatrix(const Matrix* m, const double* s, bool col, bool div) : inner(m), scale(s), column(col), divide(div) {}
    Index rows() const override { return inner->rows(); }
    Index cols() const override { return inner->cols(); }
    void apply(const double* in, double* out, Index n) const {
        if (divide) for (Index i = 0; i < n; ++i) out[i] = in[i] / scale[i];
        else for (Index i = 0; i < n; ++i) out[i] = in[i] * scale[i];
    }
    void multiply(const double* x, double* out) const override {  // scaled.hpp:52-69
        if (column) {
            std::vector<double> buf(cols());
            apply(x, buf.data(), cols());
            inner->multiply(buf.data(), out);
        } else {
            inner->multiply(x, out);
            apply(out, out, rows());
        }
    }
    void adjoint_multiply(const double* y, double* out) const override {  // scaled.hpp:106-123
        if (column) {
            inner->adjoint_multiply(y, out);
            apply(out, out, cols());
        } else {
            std::vector<double> buf(rows());
            apply(y, buf.data(), rows());
            inner->adjoint_multiply(buf.data(), out);
        }
    }
    void realize(double* buf) const override {  // scaled.hpp:158-177
        inner->realize(buf);
        const Index nr = rows(), nc = cols();
        for (Index c = 0; c < nc; ++c)
            for (Index r = 0; r < nr; ++r) {
                const double s = column ? scale[c] : scale[r];
                if (divide) buf[c * nr + r] /= s; else buf[c * nr + r] *= s;
            }
    }
};

// ---------------------------------------------------------------------------
// Dense helpers on column-major arrays (the Eigen calls of the reference).
// ---------------------------------------------------------------------------
struct Dense {
    Index nr = 0, nc = 0;
    std::vector<double> v;
    Dense() {}
    Dense(Index r, Index c) : nr(r), nc(c), v(static_cast<size_t>(r * c), 0.0) {}
    double* col(Index c) { return v.data() + c * nr; }
    const double* col(Index c) const { return v.data() + c * nr; }
    double& operator()(Index r, Index c) { return v[c * nr + r]; }
    double operator()(Index r, Index c) const { return v[c * nr + r]; }
};

inline double dot(const double* a, const double* b, Index n) {
    double s = 0;
    for (Index i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}
inline double norm(const double* a, Index n) { return std::sqrt(dot(a, a, n)); }

// Threads used by the oracle's dense loops (CGS and rotations); 1 by default.
// With more threads these loops run in parallel over fixed row blocks, so the
// results do not depend on the thread count. (The reference's Eigen GEMV of
// orthogonalize_vector is single-threaded; only its GEMMs use Eigen's threads.)
static int g_dense_threads = 1;

// Rows per block of the dense loops: the block of Q stays in L1/L2 while its
// columns are combined.
constexpr Index kDenseRowBlock = 512;

// orthogonalize_vector, lanczos.hpp:17-21: tmp = Q[:, :ncols]^T v; v -= Q[:, :ncols] tmp.
// The dot products sum each row block in row order, then the blocks in block
// order; the update forms sum_j Q[r, j] tmp[j] in column order and subtracts it.
void orthogonalize_vector(const Dense& Q, double* vec, Index ncols, double* tmp) {
    const Index L = Q.nr;
    const int nt = g_dense_threads;
    const Index nblocks = (L + kDenseRowBlock - 1) / kDenseRowBlock;
    std::vector<double> part(static_cast<size_t>(nblocks * ncols));
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1 && L > 4096)
    for (Index b = 0; b < nblocks; ++b) {
        const Index r0 = b * kDenseRowBlock, r1 = std::min(L, r0 + kDenseRowBlock);
        for (Index j = 0; j < ncols; ++j) {
            const double* q = Q.v.data() + j * L;
            double s = 0;
            for (Index r = r0; r < r1; ++r) s += q[r] * vec[r];
            part[b * ncols + j] = s;
        }
    }
    for (Index j = 0; j < ncols; ++j) {
        double s = 0;
        for (Index b = 0; b < nblocks; ++b) s += part[b * ncols + j];
        tmp[j] = s;
    }
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1 && L > 4096)
    for (Index b = 0; b < nblocks; ++b) {
        const Index r0 = b * kDenseRowBlock, r1 = std::min(L, r0 + kDenseRowBlock), nr = r1 - r0;
        double acc[kDenseRowBlock];
        for (Index i = 0; i < nr; ++i) acc[i] = 0;
        for (Index j = 0; j < ncols; ++j) {
            const double tj = tmp[j];
            const double* q = Q.v.data() + j * L + r0;
            for (Index i = 0; i < nr; ++i) acc[i] += q[i] * tj;
        }
        for (Index i = 0; i < nr; ++i) vec[r0 + i] -= acc[i];
    }
}

// ---------------------------------------------------------------------------
// One-sided Jacobi SVD (Hestenes), standing in for Eigen::JacobiSVD with thin U/V
// (compute.hpp:27-28). Input A is m x n column-major with m >= n. Outputs: S (n,
// descending), U (m x n, orthonormal columns), V (n x n, orthogonal).
// ---------------------------------------------------------------------------
void jacobi_svd_tall(Index m, Index n, const double* A, double* S, double* U, double* V) {
    std::vector<double> G(A, A + m * n);
    std::vector<double> VV(n * n, 0.0);
    for (Index i = 0; i < n; ++i) VV[i * n + i] = 1.0;
    const double eps = std::numeric_limits<double>::epsilon();
    std::vector<double> nrm(n);
    for (Index j = 0; j < n; ++j) nrm[j] = dot(&G[j * m], &G[j * m], m);

    for (int sweep = 0; sweep < 80; ++sweep) {
        bool rotated = false;
        for (Index p = 0; p < n - 1; ++p) {
            for (Index q = p + 1; q < n; ++q) {
                double* gp = &G[p * m];
                double* gq = &G[q * m];
                const double alpha = nrm[p], beta = nrm[q];
                const double gamma = dot(gp, gq, m);
                if (gamma == 0 || std::abs(gamma) <= eps * static_cast<double>(m) * std::sqrt(alpha * beta)) continue;
                rotated = true;
                // Rutishauser's formulas for the Jacobi rotation that zeroes gamma.
                const double zeta = (beta - alpha) / (2 * gamma);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::abs(zeta) + std::sqrt(1 + zeta * zeta));
                const double c = 1 / std::sqrt(1 + t * t);
                const double s = c * t;
                for (Index i = 0; i < m; ++i) {
                    const double a = gp[i], b = gq[i];
                    gp[i] = c * a - s * b;
                    gq[i] = s * a + c * b;
                }
                double* vp = &VV[p * n];
                double* vq = &VV[q * n];
                for (Index i = 0; i < n; ++i) {
                    const double a = vp[i], b = vq[i];
                    vp[i] = c * a - s * b;
                    vq[i] = s * a + c * b;
                }
                nrm[p] = dot(gp, gp, m);
                nrm[q] = dot(gq, gq, m);
            }
        }
        if (!rotated) break;
    }

    // Singular values are the column norms; sort descending (stable).
    std::vector<double> sv(n);
    for (Index j = 0; j < n; ++j) sv[j] = norm(&G[j * m], m);
    std::vector<Index> order(n);
    for (Index j = 0; j < n; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](Index a, Index b) { return sv[a] > sv[b]; });

    const double smax = n ? sv[order[0]] : 0.0;
    const double zero_tol = smax * eps * static_cast<double>(std::max(m, n));
    Index nonzero = 0;
    for (Index jj = 0; jj < n; ++jj) {
        const Index j = order[jj];
        S[jj] = sv[j];
        std::copy(&VV[j * n], &VV[j * n] + n, V + jj * n);
        if (sv[j] > zero_tol) {
            for (Index i = 0; i < m; ++i) U[jj * m + i] = G[j * m + i] / sv[j];
            ++nonzero;
        } else {
            S[jj] = (sv[j] > 0 ? sv[j] : 0.0);
            std::fill(U + jj * m, U + (jj + 1) * m, 0.0);
        }
    }

    // Orthonormal completion for the zero singular values: Gram-Schmidt (twice)
    // of canonical basis vectors against the columns found so far.
    Index e = 0;
    for (Index jj = nonzero; jj < n; ++jj) {
        double* u = U + jj * m;
        while (e < m) {
            std::fill(u, u + m, 0.0);
            u[e++] = 1.0;
            for (int pass = 0; pass < 2; ++pass)
                for (Index k = 0; k < jj; ++k) {
                    const double d = dot(U + k * m, u, m);
                    for (Index i = 0; i < m; ++i) u[i] -= d * U[k * m + i];
                }
            const double nn = norm(u, m);
            if (nn > 0.5) {
                for (Index i = 0; i < m; ++i) u[i] /= nn;
                break;
            }
        }
    }

    // Canonical signs: the largest-magnitude entry of each V column (first one
    // on ties) is made positive, and the U column follows. Eigen's convention is
    // not reproducible here; a fixed one keeps the oracle and the GPU engine
    // comparable wherever the outputs depend on the signs of B's singular
    // vectors (the max-iterations output of compute.hpp:268-305).
    for (Index jj = 0; jj < n; ++jj) {
        double* v = V + jj * n;
        Index arg = 0;
        for (Index i = 1; i < n; ++i)
            if (std::abs(v[i]) > std::abs(v[arg])) arg = i;
        if (v[arg] < 0) {
            for (Index i = 0; i < n; ++i) v[i] = -v[i];
            for (Index i = 0; i < m; ++i) U[jj * m + i] = -U[jj * m + i];
        }
    }
}

// Canonical signs shared by both SVD forms: the largest-magnitude entry of each
// V column (first one on ties) is made positive, and the U column follows.
// Eigen's own signs follow from its rotation sequence; a fixed convention keeps
// the oracle and the GPU engine comparable wherever outputs depend on the signs
// of B's singular vectors (the max-iterations output of compute.hpp:268-305).
// Flipping a (u, v) pair leaves the restart (compute.hpp:244-293) unchanged up
// to the signs of the rotated basis columns.
void canonical_signs(Index m, Index n, double* U, double* V) {
    for (Index jj = 0; jj < n; ++jj) {
        double* v = V + jj * n;
        Index arg = 0;
        for (Index i = 1; i < n; ++i)
            if (std::abs(v[i]) > std::abs(v[arg])) arg = i;
        if (v[arg] < 0) {
            for (Index i = 0; i < n; ++i) v[i] = -v[i];
            for (Index i = 0; i < m; ++i) U[jj * m + i] = -U[jj * m + i];
        }
    }
}

// Two-sided Jacobi SVD of a real square n x n matrix A (column-major): the
// algorithm of Eigen::JacobiSVD (Eigen 5.0.0) for square input, restated.
//  * A is divided by its largest |entry| (1 if zero); U = V = I.
//  * Sweeps over p = 1..n-1, q = 0..p-1 until a sweep finds every |A_pq| and
//    |A_qp| at most max(smallest normal, 2 eps d), d the largest |A_ii| seen
//    (updated after each rotation).
//  * Each such 2x2 block [a b; c d'] is made symmetric by a left rotation
//    (t = a + d', e = c - b; if |e| is below the smallest normal the identity,
//    else s1 = 1 / sqrt(1 + (t/e)^2), c1 = (t/e) s1), then diagonalized by the
//    symmetric Jacobi rotation of [x y; y z] (tau = (x - z) / (2|y|),
//    t = 1 / (tau +- sqrt(tau^2 + 1)) with the sign of tau, n = 1/sqrt(t^2 + 1),
//    c = n, s = -sign(t) sign(y) |t| n); the left rotation applied to A is
//    the product of the first with the transpose of the second.
//  * Rotations (c, s) act on a pair (x, y) as x' = c x + s y, y' = -s x + c y:
//    on rows p, q of A from the left; on columns of A and V from the right with
//    (c, -s); on columns of U with the left rotation.
//  * Singular values |A_ii| times the scale, U column negated where A_ii < 0,
//    then ordered decreasingly by repeatedly taking the largest remaining value
//    (first on ties) and swapping it, with its U and V columns, into place.
// Outputs: S (n), U (n x n), V (n x n); canonical signs applied.
void jacobi_svd_square(Index n, const double* Ain, double* S, double* U, double* V) {
    const double eps = std::numeric_limits<double>::epsilon();
    const double tiny = std::numeric_limits<double>::min();
    const double precision = 2 * eps;
    double scale = 0;
    for (Index e = 0; e < n * n; ++e) scale = std::max(scale, std::abs(Ain[e]));
    if (scale == 0) scale = 1;
    std::vector<double> A(static_cast<size_t>(n * n));
    for (Index e = 0; e < n * n; ++e) A[e] = Ain[e] / scale;
    std::fill(U, U + n * n, 0.0);
    std::fill(V, V + n * n, 0.0);
    for (Index i = 0; i < n; ++i) U[i * n + i] = V[i * n + i] = 1.0;
    auto a = [&](Index r, Index c) -> double& { return A[c * n + r]; };
    // x' = c x + s y, y' = -s x + c y over `len` entries with strides.
    auto rot = [](double* x, double* y, Index len, Index stride, double c, double s) {
        for (Index i = 0; i < len; ++i) {
            const double xi = x[i * stride], yi = y[i * stride];
            x[i * stride] = c * xi + s * yi;
            y[i * stride] = -s * xi + c * yi;
        }
    };
    double maxdiag = 0;
    for (Index i = 0; i < n; ++i) maxdiag = std::max(maxdiag, std::abs(a(i, i)));
    bool finished = false;
    while (!finished) {
        finished = true;
        for (Index p = 1; p < n; ++p) {
            for (Index q = 0; q < p; ++q) {
                const double threshold = std::max(tiny, precision * maxdiag);
                if (!(std::abs(a(p, q)) > threshold || std::abs(a(q, p)) > threshold)) continue;
                finished = false;
                // 2x2 block of rows/columns (p, q): [m00 m01; m10 m11].
                double m00 = a(p, p), m01 = a(p, q), m10 = a(q, p), m11 = a(q, q);
                double c1 = 1, s1 = 0;
                const double t = m00 + m11, d = m10 - m01;
                if (!(std::abs(d) < tiny)) {
                    const double u = t / d;
                    const double tmp = std::sqrt(1 + u * u);
                    s1 = 1 / tmp;
                    c1 = u / tmp;
                }
                {   // the left rotation (c1, s1) on the block's rows
                    const double r00 = c1 * m00 + s1 * m10, r01 = c1 * m01 + s1 * m11;
                    const double r10 = -s1 * m00 + c1 * m10, r11 = -s1 * m01 + c1 * m11;
                    m00 = r00;
                    m01 = r01;
                    m10 = r10;
                    m11 = r11;
                }
                double cr = 1, sr = 0;   // the symmetric Jacobi rotation of [m00 m01; m01 m11]
                const double deno = 2 * std::abs(m01);
                if (!(deno < tiny)) {
                    const double tau = (m00 - m11) / deno;
                    const double w = std::sqrt(tau * tau + 1);
                    const double tt = tau > 0 ? 1 / (tau + w) : 1 / (tau - w);
                    const double sign_t = tt > 0 ? 1.0 : -1.0;
                    const double nn = 1 / std::sqrt(tt * tt + 1);
                    sr = -sign_t * (m01 / std::abs(m01)) * std::abs(tt) * nn;
                    cr = nn;
                }
                // Left rotation of A: (c1, s1) times the transpose (cr, -sr).
                const double cl = c1 * cr + s1 * sr, sl = s1 * cr - c1 * sr;
                rot(&a(p, 0), &a(q, 0), n, n, cl, sl);          // rows p, q
                rot(U + p * n, U + q * n, n, 1, cl, sl);         // columns of U
                rot(&a(0, p), &a(0, q), n, 1, cr, -sr);         // columns of A
                rot(V + p * n, V + q * n, n, 1, cr, -sr);        // columns of V
                maxdiag = std::max(maxdiag, std::max(std::abs(a(p, p)), std::abs(a(q, q))));
            }
        }
    }
    for (Index i = 0; i < n; ++i) {
        const double d = a(i, i);
        S[i] = std::abs(d);
        if (d < 0)
            for (Index r = 0; r < n; ++r) U[i * n + r] = -U[i * n + r];
    }
    for (Index i = 0; i < n; ++i) S[i] *= scale;
    for (Index i = 0; i < n; ++i) {
        Index pos = i;
        for (Index j = i + 1; j < n; ++j)
            if (S[j] > S[pos]) pos = j;
        if (S[pos] == 0) break;
        if (pos != i) {
            std::swap(S[i], S[pos]);
            for (Index r = 0; r < n; ++r) {
                std::swap(U[i * n + r], U[pos * n + r]);
                std::swap(V[i * n + r], V[pos * n + r]);
            }
        }
    }
    canonical_signs(n, n, U, V);
}

// Thin SVD of any m x n matrix: U (m x p), S (p), V (n x p), p = min(m, n).
void jacobi_svd(Index m, Index n, const double* A, std::vector<double>& S, Dense& U, Dense& V) {
    const Index p = std::min(m, n);
    S.assign(p, 0.0);
    U = Dense(m, p);
    V = Dense(n, p);
    if (m >= n) {
        Dense Vsq(n, n);
        jacobi_svd_tall(m, n, A, S.data(), U.v.data(), Vsq.v.data());
        V = Vsq;
    } else {
        std::vector<double> At(static_cast<size_t>(m * n));
        for (Index c = 0; c < n; ++c)
            for (Index r = 0; r < m; ++r) At[r * n + c] = A[c * m + r];
        Dense Usq(m, m);
        jacobi_svd_tall(n, m, At.data(), S.data(), V.v.data(), Usq.v.data());
        U = Usq;
    }
}

// ---------------------------------------------------------------------------
// compute.hpp helpers.
// ---------------------------------------------------------------------------
// compute.hpp:49-56
bool requested_greater_than_or_equal_to_half_smaller(Index requested, Index smaller) {
    const Index half = smaller / 2;
    if (requested == half) return smaller % 2 == 0;
    return requested > half;
}

// compute.hpp:59-67
Index choose_requested_plus_extra_work_or_smaller(Index requested, int extra_work, Index smaller) {
    if (requested >= smaller) return smaller;
    return requested + std::min<Index>(smaller - requested, extra_work);
}

// compute.hpp:78-111
Index update_k(Index k, Index requested, Index n_converged, Index work) {
    if (work <= 3) return 1;
    const Index limit = work - 3;
    auto less = [&](Index val) { return val < requested || (val - requested) < n_converged; };
    if (less(k)) {
        if (less(limit)) return limit;
        return std::max<Index>(requested + n_converged, 1);
    }
    return std::max<Index>(std::min(k, limit), 1);
}

// compute.hpp:30-46: exact SVD of the realized matrix.
void exact(const Matrix& mat, Index requested, double* U, double* V, double* D) {
    const Index nr = mat.rows(), nc = mat.cols();
    std::vector<double> buf(static_cast<size_t>(nr * nc));
    mat.realize(buf.data());
    std::vector<double> S;
    Dense UU, VV;
    jacobi_svd(nr, nc, buf.data(), S, UU, VV);
    for (Index j = 0; j < requested; ++j) {
        D[j] = S[j];
        std::copy(UU.col(j), UU.col(j) + nr, U + j * nr);
        std::copy(VV.col(j), VV.col(j) + nc, V + j * nc);
    }
}

// LanczosWorkspace, lanczos.hpp:23-39.
struct LanczosWorkspace {
    std::vector<double> F, W_next, otmp;
    LanczosWorkspace(const Matrix& m) : F(m.cols()), W_next(m.rows()), otmp(m.cols() > m.rows() ? m.cols() : m.rows()) {}
};

// run_lanczos_bidiagonalization, lanczos.hpp:54-143.
void run_lanczos_bidiagonalization(const Matrix& mat, LanczosWorkspace& inter, Dense& W, Dense& V, Dense& B,
                                   std::mt19937_64& eng, Index start, const Options& opt) {
    const double raw_eps = opt.invariant_subspace_tolerance;
    const double eps = (raw_eps < 0 ? std::pow(std::numeric_limits<double>::epsilon(), 0.8) : raw_eps);
    const Index work = W.nc;
    const Index nr = mat.rows(), nc = mat.cols();
    double* F = inter.F.data();
    double* Wn = inter.W_next.data();
    double* otmp = inter.otmp.data();

    std::copy(V.col(start), V.col(start) + nc, F);
    mat.multiply(F, Wn);                                  // lanczos.hpp:73-74
    if (start) orthogonalize_vector(W, Wn, start, otmp);  // :77-79

    double S = norm(Wn, nr);                              // :81-84
    if (S < eps) throw std::runtime_error("starting vector near the null space of the input matrix");
    for (Index r = 0; r < nr; ++r) Wn[r] /= S;            // :85-86
    std::copy(Wn, Wn + nr, W.col(start));

    for (Index j = start; j < work; ++j) {                // :89
        mat.adjoint_multiply(Wn, F);                      // :93
        const double* vj = V.col(j);
        for (Index c = 0; c < nc; ++c) F[c] -= S * vj[c]; // :95
        orthogonalize_vector(V, F, j + 1, otmp);          // :96

        if (j + 1 < work) {
            double R_F = norm(F, nc);                     // :99
            if (R_F < eps) {                              // :101-106
                fill_with_random_normals(F, nc, eng);
                orthogonalize_vector(V, F, j + 1, otmp);
                R_F = norm(F, nc);
                for (Index c = 0; c < nc; ++c) F[c] /= R_F;
                R_F = 0;
            } else {
                for (Index c = 0; c < nc; ++c) F[c] /= R_F;
            }
            std::copy(F, F + nc, V.col(j + 1));           // :111
            B(j, j) = S;                                  // :112
            B(j, j + 1) = R_F;                            // :113

            mat.multiply(F, Wn);                          // :115
            const double* wj = W.col(j);
            for (Index r = 0; r < nr; ++r) Wn[r] -= R_F * wj[r];  // :116
            orthogonalize_vector(W, Wn, j + 1, otmp);     // :121

            S = norm(Wn, nr);                             // :123
            if (S < eps) {                                // :124-129
                fill_with_random_normals(Wn, nr, eng);
                orthogonalize_vector(W, Wn, j + 1, otmp);
                S = norm(Wn, nr);
                for (Index r = 0; r < nr; ++r) Wn[r] /= S;
                S = 0;
            } else {
                for (Index r = 0; r < nr; ++r) Wn[r] /= S;
            }
            std::copy(Wn, Wn + nr, W.col(j + 1));         // :134
        } else {
            B(j, j) = S;                                  // :140
        }
    }
}

// out[:, :k] = Q[:, :w] * R[:, :k]  (the rotation GEMMs of compute.hpp:268,279,302,305).
// Each output entry sums over j in column order; rows are processed in blocks
// that stay cache-resident while the output columns are formed four at a time
// (each loaded row entry of Q feeds four products, as an optimized GEMM's
// register blocking does; the sums are the same, term by term).
void rotate(const Dense& Q, const Dense& R, Index k, Dense& out) {
    const Index L = Q.nr, w = Q.nc;
    const int nt = g_dense_threads;
    const Index nblocks = (L + kDenseRowBlock - 1) / kDenseRowBlock;
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1 && L > 4096)
    for (Index b = 0; b < nblocks; ++b) {
        const Index r0 = b * kDenseRowBlock, r1 = std::min(L, r0 + kDenseRowBlock), nr = r1 - r0;
        double acc[4][kDenseRowBlock];
        for (Index c = 0; c < k; c += 4) {
            const Index cn = std::min<Index>(4, k - c);
            for (Index u = 0; u < 4; ++u)
                for (Index i = 0; i < nr; ++i) acc[u][i] = 0;
            for (Index j = 0; j < w; ++j) {
                const double* q = Q.v.data() + j * L + r0;
                const double ra = R(j, c), rb = cn > 1 ? R(j, c + 1) : 0.0, rc = cn > 2 ? R(j, c + 2) : 0.0,
                             rd = cn > 3 ? R(j, c + 3) : 0.0;
                for (Index i = 0; i < nr; ++i) {
                    const double qi = q[i];
                    acc[0][i] += qi * ra;
                    acc[1][i] += qi * rb;
                    acc[2][i] += qi * rc;
                    acc[3][i] += qi * rd;
                }
            }
            for (Index u = 0; u < cn; ++u) {
                double* o = out.v.data() + (c + u) * out.nr + r0;
                for (Index i = 0; i < nr; ++i) o[i] = acc[u][i];
            }
        }
    }
}

struct Stats {
    int64_t matvecs = 0;
    int64_t lanczos_steps = 0;
};

// compute, compute.hpp:141-308.
std::pair<bool, int> compute(const Matrix& mat, Index number, double* outU, double* outV, double* outD,
                             Index* out_number, const Options& opt, Stats* stats, int max_restarts_override) {
    const Index smaller = std::min(mat.rows(), mat.cols());
    Index requested = number;
    if (requested > smaller) {                                    // :152-160
        if (opt.cap_number) requested = smaller;
        else throw std::runtime_error("requested number of singular values cannot be greater than the smaller matrix dimension");
    } else if (requested == smaller && !opt.exact_for_large_number) {
        throw std::runtime_error("requested number of singular values must be less than the smaller matrix dimension for IRLBA iterations");
    }
    *out_number = requested;

    if ((opt.exact_for_small_matrix && smaller < 6) ||            // :164-170
        (opt.exact_for_large_number && requested_greater_than_or_equal_to_half_smaller(requested, smaller))) {
        exact(mat, requested, outU, outV, outD);
        return {true, 0};
    }

    const Index work = choose_requested_plus_extra_work_or_smaller(requested, opt.extra_work, smaller);  // :172
    if (work == 0) throw std::runtime_error("number of requested dimensions must be positive");

    const Index nr = mat.rows(), nc = mat.cols();
    Dense V(nc, work);                                            // :179-190
    std::mt19937_64 eng(opt.seed);
    if (opt.initial) {
        if (opt.initial_size != nc) throw std::runtime_error("initialization vector does not have expected number of rows");
        std::copy(opt.initial, opt.initial + nc, V.col(0));
    } else {
        fill_with_random_normals(V.col(0), nc, eng);
    }
    {
        const double n0 = norm(V.col(0), nc);
        for (Index c = 0; c < nc; ++c) V(c, 0) /= n0;
    }

    bool converged = false;
    int iter = 0;
    Index k = 0;
    LanczosWorkspace lp(mat);
    Dense W(nr, work), Wtmp(nr, work), Vtmp(nc, work), B(work, work);
    std::vector<double> res(work), prevS(work);
    const double tol = opt.convergence_tolerance;
    const double svtol = opt.singular_value_ratio_tolerance;
    const double svtol_actual = (svtol >= 0 ? svtol : tol);

    std::vector<double> BS;
    Dense BU, BV;
    const int max_iter = (max_restarts_override >= 0 ? max_restarts_override : opt.max_iterations);

    for (; iter < max_iter; ++iter) {                             // :213
        run_lanczos_bidiagonalization(mat, lp, W, V, B, eng, k, opt);
        if (stats) {
            stats->matvecs += 2 * (work - k);
            stats->lanczos_steps += work - k;
        }

        BS.assign(work, 0.0);                                     // :225
        BU = Dense(work, work);
        BV = Dense(work, work);
        jacobi_svd_square(work, B.v.data(), BS.data(), BU.v.data(), BV.v.data());
        if (B(work - 1, work - 1) == 0) {                         // :231-234
            converged = true;
            break;
        }

        const double R_F = norm(lp.F.data(), nc);                 // :236-237
        for (Index j = 0; j < work; ++j) res[j] = R_F * BU(work - 1, j);  // :244

        Index n_converged = 0;
        if (iter > 0) {                                           // :246-264
            const double Smax = *std::max_element(BS.begin(), BS.end());
            const double threshold = Smax * tol;
            for (Index j = 0; j < work; ++j) {
                if (std::abs(res[j]) <= threshold) {
                    const double ratio = std::abs(BS[j] - prevS[j]) / BS[j];
                    if (ratio <= svtol_actual) ++n_converged;
                }
            }
            if (n_converged >= requested) {
                converged = true;
                break;
            }
        }
        prevS = BS;                                               // :265

        k = update_k(k, requested, n_converged, work);            // :267
        rotate(V, BV, k, Vtmp);                                   // :268-269
        for (Index c = 0; c < k; ++c) std::copy(Vtmp.col(c), Vtmp.col(c) + nc, V.col(c));
        for (Index c = 0; c < nc; ++c) V(c, k) = lp.F[c] / R_F;   // :277
        rotate(W, BU, k, Wtmp);                                   // :279-280
        for (Index c = 0; c < k; ++c) std::copy(Wtmp.col(c), Wtmp.col(c) + nr, W.col(c));

        std::fill(B.v.begin(), B.v.end(), 0.0);                   // :282-293
        for (Index l = 0; l < k; ++l) {
            B(l, l) = BS[l];
            B(l, k) = res[l];
        }
    }

    // Output assembly, compute.hpp:298-305 (uses the last SVD of B, which on a
    // max-iterations exit predates the final rotation, as in the reference).
    if (BS.empty()) {  // no restart ran (max_iterations == 0): no SVD of B exists
        BS.assign(work, 0.0);
        BU = Dense(work, work);
        BV = Dense(work, work);
    }
    for (Index j = 0; j < requested; ++j) outD[j] = BS[j];
    Dense Uo(nr, requested), Vo(nc, requested);
    rotate(W, BU, requested, Uo);
    rotate(V, BV, requested, Vo);
    std::copy(Uo.v.begin(), Uo.v.end(), outU);
    std::copy(Vo.v.begin(), Vo.v.end(), outV);
    return {converged, converged ? iter + 1 : iter};
}

// pca column statistics, pca.hpp:85-109 (dense) and the same quantities for a
// compressed sparse matrix with implicit zeros.
void column_stats_dense(const DenseMatrix& m, bool center, bool scale, double* center0, double* scale0) {
    const Index nr = m.nr, nc = m.nc;
    std::vector<double> buffer(nr);
    for (Index i = 0; i < nc; ++i) {
        for (Index r = 0; r < nr; ++r) buffer[r] = m.at(r, i);
        double mean = 0;
        if (center) {
            double s = 0;
            for (Index r = 0; r < nr; ++r) s += buffer[r];
            mean = s / nr;
            center0[i] = mean;
        }
        if (scale) {
            double var = 0;
            for (Index r = 0; r < nr; ++r) var += (buffer[r] - mean) * (buffer[r] - mean);
            scale0[i] = var ? std::sqrt(var / (nr - 1)) : 1.0;
        }
    }
}

void column_stats_sparse(const SparseMatrix& m, bool center, bool scale, double* center0, double* scale0) {
    const Index nr = m.rows(), nc = m.cols();
    std::vector<double> sum(nc, 0.0), cnt(nc, 0.0);
    for (Index p = 0; p < m.primary_dim; ++p)
        for (int64_t s = m.ptrs[p]; s < m.ptrs[p + 1]; ++s) {
            const Index c = m.column_major ? p : m.indices[s];
            sum[c] += m.value(s);
            cnt[c] += 1;
        }
    std::vector<double> mean(nc, 0.0);
    for (Index c = 0; c < nc; ++c) {
        if (center) {
            mean[c] = sum[c] / nr;
            center0[c] = mean[c];
        }
    }
    if (scale) {
        std::vector<double> var(nc, 0.0);
        for (Index p = 0; p < m.primary_dim; ++p)
            for (int64_t s = m.ptrs[p]; s < m.ptrs[p + 1]; ++s) {
                const Index c = m.column_major ? p : m.indices[s];
                const double d = m.value(s) - mean[c];
                var[c] += d * d;
            }
        for (Index c = 0; c < nc; ++c) {
            var[c] += (nr - cnt[c]) * mean[c] * mean[c];
            scale0[c] = var[c] ? std::sqrt(var[c] / (nr - 1)) : 1.0;
        }
    }
}

}  // namespace oracle

// ===========================================================================
// C interface used by the Python tests and bench (ctypes).
// ===========================================================================
using namespace oracle;

extern "C" {

struct OracleOptions {
    double invariant_subspace_tolerance;
    double convergence_tolerance;
    double singular_value_ratio_tolerance;
    int32_t extra_work;
    int32_t max_iterations;
    int32_t exact_for_small_matrix;
    int32_t exact_for_large_number;
    int32_t cap_number;
    int32_t pad0;
    uint64_t seed;
    const double* initial;  // may be NULL
    int64_t initial_size;
};

// Base matrix + decorator chain description.
//   kind 0: dense column-major (data, ld); kind 1: dense row-major; kind 2: sparse.
//   chain: center (length ncol, or NULL) then scale (or NULL) applied on top, in
//   the order given by center_outer (0: Scaled(Centered(base)), 1: Centered(Scaled(base))).
struct OracleMatrixSpec {
    int32_t kind;
    int32_t column_major;
    int32_t num_threads;
    int32_t center_outer;
    int64_t nrow, ncol, ld;
    const double* dense;
    const double* values;
    const int32_t* indices;
    const int64_t* pointers;
    const double* center;
    const double* scale;
    int32_t scale_column;
    int32_t scale_divide;
    const float* values32;   // FP32 values of a sparse base (kind 2) instead of `values`, or NULL
};

static thread_local std::string g_error;

const char* oracle_last_error() { return g_error.c_str(); }

void oracle_set_dense_threads(int nt) { oracle::g_dense_threads = nt < 1 ? 1 : nt; }

struct Chain {
    std::unique_ptr<Matrix> base, first, second;
    const Matrix* top = nullptr;
};

static void build_chain(const OracleMatrixSpec* s, Chain& ch) {
    if (s->kind == 2) {
        ch.base.reset(new SparseMatrix(s->nrow, s->ncol, s->values, s->indices, s->pointers, s->column_major != 0,
                                       s->num_threads < 1 ? 1 : s->num_threads, s->values32));
    } else {
        ch.base.reset(new DenseMatrix(s->nrow, s->ncol, s->dense, s->ld, s->kind == 1));
    }
    ch.top = ch.base.get();
    auto add_center = [&](std::unique_ptr<Matrix>& slot) {
        slot.reset(new CenteredMatrix(ch.top, s->center));
        ch.top = slot.get();
    };
    auto add_scale = [&](std::unique_ptr<Matrix>& slot) {
        slot.reset(new ScaledMatrix(ch.top, s->scale, s->scale_column != 0, s->scale_divide != 0));
        ch.top = slot.get();
    };
    if (s->center_outer) {
        if (s->scale) add_scale(ch.first);
        if (s->center) add_center(ch.second);
    } else {
        if (s->center) add_center(ch.first);
        if (s->scale) add_scale(ch.second);
    }
}

static Options to_options(const OracleOptions* o) {
    Options opt;
    if (!o) return opt;
    opt.invariant_subspace_tolerance = o->invariant_subspace_tolerance;
    opt.convergence_tolerance = o->convergence_tolerance;
    opt.singular_value_ratio_tolerance = o->singular_value_ratio_tolerance;
    opt.extra_work = o->extra_work;
    opt.max_iterations = o->max_iterations;
    opt.exact_for_small_matrix = o->exact_for_small_matrix != 0;
    opt.exact_for_large_number = o->exact_for_large_number != 0;
    opt.cap_number = o->cap_number != 0;
    opt.seed = o->seed;
    opt.initial = o->initial;
    opt.initial_size = o->initial_size;
    return opt;
}

void oracle_default_options(OracleOptions* o) {
    Options d;
    o->invariant_subspace_tolerance = d.invariant_subspace_tolerance;
    o->convergence_tolerance = d.convergence_tolerance;
    o->singular_value_ratio_tolerance = d.singular_value_ratio_tolerance;
    o->extra_work = d.extra_work;
    o->max_iterations = d.max_iterations;
    o->exact_for_small_matrix = d.exact_for_small_matrix;
    o->exact_for_large_number = d.exact_for_large_number;
    o->cap_number = d.cap_number;
    o->pad0 = 0;
    o->seed = d.seed;
    o->initial = nullptr;
    o->initial_size = 0;
}

int oracle_multiply(const OracleMatrixSpec* s, const double* x, double* out) {
    try { Chain ch; build_chain(s, ch); ch.top->multiply(x, out); return 0; }
    catch (const std::exception& e) { g_error = e.what(); return 1; }
}

int oracle_adjoint_multiply(const OracleMatrixSpec* s, const double* y, double* out) {
    try { Chain ch; build_chain(s, ch); ch.top->adjoint_multiply(y, out); return 0; }
    catch (const std::exception& e) { g_error = e.what(); return 1; }
}

int oracle_realize(const OracleMatrixSpec* s, double* out) {
    try { Chain ch; build_chain(s, ch); ch.top->realize(out); return 0; }
    catch (const std::exception& e) { g_error = e.what(); return 1; }
}

// Thread partitions of the ParallelSparseMatrix core (sparse.hpp:35-115).
int oracle_sparse_partitions(const OracleMatrixSpec* s, int64_t* primary, int64_t* secondary, int64_t* secondary_nz) {
    try {
        SparseMatrix m(s->nrow, s->ncol, s->values, s->indices, s->pointers, s->column_major != 0, s->num_threads,
                       s->values32);
        const int nt = s->num_threads;
        for (int t = 0; t <= nt; ++t) {
            primary[t] = m.primary_boundaries[t];
            secondary[t] = m.secondary_boundaries[t];
            for (Index c = 0; c < m.primary_dim; ++c) secondary_nz[t * m.primary_dim + c] = m.secondary_nonzero_boundaries[t][c];
        }
        return 0;
    } catch (const std::exception& e) { g_error = e.what(); return 1; }
}

// compute() with outputs sized for `number` (capped numbers are reported back).
int oracle_compute(const OracleMatrixSpec* s, int64_t number, const OracleOptions* o, double* U, double* V, double* D,
                   int64_t* out_number, int32_t* converged, int32_t* iterations, int64_t* matvecs, int32_t max_restarts) {
    try {
        Chain ch;
        build_chain(s, ch);
        Options opt = to_options(o);
        Stats st;
        auto r = compute(*ch.top, number, U, V, D, out_number, opt, &st, max_restarts);
        *converged = r.first;
        *iterations = r.second;
        if (matvecs) *matvecs = st.matvecs;
        return 0;
    } catch (const std::exception& e) { g_error = e.what(); return 1; }
}

// pca(), pca.hpp:55-139, for dense (kind 0/1) or sparse (kind 2) input; the
// spec's own center/scale pointers are ignored.
int oracle_pca(const OracleMatrixSpec* s, int32_t center, int32_t scale, int64_t number, const OracleOptions* o,
               double* scores, double* rotation, double* variances, int64_t* out_number, int32_t* converged,
               int32_t* iterations, double* center_out, double* scale_out, int32_t max_restarts, int64_t* steps) {
    try {
        const Index nr = s->nrow, nc = s->ncol;
        std::vector<double> center0, scale0;
        if (center) {
            if (nr < 1) throw std::runtime_error("cannot center with no observations");
            center0.resize(nc);
        }
        if (scale) {
            if (nr < 2) throw std::runtime_error("cannot scale with fewer than two observations");
            scale0.resize(nc);
        }
        OracleMatrixSpec spec = *s;
        spec.center = nullptr;
        spec.scale = nullptr;
        Chain base;
        build_chain(&spec, base);
        if (center || scale) {
            if (s->kind == 2) column_stats_sparse(*static_cast<SparseMatrix*>(base.base.get()), center, scale, center0.data(), scale0.data());
            else column_stats_dense(*static_cast<DenseMatrix*>(base.base.get()), center, scale, center0.data(), scale0.data());
        }
        spec.center = center ? center0.data() : nullptr;
        spec.scale = scale ? scale0.data() : nullptr;
        spec.scale_column = 1;
        spec.scale_divide = 1;
        spec.center_outer = 0;
        Chain ch;
        build_chain(&spec, ch);
        Options opt = to_options(o);
        Stats st;
        auto r = compute(*ch.top, number, scores, rotation, variances, out_number, opt, &st, max_restarts);
        if (steps) *steps = st.lanczos_steps;
        const Index num = *out_number;
        for (Index j = 0; j < num; ++j)
            for (Index i = 0; i < nr; ++i) scores[j * nr + i] *= variances[j];   // pca.hpp:130
        if (nc > 1) {                                                            // pca.hpp:131-136
            const double denom = static_cast<double>(nr - 1);
            for (Index j = 0; j < num; ++j) variances[j] = variances[j] * variances[j] / denom;
        }
        if (center_out && center) std::copy(center0.begin(), center0.end(), center_out);
        if (scale_out && scale) std::copy(scale0.begin(), scale0.end(), scale_out);
        *converged = r.first;
        *iterations = r.second;
        return 0;
    } catch (const std::exception& e) { g_error = e.what(); return 1; }
}

// One Lanczos bidiagonalization from column `start` (lanczos.hpp:54-143); W, V, B
// column-major, updated in place. F receives the final residual.
int oracle_lanczos(const OracleMatrixSpec* s, double* W, double* V, double* B, int64_t work, int64_t start,
                   uint64_t seed, double* F, const OracleOptions* o) {
    try {
        Chain ch;
        build_chain(s, ch);
        const Index nr = ch.top->rows(), nc = ch.top->cols();
        Dense Wd(nr, work), Vd(nc, work), Bd(work, work);
        std::copy(W, W + nr * work, Wd.v.begin());
        std::copy(V, V + nc * work, Vd.v.begin());
        std::copy(B, B + work * work, Bd.v.begin());
        std::mt19937_64 eng(seed);
        LanczosWorkspace lp(*ch.top);
        Options opt = to_options(o);
        run_lanczos_bidiagonalization(*ch.top, lp, Wd, Vd, Bd, eng, start, opt);
        std::copy(Wd.v.begin(), Wd.v.end(), W);
        std::copy(Vd.v.begin(), Vd.v.end(), V);
        std::copy(Bd.v.begin(), Bd.v.end(), B);
        std::copy(lp.F.begin(), lp.F.end(), F);
        return 0;
    } catch (const std::exception& e) { g_error = e.what(); return 1; }
}

void oracle_orthogonalize_vector(const double* Q, int64_t L, int64_t ncols_total, double* vec, int64_t ncols) {
    Dense Qd(L, ncols_total);
    std::copy(Q, Q + L * ncols_total, Qd.v.begin());
    std::vector<double> tmp(ncols_total > 0 ? ncols_total : 1);
    orthogonalize_vector(Qd, vec, ncols, tmp.data());
}

int64_t oracle_update_k(int64_t k, int64_t requested, int64_t n_converged, int64_t work) {
    return update_k(k, requested, n_converged, work);
}
int32_t oracle_requested_ge_half_smaller(int64_t requested, int64_t smaller) {
    return requested_greater_than_or_equal_to_half_smaller(requested, smaller);
}
int64_t oracle_choose_work(int64_t requested, int32_t extra_work, int64_t smaller) {
    return choose_requested_plus_extra_work_or_smaller(requested, extra_work, smaller);
}

// Thin SVD (the JacobiSVD stand-in): U m x p, S p, V n x p.
void oracle_svd(int64_t m, int64_t n, const double* A, double* U, double* S, double* V) {
    std::vector<double> SS;
    Dense UU, VV;
    jacobi_svd(m, n, A, SS, UU, VV);
    std::copy(SS.begin(), SS.end(), S);
    std::copy(UU.v.begin(), UU.v.end(), U);
    std::copy(VV.v.begin(), VV.v.end(), V);
}

// The restart SVD of a square matrix (the Eigen::JacobiSVD restatement): U, V n x n.
void oracle_svd_square(int64_t n, const double* A, double* U, double* S, double* V) {
    jacobi_svd_square(n, A, S, U, V);
}

void oracle_fill_random_normals(double* vec, int64_t n, uint64_t seed) {
    std::mt19937_64 eng(seed);
    fill_with_random_normals(vec, n, eng);
}

}  // extern "C"
