// Host side of the differentiation form: the truncated-SVD adjoint.
//
// For A' (m x n; the base matrix or its centre/scale chain) with top-k SVD
// A' ~ U S V^T and cotangents gU, gS, gV of a scalar loss, the gradient is
//   dL/dA' = U M V^T + (Y S + A_perp Z) V^T + U (S Z^T + Y^T A_perp)
// with A_perp = (I - U U^T) A' (I - V V^T),
//   M = diag(gS) + (F o (U^T gU - gU^T U)) S + S (F o (V^T gV - gV^T V)),
//   F_ab = 1 / (s_b^2 - s_a^2) (a != b), 0 on the diagonal (Townsend 2016),
// and the complement terms solved column by column from
//   (s_j^2 I - A_perp A_perp^T) y_j = (I - U U^T) gU_j,
//   (s_j^2 I - A_perp^T A_perp) z_j = (I - V V^T) gV_j
// by conjugate gradients (positive definite on the complement when s_k
// exceeds the largest singular value of A_perp). When A' has rank k these
// reduce to the projection terms (I - U U^T) gU S^-1 V^T + U S^-1 gV^T (I - V V^T)
// (the first-order perturbation of a singular vector, e.g. Townsend 2016
// eq. 22-23, taken without assuming the trailing singular values vanish).
// The gradient is returned as the rank-2k product Z1 Z2^T with
//   Z1 = [U M + Y S + P_U A' Z | U],  Z2 = [V | Z S + P_V A'^T Y].

#include <cstring>
#include <vector>

#include "matrix.hpp"

namespace irlba_gb300 {

namespace {

struct StreamUse {
    cudaStream_t s = nullptr;
    bool own = false;
    explicit StreamUse(void* user) {
        if (user) {
            s = static_cast<cudaStream_t>(user);
        } else {
            CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            own = true;
        }
    }
    ~StreamUse() {
        if (own) cudaStreamDestroy(s);
    }
};

// The operator A' of a decorator chain on k-column row-major blocks.
struct BlockOp {
    const Chain ch;
    int64_t m = 0, n = 0;
    int k = 0;
    cudaStream_t s;
    DevBuf cvec, svec, tmp, w, part;

    BlockOp(const Chain& c, int kcols, cudaStream_t st) : ch(c), k(kcols), s(st) {
        m = ch.base->nrow;
        n = ch.base->ncol;
        if (ch.scale && !ch.scale_column)
            throw Error(IRLBA_GB300_ERROR_UNSUPPORTED, "the SVD adjoint supports column scaling only");
        if (ch.center) cvec = upload(ch.center->data(), ch.center->size());
        if (ch.scale) svec = upload(ch.scale->data(), ch.scale->size());
        tmp.alloc(sizeof(double) * std::max<int64_t>(n * k, 1));
        w.alloc(sizeof(double) * 128);
        part.alloc(sizeof(double) * static_cast<int64_t>(gram_parts(std::max(m, n))) * 128);
    }

    // Y (m x k) = A' X, X (n x k).
    void mul(const double* X, double* Y) {
        const double* xin = X;
        if (ch.scale) {
            launch_scale_rows(n, k, X, svec.as<double>(), ch.scale_divide, tmp.as<double>(), s);
            xin = tmp.as<double>();
        }
        launch_spmm(ch.base->mul.dev, xin, k, Y, s);
        if (ch.center) {
            launch_coldot(ch.center_outer ? X : xin, nullptr, cvec.as<double>(), n, k, part.as<double>(),
                          w.as<double>(), s);
            launch_rank1(m, k, nullptr, w.as<double>(), -1.0, Y, s);
        }
    }

    // Out (n x k) = A'^T Y, Y (m x k).
    void adj(const double* Y, double* Out) {
        launch_spmm(ch.base->adj.dev, Y, k, Out, s);
        if (ch.center) launch_coldot(Y, nullptr, nullptr, m, k, part.as<double>(), w.as<double>(), s);
        if (ch.center && !ch.center_outer) launch_rank1(n, k, cvec.as<double>(), w.as<double>(), -1.0, Out, s);
        if (ch.scale) launch_scale_rows(n, k, Out, svec.as<double>(), ch.scale_divide, Out, s);
        if (ch.center && ch.center_outer) launch_rank1(n, k, cvec.as<double>(), w.as<double>(), -1.0, Out, s);
    }
};

// X -= Q (Q^T X) for row-major L x k blocks (G: k x k scratch on the device).
void project_out(const double* Q, int64_t L, int k, double* X, double* G, double* part, cudaStream_t s) {
    launch_gram(Q, X, L, k, part, G, s);
    launch_block_update(L, k, k, Q, k, G, -1.0, X, k, nullptr, 1.0, X, k, s);
}

std::vector<double> fetch(const double* d, size_t n, cudaStream_t s) {
    std::vector<double> h(n);
    if (n) {
        CUDA_TRY(d2h_async(h.data(), d, sizeof(double) * n, s));
        CUDA_TRY(cudaStreamSynchronize(s));
    }
    return h;
}

void put(double* d, const std::vector<double>& h, cudaStream_t s) {
    if (!h.empty()) CUDA_TRY(h2d_async(d, h.data(), sizeof(double) * h.size(), s));
}

// Solves (shift_j I - Op) x_j = b_j for every column j by conjugate gradients,
// Op = P A'A'^T P (left) or P A'^T A' P (right), P the projector off the basis
// Qb. Columns stop when ||r_j|| <= tol ||b_j||. The CG scalars live on the
// device (launch_cg_alpha / launch_cg_beta), so iterations are issued in
// groups of kCgCheck without a host round trip; the host reads the status
// once per group. Iterations issued after every column has stopped change
// nothing (alpha = 0 leaves X and R as they are). Returns the number of
// iterations that had an active column.
constexpr int kCgCheck = 8;

int shifted_cg(BlockOp& op, bool left, const double* Qb, const double* B, const std::vector<double>& shift, double tol,
               int max_iter, double* X, cudaStream_t s) {
    const int k = op.k;
    const int64_t L = left ? op.m : op.n, O = left ? op.n : op.m;
    DevBuf R(sizeof(double) * L * k), P(sizeof(double) * L * k), Q(sizeof(double) * L * k),
        W(sizeof(double) * L * k), T(sizeof(double) * std::max<int64_t>(O * k, 1)), G(sizeof(double) * k * k),
        part(sizeof(double) * static_cast<int64_t>(gram_parts(L)) * k * k), dshift(sizeof(double) * k),
        scal(sizeof(double) * 6 * kAdjointMaxK), flags(sizeof(int32_t) * (kAdjointMaxK + 4));
    double* dv = scal.as<double>();                  // coldot outputs
    double* rr = dv + kAdjointMaxK;
    double* bnorm = dv + 2 * kAdjointMaxK;
    double* alpha = dv + 3 * kAdjointMaxK;
    double* beta = dv + 4 * kAdjointMaxK;
    int32_t* st = flags.as<int32_t>();
    int32_t* active = st + 4;
    put(dshift.as<double>(), shift, s);
    CUDA_TRY(cudaMemsetAsync(X, 0, sizeof(double) * L * k, s));
    CUDA_TRY(cudaMemcpyAsync(R.ptr, B, sizeof(double) * L * k, cudaMemcpyDeviceToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(P.ptr, B, sizeof(double) * L * k, cudaMemcpyDeviceToDevice, s));
    launch_coldot(R.as<double>(), R.as<double>(), nullptr, L, k, part.as<double>(), dv, s);
    launch_cg_init(k, dv, rr, bnorm, active, st, s);
    int32_t hst[3] = {0, 0, 0};
    CUDA_TRY(d2h_async(hst, st, sizeof(hst), s));
    CUDA_TRY(cudaStreamSynchronize(s));
    int issued = 0;
    while (hst[0] && issued < max_iter) {
        const int group = std::min(kCgCheck, max_iter - issued);
        for (int g = 0; g < group; ++g, ++issued) {
            project_out(Qb, L, k, P.as<double>(), G.as<double>(), part.as<double>(), s);
            if (left) {
                op.adj(P.as<double>(), T.as<double>());
                op.mul(T.as<double>(), W.as<double>());
            } else {
                op.mul(P.as<double>(), T.as<double>());
                op.adj(T.as<double>(), W.as<double>());
            }
            project_out(Qb, L, k, W.as<double>(), G.as<double>(), part.as<double>(), s);
            launch_shift(L, k, dshift.as<double>(), P.as<double>(), W.as<double>(), Q.as<double>(), s);
            launch_coldot(P.as<double>(), Q.as<double>(), nullptr, L, k, part.as<double>(), dv, s);
            launch_cg_alpha(k, dv, rr, active, alpha, st, s);
            launch_cg_step(L, k, alpha, P.as<double>(), Q.as<double>(), X, R.as<double>(), s);
            launch_coldot(R.as<double>(), R.as<double>(), nullptr, L, k, part.as<double>(), dv, s);
            launch_cg_beta(k, dv, rr, bnorm, tol, active, beta, st, s);
            launch_cg_dir(L, k, beta, R.as<double>(), P.as<double>(), s);
        }
        CUDA_TRY(d2h_async(hst, st, sizeof(hst), s));
        CUDA_TRY(cudaStreamSynchronize(s));
        if (hst[1])
            throw Error(IRLBA_GB300_ERROR_NUMERICAL,
                        "the SVD adjoint needs the k-th singular value to exceed the (k+1)-th "
                        "(complement system not positive definite)");
    }
    if (hst[0])
        throw Error(IRLBA_GB300_ERROR_NUMERICAL,
                    "the SVD adjoint's complement solve did not reach its tolerance within the iteration limit");
    return hst[2];
}

}  // namespace

}  // namespace irlba_gb300

using namespace irlba_gb300;

extern "C" {

irlba_gb300_status irlba_gb300_svd_adjoint_factors(const irlba_gb300_matrix* matrix, int64_t k, const double* U,
                                                   const double* S, const double* V, const double* gU,
                                                   const double* gS, const double* gV, double cg_tol,
                                                   int32_t cg_max_iter, double* Z1, double* Z2,
                                                   int32_t* cg_iterations, void* stream) {
    return guarded([&]() {
        if (!matrix) invalid("matrix is NULL");
        if (!U || !S || !V || !Z1 || !Z2) invalid("U, S, V, Z1 and Z2 must not be NULL");
        const Chain ch = flatten(matrix);
        require_stored(ch.base, "the differentiation form");
        const int64_t m = ch.base->nrow, n = ch.base->ncol;
        if (k < 1 || k > kAdjointMaxK) invalid("the SVD adjoint supports 1 <= k <= 64");
        if (k > std::min(m, n)) invalid("k cannot exceed the smaller matrix dimension");
        const int kk = static_cast<int>(k);
        device_info();
        StreamUse su(stream);
        const cudaStream_t s = su.s;
        BlockOp op(ch, kk, s);
        DevBuf Ur(sizeof(double) * m * k), Vr(sizeof(double) * n * k), gUr(sizeof(double) * m * k),
            gVr(sizeof(double) * n * k), T1(sizeof(double) * k * k), T2(sizeof(double) * k * k),
            part(sizeof(double) * static_cast<int64_t>(gram_parts(std::max(m, n))) * k * k),
            dM(sizeof(double) * k * k), dS(sizeof(double) * k * k), dI(sizeof(double) * k);
        launch_to_rows(m, kk, U, m, Ur.as<double>(), s);
        launch_to_rows(n, kk, V, n, Vr.as<double>(), s);
        launch_to_rows(m, kk, gU, m, gUr.as<double>(), s);
        launch_to_rows(n, kk, gV, n, gVr.as<double>(), s);
        launch_gram(Ur.as<double>(), gUr.as<double>(), m, kk, part.as<double>(), T1.as<double>(), s);
        launch_gram(Vr.as<double>(), gVr.as<double>(), n, kk, part.as<double>(), T2.as<double>(), s);
        const std::vector<double> hS = fetch(S, k, s);
        const std::vector<double> hgS = gS ? fetch(gS, k, s) : std::vector<double>(k, 0.0);
        const std::vector<double> t1 = fetch(T1.as<double>(), k * k, s);
        const std::vector<double> t2 = fetch(T2.as<double>(), k * k, s);
        for (int64_t a = 0; a < k; ++a)
            if (!(hS[a] > 0)) throw Error(IRLBA_GB300_ERROR_NUMERICAL, "the SVD adjoint needs positive singular values");

        // M (k x k, row-major [a * k + b]) on the host: O(k^2).
        std::vector<double> M(k * k, 0.0), Sdiag(k * k, 0.0), inv2(k), shift(k);
        for (int64_t a = 0; a < k; ++a) {
            for (int64_t b = 0; b < k; ++b) {
                if (a == b) {
                    M[a * k + b] = hgS[a];
                    continue;
                }
                const double den = hS[b] * hS[b] - hS[a] * hS[a];
                if (den == 0)
                    throw Error(IRLBA_GB300_ERROR_NUMERICAL, "the SVD adjoint is undefined for repeated singular values");
                const double F = 1.0 / den;
                const double J = F * (t1[a * k + b] - t1[b * k + a]);
                const double K = F * (t2[a * k + b] - t2[b * k + a]);
                M[a * k + b] = J * hS[b] + hS[a] * K;
            }
            Sdiag[a * k + a] = hS[a];
            shift[a] = hS[a] * hS[a];
            inv2[a] = 1.0 / shift[a];
        }
        put(dM.as<double>(), M, s);
        put(dS.as<double>(), Sdiag, s);

        // Right-hand sides of the complement systems: (I - U U^T) gU, (I - V V^T) gV.
        // gU - U T1 with T1 = U^T gU, then one more projection pass.
        launch_block_update(m, kk, kk, Ur.as<double>(), k, T1.as<double>(), -1.0, gUr.as<double>(), k, nullptr, 1.0,
                            gUr.as<double>(), k, s);
        launch_block_update(n, kk, kk, Vr.as<double>(), k, T2.as<double>(), -1.0, gVr.as<double>(), k, nullptr, 1.0,
                            gVr.as<double>(), k, s);
        project_out(Ur.as<double>(), m, kk, gUr.as<double>(), T1.as<double>(), part.as<double>(), s);
        project_out(Vr.as<double>(), n, kk, gVr.as<double>(), T2.as<double>(), part.as<double>(), s);

        DevBuf Y(sizeof(double) * m * k), Zc(sizeof(double) * n * k);
        int its = 0;
        if (cg_tol < 0) {
            put(dI.as<double>(), inv2, s);
            launch_block_update(m, kk, kk, nullptr, k, nullptr, 0.0, gUr.as<double>(), k, dI.as<double>(), 1.0,
                                Y.as<double>(), k, s);
            launch_block_update(n, kk, kk, nullptr, k, nullptr, 0.0, gVr.as<double>(), k, dI.as<double>(), 1.0,
                                Zc.as<double>(), k, s);
        } else {
            const int maxit = cg_max_iter > 0 ? cg_max_iter : 1000;
            its += shifted_cg(op, true, Ur.as<double>(), gUr.as<double>(), shift, cg_tol, maxit, Y.as<double>(), s);
            its += shifted_cg(op, false, Vr.as<double>(), gVr.as<double>(), shift, cg_tol, maxit, Zc.as<double>(), s);
        }

        // Z1[:, :k] = U M + Y S + P_U A' Z;  Z1[:, k:] = U.
        DevBuf AZ(sizeof(double) * m * k), AtY(sizeof(double) * n * k);
        op.mul(Zc.as<double>(), AZ.as<double>());
        project_out(Ur.as<double>(), m, kk, AZ.as<double>(), T1.as<double>(), part.as<double>(), s);
        launch_block_update(m, kk, kk, Y.as<double>(), k, dS.as<double>(), 1.0, AZ.as<double>(), k, nullptr, 1.0,
                            AZ.as<double>(), k, s);
        launch_block_update(m, kk, kk, Ur.as<double>(), k, dM.as<double>(), 1.0, AZ.as<double>(), k, nullptr, 1.0, Z1,
                            2 * k, s);
        launch_block_update(m, kk, kk, nullptr, k, nullptr, 0.0, Ur.as<double>(), k, nullptr, 1.0, Z1 + k, 2 * k, s);
        // Z2[:, :k] = V;  Z2[:, k:] = Z S + P_V A'^T Y.
        op.adj(Y.as<double>(), AtY.as<double>());
        project_out(Vr.as<double>(), n, kk, AtY.as<double>(), T2.as<double>(), part.as<double>(), s);
        launch_block_update(n, kk, kk, nullptr, k, nullptr, 0.0, Vr.as<double>(), k, nullptr, 1.0, Z2, 2 * k, s);
        launch_block_update(n, kk, kk, Zc.as<double>(), k, dS.as<double>(), 1.0, AtY.as<double>(), k, nullptr, 1.0,
                            Z2 + k, 2 * k, s);
        CUDA_TRY(cudaStreamSynchronize(s));
        CUDA_TRY(cudaGetLastError());
        if (cg_iterations) *cg_iterations = its;
    });
}

irlba_gb300_status irlba_gb300_svd_adjoint_dense(int64_t m, int64_t n, int64_t k, const double* Z1, const double* Z2,
                                                 void* grad, int64_t ld, int32_t row_major,
                                                 irlba_gb300_value_type type, void* stream) {
    return guarded([&]() {
        if (m < 0 || n < 0 || k < 1 || k > kAdjointMaxK) invalid("invalid dimensions");
        if (!Z1 || !Z2 || !grad) invalid("Z1, Z2 and grad must not be NULL");
        if (ld < (row_major ? n : m)) invalid("leading dimension too small");
        device_info();
        StreamUse su(stream);
        launch_outer(m, n, static_cast<int>(2 * k), Z1, Z2, grad, ld, row_major, type == IRLBA_GB300_VALUE_F64, su.s);
        CUDA_TRY(cudaStreamSynchronize(su.s));
        CUDA_TRY(cudaGetLastError());
    });
}

irlba_gb300_status irlba_gb300_svd_adjoint_sparse(const irlba_gb300_matrix* matrix, int64_t k, const double* Z1,
                                                  const double* Z2, const int64_t* pointers, const int32_t* indices,
                                                  const void* values, irlba_gb300_value_type type,
                                                  int32_t column_major, int32_t statistics, void* grad_values,
                                                  void* stream) {
    return guarded([&]() {
        if (!matrix) invalid("matrix is NULL");
        if (!Z1 || !Z2 || !pointers || !indices || !values || !grad_values) invalid("array arguments must not be NULL");
        if (k < 1 || k > kAdjointMaxK) invalid("the SVD adjoint supports 1 <= k <= 64");
        const Chain ch = flatten(matrix);
        require_stored(ch.base, "the differentiation form");
        const int64_t m = ch.base->nrow, n = ch.base->ncol;
        if (ch.scale && !ch.scale_column)
            throw Error(IRLBA_GB300_ERROR_UNSUPPORTED, "the SVD adjoint supports column scaling only");
        if (statistics && ((ch.center && ch.center_outer) || (ch.scale && !ch.scale_divide)))
            throw Error(IRLBA_GB300_ERROR_UNSUPPORTED,
                        "statistics = 1 needs pca()'s chain: centring inside division by the column scale");
        if (statistics && ch.scale && m < 2) invalid("cannot scale with fewer than two observations");
        device_info();
        StreamUse su(stream);
        const cudaStream_t s = su.s;
        const int kk = static_cast<int>(2 * k);
        const int64_t nprimary = column_major ? n : m;

        // Per-column factors of the chain rule.
        DevBuf f, c, cmean, qf;
        if (ch.scale) {
            std::vector<double> hf(n);
            for (int64_t j = 0; j < n; ++j) hf[j] = ch.scale_divide ? 1.0 / (*ch.scale)[j] : (*ch.scale)[j];
            f = upload(hf.data(), hf.size());
        }
        if (statistics && (ch.center || ch.scale)) {
            DevBuf part(sizeof(double) * static_cast<int64_t>(gram_parts(std::max(m, n))) * 128),
                u(sizeof(double) * 128);
            // Column sums of Z1 Z2^T: (1^T Z1) . Z2_j, divided by m.
            launch_coldot(Z1, nullptr, nullptr, m, kk, part.as<double>(), u.as<double>(), s);
            if (ch.center) {
                cmean.alloc(sizeof(double) * std::max<int64_t>(n, 1));
                launch_rowdot(n, kk, Z2, nullptr, u.as<double>(), 1.0 / static_cast<double>(m), cmean.as<double>(), s);
                c = upload(ch.center->data(), ch.center->size());
            }
            if (ch.scale) {
                // q_j = sum_r (Z1 Z2^T)_rj A'_rj = Z2_j . (A'^T Z1)_j;  qf_j = q_j / ((m - 1) s_j).
                BlockOp op(ch, kk, s);
                DevBuf AtZ(sizeof(double) * std::max<int64_t>(n * kk, 1));
                op.adj(Z1, AtZ.as<double>());
                qf.alloc(sizeof(double) * std::max<int64_t>(n, 1));
                launch_rowdot(n, kk, Z2, AtZ.as<double>(), nullptr, 1.0 / static_cast<double>(m - 1), qf.as<double>(),
                              s);
                launch_scale_rows(n, 1, qf.as<double>(), op.svec.as<double>(), 1, qf.as<double>(), s);
                CUDA_TRY(cudaStreamSynchronize(s));
            }
        }
        launch_sddmm(nprimary, pointers, indices, values, type == IRLBA_GB300_VALUE_F64, column_major, Z1, Z2, kk,
                     f.as<double>(), cmean.as<double>(), c.as<double>(), qf.as<double>(), grad_values, s);
        CUDA_TRY(cudaStreamSynchronize(s));
        CUDA_TRY(cudaGetLastError());
    });
}

}  // extern "C"
