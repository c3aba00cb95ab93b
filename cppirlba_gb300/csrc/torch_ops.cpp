// libtorch autograd Functions over the engine's C ABI (differentiation form).
//
// TruncatedSvd: A (dense m x n, CUDA, FP32 or FP64) -> (U, S, V), the top-k SVD
// computed by the IRLBA engine (irlba::compute, compute.hpp:141-308; FP32 form
// for FP32 input). Backward: irlba_gb300_svd_adjoint_factors + _dense.
//
// SparsePcaSvd: the stored values of a compressed sparse matrix (nrow x ncol,
// the ParallelSparseMatrix layout) -> (U, S, V, center, scale) of pca()'s
// centred/scaled operator (pca.hpp:55-139: column means and standard
// deviations, CenteredMatrix then ScaledMatrix). Backward returns the gradient
// on the sparsity pattern (irlba_gb300_svd_adjoint_sparse), including the
// derivatives of the column statistics. center and scale are returned for
// reference and are not differentiable outputs.
//
// Both build the engine matrix from a host copy of the input (the C ABI
// ingests host arrays) in forward and again in backward.

#include <torch/extension.h>
#include <c10/cuda/CUDAStream.h>

#include <cmath>
#include <vector>

#include "../../include/irlba_gb300.h"

namespace {

using torch::Tensor;
using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

void check(irlba_gb300_status st) {
    TORCH_CHECK(st == IRLBA_GB300_OK, "irlba_gb300: ", irlba_gb300_last_error());
}

void* current_stream() { return static_cast<void*>(c10::cuda::getCurrentCUDAStream().stream()); }

// Owns up to three handles (base, centre, scale), destroyed outermost first.
struct Handles {
    irlba_gb300_matrix* h[3] = {nullptr, nullptr, nullptr};
    ~Handles() {
        for (int i = 2; i >= 0; --i)
            if (h[i]) irlba_gb300_matrix_destroy(h[i]);
    }
    irlba_gb300_matrix* top() const { return h[2] ? h[2] : (h[1] ? h[1] : h[0]); }
};

irlba_gb300_options make_options(double tol, int64_t seed) {
    irlba_gb300_options o;
    irlba_gb300_default_options(&o);
    o.convergence_tolerance = tol;
    o.seed = static_cast<uint64_t>(seed);
    return o;
}

irlba_gb300_value_type value_type_of(const Tensor& t) {
    return t.scalar_type() == torch::kFloat64 ? IRLBA_GB300_VALUE_F64 : IRLBA_GB300_VALUE_F32;
}

irlba_gb300_form form_of(const Tensor& t) {
    return t.scalar_type() == torch::kFloat64 ? IRLBA_GB300_FORM_FP64 : IRLBA_GB300_FORM_FP32_FP64STEPS;
}

void dense_handle(const Tensor& A, Handles& hs) {
    Tensor h = A.detach().to(torch::kCPU).contiguous();
    check(irlba_gb300_matrix_create_dense(A.size(0), A.size(1), h.data_ptr(), value_type_of(A), A.size(1), 1,
                                          form_of(A), &hs.h[0]));
}

// pca()'s column statistics (pca.hpp:85-109) of a compressed matrix, FP64.
void column_stats(const Tensor& vals, const Tensor& ptr, const Tensor& idx, int64_t nrow, int64_t ncol,
                  bool column_major, bool center, bool scale, std::vector<double>& c, std::vector<double>& s) {
    Tensor v = vals.detach().to(torch::kCPU).to(torch::kFloat64).contiguous();
    const double* x = v.data_ptr<double>();
    const int64_t* p = ptr.data_ptr<int64_t>();
    const int32_t* ix = idx.data_ptr<int32_t>();
    const int64_t primary = column_major ? ncol : nrow;
    std::vector<double> sum(ncol, 0.0), cnt(ncol, 0.0);
    for (int64_t q = 0; q < primary; ++q)
        for (int64_t e = p[q]; e < p[q + 1]; ++e) {
            const int64_t j = column_major ? q : ix[e];
            sum[j] += x[e];
            cnt[j] += 1;
        }
    c.assign(ncol, 0.0);
    if (center)
        for (int64_t j = 0; j < ncol; ++j) c[j] = sum[j] / static_cast<double>(nrow);
    if (scale) {
        std::vector<double> ss(ncol, 0.0);
        for (int64_t q = 0; q < primary; ++q)
            for (int64_t e = p[q]; e < p[q + 1]; ++e) {
                const int64_t j = column_major ? q : ix[e];
                const double d = x[e] - c[j];
                ss[j] += d * d;
            }
        s.assign(ncol, 1.0);
        for (int64_t j = 0; j < ncol; ++j) {
            const double var = ss[j] + (static_cast<double>(nrow) - cnt[j]) * c[j] * c[j];
            s[j] = var != 0 ? std::sqrt(var / static_cast<double>(nrow - 1)) : 1.0;
        }
    }
}

void sparse_handles(const Tensor& vals, const Tensor& ptr, const Tensor& idx, int64_t nrow, int64_t ncol,
                    bool column_major, bool center, bool scale, Handles& hs, std::vector<double>& c,
                    std::vector<double>& s) {
    Tensor vh = vals.detach().to(torch::kCPU).contiguous();
    check(irlba_gb300_matrix_create_sparse(nrow, ncol, vh.data_ptr(), value_type_of(vals), idx.data_ptr<int32_t>(),
                                           ptr.data_ptr<int64_t>(), column_major ? 1 : 0, form_of(vals), &hs.h[0]));
    column_stats(vals, ptr, idx, nrow, ncol, column_major, center, scale, c, s);
    if (center) check(irlba_gb300_matrix_center(hs.h[0], c.data(), &hs.h[1]));
    if (scale) check(irlba_gb300_matrix_scale(hs.top(), s.data(), 1, 1, &hs.h[2]));
}

// Top-k SVD of the operator into FP64 device tensors Ut (k x m), S (k), Vt (k x n).
void svd_device(irlba_gb300_matrix* top, int64_t m, int64_t n, int64_t k, double tol, int64_t seed,
                const torch::TensorOptions& o64, Tensor& Ut, Tensor& S, Tensor& Vt) {
    Ut = torch::empty({k, m}, o64);
    Vt = torch::empty({k, n}, o64);
    S = torch::empty({k}, o64);
    irlba_gb300_options o = make_options(tol, seed);
    int64_t num = 0;
    int32_t conv = 0, iters = 0;
    check(irlba_gb300_compute_device(top, k, &o, Ut.data_ptr<double>(), Vt.data_ptr<double>(), S.data_ptr<double>(),
                                     &num, &conv, &iters, nullptr, current_stream()));
    TORCH_CHECK(num == k, "irlba_gb300: fewer singular values than requested");
}

// Z1 (m x 2k), Z2 (n x 2k) of the adjoint.
void factors(irlba_gb300_matrix* top, int64_t m, int64_t n, int64_t k, const Tensor& Ut, const Tensor& S,
             const Tensor& Vt, const variable_list& grads, double cg_tol, int64_t cg_max, Tensor& Z1, Tensor& Z2) {
    auto o64 = Ut.options();
    Tensor gUt, gS, gVt;
    if (grads[0].defined()) gUt = grads[0].to(torch::kFloat64).t().contiguous();
    if (grads[1].defined()) gS = grads[1].to(torch::kFloat64).contiguous();
    if (grads[2].defined()) gVt = grads[2].to(torch::kFloat64).t().contiguous();
    Z1 = torch::empty({m, 2 * k}, o64);
    Z2 = torch::empty({n, 2 * k}, o64);
    int32_t its = 0;
    check(irlba_gb300_svd_adjoint_factors(top, k, Ut.data_ptr<double>(), S.data_ptr<double>(), Vt.data_ptr<double>(),
                                          gUt.defined() ? gUt.data_ptr<double>() : nullptr,
                                          gS.defined() ? gS.data_ptr<double>() : nullptr,
                                          gVt.defined() ? gVt.data_ptr<double>() : nullptr, cg_tol,
                                          static_cast<int32_t>(cg_max), Z1.data_ptr<double>(), Z2.data_ptr<double>(),
                                          &its, current_stream()));
}

class TruncatedSvd : public torch::autograd::Function<TruncatedSvd> {
public:
    static variable_list forward(AutogradContext* ctx, Tensor A, int64_t k, double tol, int64_t seed, double cg_tol,
                                 int64_t cg_max) {
        TORCH_CHECK(A.dim() == 2, "A must be a matrix");
        TORCH_CHECK(A.is_cuda(), "A must be a CUDA tensor");
        TORCH_CHECK(A.scalar_type() == torch::kFloat32 || A.scalar_type() == torch::kFloat64, "A must be FP32 or FP64");
        const int64_t m = A.size(0), n = A.size(1);
        Handles hs;
        dense_handle(A, hs);
        Tensor Ut, S, Vt;
        svd_device(hs.top(), m, n, k, tol, seed, A.options().dtype(torch::kFloat64), Ut, S, Vt);
        ctx->save_for_backward({A, Ut, S, Vt});
        ctx->saved_data["k"] = k;
        ctx->saved_data["cg_tol"] = cg_tol;
        ctx->saved_data["cg_max"] = cg_max;
        const auto dt = A.scalar_type();
        return {Ut.t().contiguous().to(dt), S.to(dt), Vt.t().contiguous().to(dt)};
    }

    static variable_list backward(AutogradContext* ctx, variable_list grads) {
        auto saved = ctx->get_saved_variables();
        Tensor A = saved[0], Ut = saved[1], S = saved[2], Vt = saved[3];
        const int64_t k = ctx->saved_data["k"].toInt();
        const int64_t m = A.size(0), n = A.size(1);
        Handles hs;
        dense_handle(A, hs);
        Tensor Z1, Z2;
        factors(hs.top(), m, n, k, Ut, S, Vt, grads, ctx->saved_data["cg_tol"].toDouble(),
                ctx->saved_data["cg_max"].toInt(), Z1, Z2);
        Tensor gA = torch::empty({m, n}, A.options());
        check(irlba_gb300_svd_adjoint_dense(m, n, k, Z1.data_ptr<double>(), Z2.data_ptr<double>(), gA.data_ptr(), n, 1,
                                            value_type_of(A), current_stream()));
        return {gA, Tensor(), Tensor(), Tensor(), Tensor(), Tensor()};
    }
};

class SparsePcaSvd : public torch::autograd::Function<SparsePcaSvd> {
public:
    static variable_list forward(AutogradContext* ctx, Tensor values, Tensor ptr, Tensor idx, int64_t nrow,
                                 int64_t ncol, bool column_major, bool center, bool scale, int64_t k, double tol,
                                 int64_t seed, double cg_tol, int64_t cg_max, bool statistics) {
        TORCH_CHECK(values.dim() == 1, "values must be a vector");
        TORCH_CHECK(values.scalar_type() == torch::kFloat32 || values.scalar_type() == torch::kFloat64,
                    "values must be FP32 or FP64");
        TORCH_CHECK(ptr.device().is_cpu() && ptr.scalar_type() == torch::kInt64 && ptr.is_contiguous(),
                    "pointers must be a contiguous int64 CPU tensor");
        TORCH_CHECK(idx.device().is_cpu() && idx.scalar_type() == torch::kInt32 && idx.is_contiguous(),
                    "indices must be a contiguous int32 CPU tensor");
        Handles hs;
        std::vector<double> c, s;
        sparse_handles(values, ptr, idx, nrow, ncol, column_major, center, scale, hs, c, s);
        auto o64 = torch::TensorOptions().dtype(torch::kFloat64).device(torch::kCUDA, c10::cuda::current_device());
        Tensor Ut, S, Vt;
        svd_device(hs.top(), nrow, ncol, k, tol, seed, o64, Ut, S, Vt);
        ctx->save_for_backward({values, ptr, idx, Ut, S, Vt});
        ctx->saved_data["nrow"] = nrow;
        ctx->saved_data["ncol"] = ncol;
        ctx->saved_data["column_major"] = column_major;
        ctx->saved_data["center"] = center;
        ctx->saved_data["scale"] = scale;
        ctx->saved_data["k"] = k;
        ctx->saved_data["cg_tol"] = cg_tol;
        ctx->saved_data["cg_max"] = cg_max;
        ctx->saved_data["statistics"] = statistics;
        const auto dt = values.scalar_type();
        Tensor cvec = torch::from_blob(c.data(), {ncol}, torch::kFloat64).clone().to(o64).to(dt);
        Tensor svec = scale ? torch::from_blob(s.data(), {ncol}, torch::kFloat64).clone().to(o64).to(dt)
                            : torch::ones({ncol}, o64.dtype(dt));
        ctx->mark_non_differentiable({cvec, svec});
        return {Ut.t().contiguous().to(dt), S.to(dt), Vt.t().contiguous().to(dt), cvec, svec};
    }

    static variable_list backward(AutogradContext* ctx, variable_list grads) {
        auto saved = ctx->get_saved_variables();
        Tensor values = saved[0], ptr = saved[1], idx = saved[2], Ut = saved[3], S = saved[4], Vt = saved[5];
        const int64_t nrow = ctx->saved_data["nrow"].toInt(), ncol = ctx->saved_data["ncol"].toInt();
        const bool column_major = ctx->saved_data["column_major"].toBool();
        const int64_t k = ctx->saved_data["k"].toInt();
        Handles hs;
        std::vector<double> c, s;
        sparse_handles(values, ptr, idx, nrow, ncol, column_major, ctx->saved_data["center"].toBool(),
                       ctx->saved_data["scale"].toBool(), hs, c, s);
        Tensor Z1, Z2;
        factors(hs.top(), nrow, ncol, k, Ut, S, Vt, grads, ctx->saved_data["cg_tol"].toDouble(),
                ctx->saved_data["cg_max"].toInt(), Z1, Z2);
        auto dev = Ut.device();
        Tensor pd = ptr.to(dev), id = idx.to(dev), vd = values.detach().to(dev).contiguous();
        Tensor g = torch::empty_like(vd);
        check(irlba_gb300_svd_adjoint_sparse(hs.top(), k, Z1.data_ptr<double>(), Z2.data_ptr<double>(),
                                             pd.data_ptr<int64_t>(), id.data_ptr<int32_t>(), vd.data_ptr(),
                                             value_type_of(values), column_major ? 1 : 0,
                                             ctx->saved_data["statistics"].toBool() ? 1 : 0, g.data_ptr(),
                                             current_stream()));
        variable_list out(14);
        out[0] = g.to(values.device());
        return out;
    }
};

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.doc() = "libtorch autograd Functions of the GB300 IRLBA engine (truncated-SVD adjoint)";
    m.def(
        "truncated_svd",
        [](Tensor A, int64_t k, double tol, int64_t seed, double cg_tol, int64_t cg_max) {
            auto out = TruncatedSvd::apply(A, k, tol, seed, cg_tol, cg_max);
            return std::make_tuple(out[0], out[1], out[2]);
        },
        "Top-k SVD (U, S, V) of a dense CUDA matrix with a truncated-SVD backward");
    m.def(
        "sparse_pca_svd",
        [](Tensor values, Tensor ptr, Tensor idx, int64_t nrow, int64_t ncol, bool column_major, bool center,
           bool scale, int64_t k, double tol, int64_t seed, double cg_tol, int64_t cg_max, bool statistics) {
            auto out = SparsePcaSvd::apply(values, ptr, idx, nrow, ncol, column_major, center, scale, k, tol, seed,
                                           cg_tol, cg_max, statistics);
            return std::make_tuple(out[0], out[1], out[2], out[3], out[4]);
        },
        "Top-k SVD of pca()'s centred/scaled sparse operator with a backward on the stored values");
}
