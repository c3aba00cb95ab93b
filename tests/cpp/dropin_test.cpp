// Exercises the header-style drop-in (include/irlba_gb300/irlba.hpp) the way a
// CppIrlba user would: irlba::compute / compute_simple / pca over SimpleMatrix,
// ParallelSparseMatrix, the Centered/Scaled decorators, a user's own Matrix
// subclass and a gpu::DeviceMatrix. Prints inputs and
// outputs as JSON for tests/test_gpu_dropin.py to check against the oracle.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "irlba_gb300/irlba.hpp"

// Minimal column-major dense types with the Eigen members the drop-in uses.
struct Vec {
    std::vector<double> v;
    Vec() {}
    explicit Vec(std::ptrdiff_t n) : v(n) {}
    double* data() { return v.data(); }
    const double* data() const { return v.data(); }
    std::ptrdiff_t size() const { return static_cast<std::ptrdiff_t>(v.size()); }
    void resize(std::ptrdiff_t n) { v.resize(n); }
    double& operator[](std::ptrdiff_t i) { return v[i]; }
};

struct Mat {
    std::ptrdiff_t nr = 0, nc = 0;
    std::vector<double> v;
    Mat() {}
    Mat(std::ptrdiff_t r, std::ptrdiff_t c) : nr(r), nc(c), v(r * c) {}
    double* data() { return v.data(); }
    const double* data() const { return v.data(); }
    std::ptrdiff_t rows() const { return nr; }
    std::ptrdiff_t cols() const { return nc; }
    void resize(std::ptrdiff_t r, std::ptrdiff_t c) { nr = r; nc = c; v.assign(r * c, 0.0); }
    double& operator()(std::ptrdiff_t r, std::ptrdiff_t c) { return v[c * nr + r]; }
    double operator()(std::ptrdiff_t r, std::ptrdiff_t c) const { return v[c * nr + r]; }
};

// A column-major view with an outer stride larger than its rows, like an Eigen
// Map<MatrixXd, 0, OuterStride<>> or a Block of a larger matrix.
struct StridedView {
    const double* p = nullptr;
    std::ptrdiff_t nr = 0, nc = 0, ld = 0;
    const double* data() const { return p; }
    std::ptrdiff_t rows() const { return nr; }
    std::ptrdiff_t cols() const { return nc; }
    std::ptrdiff_t outerStride() const { return ld; }
    std::ptrdiff_t innerStride() const { return 1; }
    double operator()(std::ptrdiff_t r, std::ptrdiff_t c) const { return p[c * ld + r]; }
};

// A caller's own Matrix subclass (Matrix/interface.hpp:141-223) with products
// written by hand on the host; `fail` makes its multiply throw.
class UserDense final : public irlba::Matrix<Vec, Mat> {
public:
    UserDense(const Mat* a, bool fail = false) : my_a(a), my_fail(fail) {}
    irlba::Index rows() const { return my_a->rows(); }
    irlba::Index cols() const { return my_a->cols(); }

    struct Mul final : public irlba::Workspace<Vec> {
        const Mat* a;
        bool fail;
        Mul(const Mat* a_, bool f) : a(a_), fail(f) {}
        void multiply(const Vec& right, Vec& out) {
            if (fail) throw std::runtime_error("residual model is not fitted");
            for (std::ptrdiff_t r = 0; r < a->rows(); ++r) {
                double s = 0;
                for (std::ptrdiff_t c = 0; c < a->cols(); ++c) s += (*a)(r, c) * right.v[c];
                out.v[r] = s;
            }
        }
    };
    struct Adj final : public irlba::AdjointWorkspace<Vec> {
        const Mat* a;
        explicit Adj(const Mat* a_) : a(a_) {}
        void multiply(const Vec& right, Vec& out) {
            for (std::ptrdiff_t c = 0; c < a->cols(); ++c) {
                double s = 0;
                for (std::ptrdiff_t r = 0; r < a->rows(); ++r) s += (*a)(r, c) * right.v[r];
                out.v[c] = s;
            }
        }
    };
    struct Real final : public irlba::RealizeWorkspace<Mat> {
        const Mat* a;
        explicit Real(const Mat* a_) : a(a_) {}
        const Mat& realize(Mat&) { return *a; }
    };
    std::unique_ptr<irlba::Workspace<Vec>> new_workspace() const { return std::make_unique<Mul>(my_a, my_fail); }
    std::unique_ptr<irlba::AdjointWorkspace<Vec>> new_adjoint_workspace() const { return std::make_unique<Adj>(my_a); }
    std::unique_ptr<irlba::RealizeWorkspace<Mat>> new_realize_workspace() const { return std::make_unique<Real>(my_a); }

private:
    const Mat* my_a;
    bool my_fail;
};

// Options with the first `n` entries of `init` as the start vector.
static irlba::Options<Vec> opt_block(const irlba::Options<Vec>& base, const Vec& init, std::ptrdiff_t n = 50) {
    irlba::Options<Vec> o = base;
    Vec v(n);
    for (std::ptrdiff_t i = 0; i < n; ++i) v[i] = init.v[i];
    o.initial = v;
    return o;
}

static uint64_t lcg = 88172645463325252ull;
static double next_normal() {
    auto u = [&]() {
        lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
        return ((lcg >> 11) + 1.0) * (1.0 / 9007199254740992.0);
    };
    const double a = u(), b = u();
    return std::sqrt(-2.0 * std::log(a)) * std::cos(6.283185307179586 * b);
}

static void dump_vec(const char* name, const double* p, std::ptrdiff_t n, bool comma = true) {
    std::printf("\"%s\": [", name);
    for (std::ptrdiff_t i = 0; i < n; ++i) std::printf("%s%.17g", i ? ", " : "", p[i]);
    std::printf("]%s\n", comma ? "," : "");
}

int main() {
    const std::ptrdiff_t nr = 120, nc = 70;
    Mat A(nr, nc);
    for (auto& x : A.v) x = next_normal();
    Vec init(nc);
    for (auto& x : init.v) x = next_normal();

    irlba::Options<Vec> opt;
    opt.initial = init;
    std::printf("{\n");
    dump_vec("A_colmajor", A.data(), nr * nc);
    dump_vec("init", init.data(), nc);

    // compute over SimpleMatrix (compute.hpp:141) and compute_simple (compute.hpp:426).
    irlba::SimpleMatrix<Vec, Mat, const Mat*> simple(&A);
    auto res = irlba::compute<Mat, Vec>(simple, 6, opt);
    dump_vec("compute_D", res.D.data(), res.D.size());
    dump_vec("compute_U0", res.U.data(), nr);
    std::printf("\"compute_iterations\": %d, \"compute_converged\": %d,\n", res.iterations, (int)res.converged);
    auto res2 = irlba::compute_simple<Mat, Vec>(A, 6, opt);
    dump_vec("compute_simple_D", res2.D.data(), res2.D.size());

    // pca over a dense matrix (pca.hpp:197).
    auto p = irlba::pca<Mat, Vec>(A, true, true, 5, opt);
    dump_vec("pca_variances", p.variances.data(), p.variances.size());
    std::printf("\"pca_iterations\": %d,\n", p.iterations);

    // ParallelSparseMatrix (CSC) with a CenteredMatrix and ScaledMatrix chain.
    std::vector<double> x;
    std::vector<int> i;
    std::vector<std::size_t> ptr(1, 0);
    for (std::ptrdiff_t c = 0; c < nc; ++c) {
        for (std::ptrdiff_t r = 0; r < nr; ++r)
            if (((r * 7 + c * 13) % 5) == 0) {
                x.push_back(A(r, c));
                i.push_back(static_cast<int>(r));
            }
        ptr.push_back(x.size());
    }
    irlba::ParallelSparseMatrix<Vec, Mat, std::vector<double>, std::vector<int>, std::vector<std::size_t>> sp(
        nr, nc, x, i, ptr, true, 4);
    Vec center(nc), scale(nc);
    for (std::ptrdiff_t c = 0; c < nc; ++c) {
        center[c] = 0.01 * c;
        scale[c] = 1.0 + 0.02 * c;
    }
    irlba::CenteredMatrix<Vec, Mat> cen(&sp, &center);
    irlba::ScaledMatrix<Vec, Mat> scl(&cen, &scale, true, true);
    auto res3 = irlba::compute<Mat, Vec>(scl, 4, opt);
    dump_vec("chain_D", res3.D.data(), res3.D.size());
    std::printf("\"chain_iterations\": %d,\n", res3.iterations);
    dump_vec("sparse_x", x.data(), x.size());
    std::vector<double> id(i.begin(), i.end()), pd(ptr.begin(), ptr.end());
    dump_vec("sparse_i", id.data(), id.size());
    dump_vec("sparse_p", pd.data(), pd.size());
    dump_vec("center", center.data(), nc);
    dump_vec("scale", scale.data(), nc);

    // The decorators read the caller's vectors when they are used, as the
    // reference's pointers do: change the centre and scale after construction.
    for (std::ptrdiff_t c = 0; c < nc; ++c) {
        center[c] = 0.02 * c - 0.3;
        scale[c] = 2.0 - 0.01 * c;
    }
    auto res3b = irlba::compute<Mat, Vec>(scl, 4, opt);
    dump_vec("chain_changed_D", res3b.D.data(), res3b.D.size());
    std::printf("\"chain_changed_iterations\": %d,\n", res3b.iterations);
    dump_vec("center_changed", center.data(), nc);
    dump_vec("scale_changed", scale.data(), nc);
    for (std::ptrdiff_t c = 0; c < nc; ++c) {   // back to the vectors dumped above
        center[c] = 0.01 * c;
        scale[c] = 1.0 + 0.02 * c;
    }

    // Dense input held with an outer stride (the top-left 100 x 50 block of A).
    StridedView view{A.data(), 100, 50, nr};
    irlba::SimpleMatrix<Vec, Mat, const StridedView*> strided(&view);
    auto res7 = irlba::compute<Mat, Vec>(strided, 5, opt_block(opt, init));
    dump_vec("strided_D", res7.D.data(), res7.D.size());
    std::printf("\"strided_iterations\": %d,\n", res7.iterations);

    // Workspace multiply through the plug-in surface (interface.hpp:49, :87).
    auto w = scl.new_workspace();
    Vec out(nr);
    w->multiply(init, out);
    dump_vec("chain_multiply_init", out.data(), nr);

    // A caller's own Matrix subclass: the loop on the device, products on the host.
    UserDense user(&A);
    auto res4 = irlba::compute<Mat, Vec>(user, 6, opt);
    dump_vec("user_D", res4.D.data(), res4.D.size());
    std::printf("\"user_iterations\": %d,\n", res4.iterations);
    irlba::CenteredMatrix<Vec, Mat> ucen(&user, &center);
    auto res5 = irlba::compute<Mat, Vec>(ucen, 4, opt);
    dump_vec("user_centered_D", res5.D.data(), res5.D.size());
    std::printf("\"user_centered_iterations\": %d,\n", res5.iterations);
    std::string user_msg;
    try {
        UserDense broken(&A, true);
        irlba::compute<Mat, Vec>(broken, 6, opt);
    } catch (const std::exception& e) {
        user_msg = e.what();
    }
    std::printf("\"user_error_message\": \"%s\",\n", user_msg.c_str());

    // A matrix whose products are device code on the engine's stream (here the
    // engine's own SpMV of the sparse matrix, through its raw entry point).
    const irlba_gb300_matrix* sph = sp.gpu_handle();
    irlba::gpu::DeviceMatrix<Vec, Mat> dev(nr, nc, [sph](bool adjoint, const void* in, void* out, void* stream) {
        irlba::gpu::check(irlba_gb300_spmv_device(sph, adjoint ? 1 : 0, in, out, stream));
    });
    auto res6 = irlba::compute<Mat, Vec>(dev, 4, opt);
    dump_vec("device_D", res6.D.data(), res6.D.size());
    std::printf("\"device_iterations\": %d,\n", res6.iterations);

    // An error with the reference's message (compute.hpp:156).
    std::string msg;
    try {
        irlba::compute<Mat, Vec>(simple, 1000, opt);
    } catch (const std::exception& e) {
        msg = e.what();
    }
    std::printf("\"error_message\": \"%s\"\n}\n", msg.c_str());
    return 0;
}
