// Eigen-style sparse input to the header-style drop-in, and the reference's
// default template types (Options, compute, compute_simple, pca): the conversion of
// compressed and uncompressed storage (column- and row-major) into the C ABI's
// compressed arrays, checked on the host. SimpleMatrix / compute_simple / pca
// over a sparse matrix are instantiated too (they need a GPU to run, so the
// program only calls them when given the argument "gpu").
//
// SparseStore mimics the storage members Eigen documents for
// Eigen::SparseMatrix (valuePtr, innerIndexPtr, outerIndexPtr, innerNonZeroPtr,
// IsRowMajor); Eigen itself is not needed.
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

struct Vec {
    std::vector<double> v;
    double* data() { return v.data(); }
    const double* data() const { return v.data(); }
    std::ptrdiff_t size() const { return static_cast<std::ptrdiff_t>(v.size()); }
    void resize(std::ptrdiff_t n) { v.resize(n); }
};

struct Mat {
    std::ptrdiff_t nr = 0, nc = 0;
    std::vector<double> v;
    double* data() { return v.data(); }
    const double* data() const { return v.data(); }
    std::ptrdiff_t rows() const { return nr; }
    std::ptrdiff_t cols() const { return nc; }
    void resize(std::ptrdiff_t r, std::ptrdiff_t c) { nr = r; nc = c; v.assign(r * c, 0.0); }
    double& operator()(std::ptrdiff_t r, std::ptrdiff_t c) { return v[c * nr + r]; }
};

// The reference's callers rely on Eigen::VectorXd / Eigen::MatrixXd being the
// default types of Options, compute(), compute_simple() and pca(); here the
// stand-in types play that part.
#define IRLBA_GB300_DEFAULT_VECTOR Vec
#define IRLBA_GB300_DEFAULT_MATRIX Mat
#include "irlba_gb300/irlba.hpp"

template <bool RowMajor, typename Scalar>
struct SparseStore {
    static constexpr bool IsRowMajor = RowMajor;
    std::ptrdiff_t nr = 0, nc = 0;
    std::vector<int> outer, inner, nonzeros;  // nonzeros empty = compressed mode
    std::vector<Scalar> values;
    std::ptrdiff_t rows() const { return nr; }
    std::ptrdiff_t cols() const { return nc; }
    const Scalar* valuePtr() const { return values.data(); }
    const int* innerIndexPtr() const { return inner.data(); }
    const int* outerIndexPtr() const { return outer.data(); }
    const int* innerNonZeroPtr() const { return nonzeros.empty() ? nullptr : nonzeros.data(); }
};

// Dense 4 x 5 matrix with entry (r, c) = 10 r + c + 1 where (r + 2 c) % 3 == 0.
static double entry(int r, int c) { return ((r + 2 * c) % 3 == 0) ? 10.0 * r + c + 1 : 0.0; }

template <bool RowMajor, typename Scalar>
static SparseStore<RowMajor, Scalar> build(bool compressed) {
    SparseStore<RowMajor, Scalar> s;
    s.nr = 4;
    s.nc = 5;
    const int outer = RowMajor ? 4 : 5, inner = RowMajor ? 5 : 4;
    s.outer.push_back(0);
    for (int o = 0; o < outer; ++o) {
        int n = 0;
        for (int i = 0; i < inner; ++i) {
            const double v = RowMajor ? entry(o, i) : entry(i, o);
            if (v != 0.0) {
                s.inner.push_back(i);
                s.values.push_back(static_cast<Scalar>(v));
                ++n;
            }
        }
        if (!compressed) {
            // Uncompressed mode: each outer vector keeps two slots of free space.
            s.nonzeros.push_back(n);
            s.inner.push_back(-1);
            s.inner.push_back(-1);
            s.values.push_back(static_cast<Scalar>(-999));
            s.values.push_back(static_cast<Scalar>(-999));
        }
        s.outer.push_back(static_cast<int>(s.inner.size()));
    }
    return s;
}

template <bool RowMajor, typename Scalar>
static void check(bool compressed) {
    const auto s = build<RowMajor, Scalar>(compressed);
    std::vector<int64_t> ptr;
    std::vector<int32_t> idx;
    std::vector<double> val;
    irlba::gpu::compressed_arrays(s, ptr, idx, val);
    const int outer = RowMajor ? 4 : 5;
    if (static_cast<int>(ptr.size()) != outer + 1 || ptr[0] != 0) throw std::runtime_error("pointer length");
    for (int o = 0; o < outer; ++o)
        for (int64_t k = ptr[o]; k < ptr[o + 1]; ++k) {
            const int r = RowMajor ? o : idx[k], c = RowMajor ? idx[k] : o;
            if (k > ptr[o] && idx[k] <= idx[k - 1]) throw std::runtime_error("indices not increasing");
            if (val[k] != entry(r, c) || val[k] == 0.0) throw std::runtime_error("wrong value");
        }
    int64_t expected = 0;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 5; ++c) expected += entry(r, c) != 0.0;
    if (ptr[outer] != expected) throw std::runtime_error("entry count");
}

// Instantiated only: needs a GPU to run.
// Written as the reference's own tests call these (default template types).
static void run_on_gpu() {
    const auto s = build<false, double>(true);
    irlba::Options opt;
    irlba::SimpleMatrix<Vec, Mat, const SparseStore<false, double>*> wrapped(&s);
    auto res = irlba::compute(wrapped, 2, opt);
    auto res2 = irlba::compute_simple(s, 2, opt);
    auto pcs = irlba::pca(s, true, true, 2, opt);
    std::printf("%g %g %g\n", res.D.v[0], res2.D.v[0], pcs.variances.v[0]);
}

int main(int argc, char** argv) {
    check<false, double>(true);
    check<false, double>(false);
    check<true, double>(true);
    check<true, double>(false);
    check<false, float>(true);
    check<true, float>(false);
    if (argc > 1 && std::strcmp(argv[1], "gpu") == 0) run_on_gpu();
    std::printf("ok\n");
    return 0;
}
