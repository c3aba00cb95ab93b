// Header-style C++ drop-in for CppIrlba's IRLBA entry points, backed by the
// GB300 engine through the C ABI in irlba_gb300.h.
//
// Same names and meanings as CppIrlba (include/irlba/*.hpp):
//   irlba::Options                      Options.hpp:19-83
//   irlba::Matrix, Workspace,
//     AdjointWorkspace, RealizeWorkspace Matrix/interface.hpp:23-223
//   irlba::SimpleMatrix                 Matrix/simple.hpp:124-178 (dense or Eigen sparse input)
//   irlba::ParallelSparseMatrix         Matrix/sparse.hpp:438-589
//   irlba::CenteredMatrix               Matrix/centered.hpp:139-204
//   irlba::ScaledMatrix                 Matrix/scaled.hpp:195-268
//   irlba::compute, compute_simple,
//     Results                           compute.hpp:141-433
//   irlba::pca, PcaResults              pca.hpp:55-204
//   irlba::parallelize, EigenThreadScope parallel.hpp:32-106
// Vector and matrix types are template parameters as in the reference; they
// need data(), size() / rows(), cols() and resize(), which Eigen's dense types
// provide. Matrices are column-major (a type with a static `IsRowMajor` true is
// read as row-major). Errors are std::runtime_error with the reference's
// messages. The arithmetic form (plain FP64 or FP32 with FP64 steps) is an
// engine setting outside Options: irlba::gpu::set_form().
#ifndef IRLBA_GB300_IRLBA_HPP
#define IRLBA_GB300_IRLBA_HPP

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <functional>
#include <memory>
#include <optional>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

#include "../irlba_gb300.h"

// Default vector and matrix types of Options, compute(), compute_simple() and
// pca(), as in the reference (Options.hpp:19, compute.hpp:403,426, pca.hpp:197:
// Eigen::VectorXd and Eigen::MatrixXd). With Eigen on the include path those are
// the defaults here too; a caller may instead define both
// IRLBA_GB300_DEFAULT_VECTOR and IRLBA_GB300_DEFAULT_MATRIX before including
// this header. Without either, the types must be given explicitly.
#if !defined(IRLBA_GB300_DEFAULT_VECTOR) && defined(__has_include)
#if __has_include(<Eigen/Dense>)
#include <Eigen/Dense>
#define IRLBA_GB300_DEFAULT_VECTOR Eigen::VectorXd
#define IRLBA_GB300_DEFAULT_MATRIX Eigen::MatrixXd
#endif
#endif
#if defined(IRLBA_GB300_DEFAULT_VECTOR) && defined(IRLBA_GB300_DEFAULT_MATRIX)
#define IRLBA_GB300_VECTOR_DEFAULT_ARG = IRLBA_GB300_DEFAULT_VECTOR
#define IRLBA_GB300_MATRIX_DEFAULT_ARG = IRLBA_GB300_DEFAULT_MATRIX
#else
#define IRLBA_GB300_VECTOR_DEFAULT_ARG
#define IRLBA_GB300_MATRIX_DEFAULT_ARG
#endif

namespace irlba {

typedef std::ptrdiff_t Index;

namespace gpu {

inline irlba_gb300_form& default_form() {
    static thread_local irlba_gb300_form form = IRLBA_GB300_FORM_FP64;
    return form;
}

// Arithmetic form used by matrices constructed afterwards on this thread.
inline void set_form(irlba_gb300_form form) { default_form() = form; }

inline void check(irlba_gb300_status st) {
    if (st != IRLBA_GB300_OK) throw std::runtime_error(irlba_gb300_last_error());
}

struct HandleDeleter {
    void operator()(irlba_gb300_matrix* h) const {
        if (h) irlba_gb300_matrix_destroy(h);
    }
};
typedef std::shared_ptr<irlba_gb300_matrix> Handle;

inline Handle adopt(irlba_gb300_matrix* h) { return Handle(h, HandleDeleter()); }

template <class T, class = void>
struct is_row_major : std::false_type {};
template <class T>
struct is_row_major<T, std::void_t<decltype(T::IsRowMajor)>> : std::integral_constant<bool, static_cast<bool>(T::IsRowMajor)> {};

template <class P>
auto& deref(const P& p) { return *p; }

// Dense types with explicit strides (Eigen's Map<..., OuterStride<>>, Block,
// Ref): the storage of column (or row) j starts at data() + j * outerStride().
template <class T, class = void>
struct has_strides : std::false_type {};
template <class T>
struct has_strides<T, std::void_t<decltype(std::declval<const T&>().outerStride()),
                                  decltype(std::declval<const T&>().innerStride())>> : std::true_type {};

// Engine handle of a matrix, or NULL for one the engine cannot run directly
// (a user's own Matrix subclass, or a type without gpu_handle()).
template <class M, class = void>
struct has_gpu_handle : std::false_type {};
template <class M>
struct has_gpu_handle<M, std::void_t<decltype(std::declval<const M&>().gpu_handle())>> : std::true_type {};
template <class M>
const irlba_gb300_matrix* handle_of(const M& m) {
    if constexpr (has_gpu_handle<M>::value) return m.gpu_handle();
    else return nullptr;
}

// Products of a matrix without an engine handle, run on the host through its
// own workspaces (Workspace::multiply / AdjointWorkspace::multiply,
// Matrix/interface.hpp:49,87) for the engine's host-operator path: the IRLBA
// loop stays on the device and each product copies its vectors across.
template <class Matrix_, class EigenVector_>
class HostProducts {
public:
    explicit HostProducts(const Matrix_& m) : my_matrix(m) {}
    static int32_t call(void* self, int32_t adjoint, const double* x, double* y) {
        auto* me = static_cast<HostProducts*>(self);
        try {
            me->run(adjoint != 0, x, y);
            return 0;
        } catch (const std::exception& e) {
            me->error = e.what();
        } catch (...) {
            me->error = "user-defined product threw";
        }
        return 1;
    }
    std::string error;

private:
    void run(bool adjoint, const double* x, double* y) {
        const Index nin = adjoint ? my_matrix.rows() : my_matrix.cols();
        const Index nout = adjoint ? my_matrix.cols() : my_matrix.rows();
        my_in.resize(nin);
        for (Index i = 0; i < nin; ++i) my_in.data()[i] = x[i];
        my_out.resize(nout);
        if (adjoint) {
            if (!my_adj) my_adj = my_matrix.new_known_adjoint_workspace();
            my_adj->multiply(my_in, my_out);
        } else {
            if (!my_mul) my_mul = my_matrix.new_known_workspace();
            my_mul->multiply(my_in, my_out);
        }
        for (Index i = 0; i < nout; ++i) y[i] = static_cast<double>(my_out.data()[i]);
    }
    const Matrix_& my_matrix;
    decltype(std::declval<const Matrix_&>().new_known_workspace()) my_mul;
    decltype(std::declval<const Matrix_&>().new_known_adjoint_workspace()) my_adj;
    EigenVector_ my_in, my_out;
};

// Engine handle of `m`: its own, or a host operator over its workspaces (kept
// alive by `products` and `op`).
// Passes a decorator's centre or scale vector to the engine again when its
// contents differ from `seen` (the contents passed last).
template <class Vector_>
void refresh_vector(irlba_gb300_matrix* h, const Vector_& v, std::vector<double>& seen) {
    if (static_cast<size_t>(v.size()) != seen.size()) throw std::runtime_error("decorator vector changed length");
    const auto* d = v.data();
    bool same = true;
    for (size_t i = 0; i < seen.size(); ++i)
        if (static_cast<double>(d[i]) != seen[i]) {
            same = false;
            break;
        }
    if (same) return;
    for (size_t i = 0; i < seen.size(); ++i) seen[i] = static_cast<double>(d[i]);
    check(irlba_gb300_matrix_set_vector(h, seen.data()));
}

template <class EigenVector_, class Matrix_>
const irlba_gb300_matrix* handle_or_host_operator(const Matrix_& m, std::shared_ptr<void>& products, Handle& op) {
    const irlba_gb300_matrix* h = handle_of(m);
    if (h) return h;
    auto p = std::make_shared<HostProducts<Matrix_, EigenVector_>>(m);
    irlba_gb300_matrix* raw = nullptr;
    check(irlba_gb300_matrix_create_host_operator(m.rows(), m.cols(), &HostProducts<Matrix_, EigenVector_>::call,
                                                  p.get(), default_form(), &raw));
    op = adopt(raw);
    products = p;
    return raw;
}

}  // namespace gpu

// ---------------------------------------------------------------------------
// parallelize and EigenThreadScope (parallel.hpp:32-106), for callers' own
// Matrix implementations. The engine itself runs on the device and uses
// neither.
// ---------------------------------------------------------------------------

// Runs run_task(t) for t in [0, num_tasks), one worker per task, and returns
// when all have finished; with the IRLBA_CUSTOM_PARALLEL function-like macro
// defined, that macro is called instead (same arguments). An exception thrown
// by a task is rethrown here after every worker has joined.
template <typename Task_, class Run_>
void parallelize(Task_ num_tasks, Run_ run_task) {
#ifdef IRLBA_CUSTOM_PARALLEL
    IRLBA_CUSTOM_PARALLEL(num_tasks, run_task);
#else
    if (num_tasks <= 0) return;
    if (num_tasks == 1) {
        run_task(static_cast<Task_>(0));
        return;
    }
    std::vector<std::exception_ptr> errors(static_cast<size_t>(num_tasks));
    std::vector<std::thread> workers;
    workers.reserve(static_cast<size_t>(num_tasks) - 1);
    auto guarded_task = [&](Task_ t) {
        try {
            run_task(t);
        } catch (...) {
            errors[static_cast<size_t>(t)] = std::current_exception();
        }
    };
    for (Task_ t = 1; t < num_tasks; ++t) workers.emplace_back(guarded_task, t);
    guarded_task(static_cast<Task_>(0));
    for (auto& w : workers) w.join();
    for (auto& e : errors)
        if (e) std::rethrow_exception(e);
#endif
}

// Restricts the threads of the caller's Eigen operations while it lives, as the
// reference does: num_threads when the parallelization scheme is OpenMP
// (IRLBA_CUSTOM_PARALLEL with IRLBA_CUSTOM_PARALLEL_USES_OPENMP), else 1 (the
// default parallelize() above uses its own threads). No effect without Eigen or
// without OpenMP.
class EigenThreadScope {
public:
#if defined(_OPENMP) && defined(EIGEN_WORLD_VERSION)
    EigenThreadScope(int num_threads) : my_previous(Eigen::nbThreads()) {
#if defined(IRLBA_CUSTOM_PARALLEL) && defined(IRLBA_CUSTOM_PARALLEL_USES_OPENMP)
        Eigen::setNbThreads(num_threads);
#else
        (void)num_threads;
        Eigen::setNbThreads(1);
#endif
    }
    ~EigenThreadScope() { Eigen::setNbThreads(my_previous); }

private:
    int my_previous;

public:
#else
    EigenThreadScope(int /*num_threads*/) {}
#endif
    EigenThreadScope(const EigenThreadScope&) = delete;
    EigenThreadScope(EigenThreadScope&&) = delete;
    EigenThreadScope& operator=(const EigenThreadScope&) = delete;
    EigenThreadScope& operator=(EigenThreadScope&&) = delete;
};

// ---------------------------------------------------------------------------
// Options (Options.hpp:19-83)
// ---------------------------------------------------------------------------
template <class EigenVector_ IRLBA_GB300_VECTOR_DEFAULT_ARG>
struct Options {
    double invariant_subspace_tolerance = -1;
    double convergence_tolerance = 1e-5;
    double singular_value_ratio_tolerance = -1;
    int extra_work = 7;
    int max_iterations = 1000;
    bool exact_for_small_matrix = true;
    bool exact_for_large_number = true;
    bool cap_number = false;
    typename std::mt19937_64::result_type seed = std::mt19937_64::default_seed;
    std::optional<EigenVector_> initial;
};

namespace gpu {
template <class EigenVector_>
irlba_gb300_options to_c(const Options<EigenVector_>& o, std::vector<double>& init_buf) {
    irlba_gb300_options c;
    irlba_gb300_default_options(&c);
    c.invariant_subspace_tolerance = o.invariant_subspace_tolerance;
    c.convergence_tolerance = o.convergence_tolerance;
    c.singular_value_ratio_tolerance = o.singular_value_ratio_tolerance;
    c.extra_work = o.extra_work;
    c.max_iterations = o.max_iterations;
    c.exact_for_small_matrix = o.exact_for_small_matrix;
    c.exact_for_large_number = o.exact_for_large_number;
    c.cap_number = o.cap_number;
    c.seed = o.seed;
    if (o.initial.has_value()) {
        const auto& v = *o.initial;
        init_buf.assign(v.data(), v.data() + v.size());
        c.initial = init_buf.data();
        c.initial_size = static_cast<int64_t>(init_buf.size());
    }
    return c;
}
}  // namespace gpu

// ---------------------------------------------------------------------------
// Plug-in surface (Matrix/interface.hpp)
// ---------------------------------------------------------------------------
template <class EigenVector_>
class Workspace {
public:
    virtual ~Workspace() {}
    virtual void multiply(const EigenVector_& right, EigenVector_& output) = 0;
};

template <class EigenVector_>
class AdjointWorkspace {
public:
    virtual ~AdjointWorkspace() {}
    virtual void multiply(const EigenVector_& right, EigenVector_& output) = 0;
};

template <class EigenMatrix_>
class RealizeWorkspace {
public:
    virtual ~RealizeWorkspace() {}
    virtual const EigenMatrix_& realize(EigenMatrix_& buffer) = 0;
    void realize_copy(EigenMatrix_& buffer) {
        const auto& out = realize(buffer);
        if (&out != &buffer) buffer = out;
    }
};

template <class EigenVector_, class EigenMatrix_>
class Matrix {
public:
    virtual ~Matrix() {}
    virtual Index rows() const = 0;
    virtual Index cols() const = 0;
    virtual std::unique_ptr<Workspace<EigenVector_>> new_workspace() const = 0;
    virtual std::unique_ptr<AdjointWorkspace<EigenVector_>> new_adjoint_workspace() const = 0;
    virtual std::unique_ptr<RealizeWorkspace<EigenMatrix_>> new_realize_workspace() const = 0;
    std::unique_ptr<Workspace<EigenVector_>> new_known_workspace() const { return new_workspace(); }
    std::unique_ptr<AdjointWorkspace<EigenVector_>> new_known_adjoint_workspace() const {
        return new_adjoint_workspace();
    }
    std::unique_ptr<RealizeWorkspace<EigenMatrix_>> new_known_realize_workspace() const {
        return new_realize_workspace();
    }
    // Device handle of the engine, or NULL for a matrix the engine cannot run.
    virtual const irlba_gb300_matrix* gpu_handle() const { return nullptr; }
};

namespace gpu {

template <class EigenVector_>
class HandleWorkspace final : public Workspace<EigenVector_> {
public:
    explicit HandleWorkspace(const irlba_gb300_matrix* h) : my_h(h) {}
    void multiply(const EigenVector_& right, EigenVector_& output) {
        int64_t nr = 0, nc = 0;
        check(irlba_gb300_matrix_dims(my_h, &nr, &nc));
        std::vector<double> in(right.data(), right.data() + right.size()), out(nr);
        check(irlba_gb300_multiply(my_h, in.data(), out.data()));
        output.resize(nr);
        for (int64_t i = 0; i < nr; ++i) output.data()[i] = out[i];
    }

private:
    const irlba_gb300_matrix* my_h;
};

template <class EigenVector_>
class HandleAdjointWorkspace final : public AdjointWorkspace<EigenVector_> {
public:
    explicit HandleAdjointWorkspace(const irlba_gb300_matrix* h) : my_h(h) {}
    void multiply(const EigenVector_& right, EigenVector_& output) {
        int64_t nr = 0, nc = 0;
        check(irlba_gb300_matrix_dims(my_h, &nr, &nc));
        std::vector<double> in(right.data(), right.data() + right.size()), out(nc);
        check(irlba_gb300_adjoint_multiply(my_h, in.data(), out.data()));
        output.resize(nc);
        for (int64_t i = 0; i < nc; ++i) output.data()[i] = out[i];
    }

private:
    const irlba_gb300_matrix* my_h;
};

template <class EigenMatrix_>
class HandleRealizeWorkspace final : public RealizeWorkspace<EigenMatrix_> {
public:
    explicit HandleRealizeWorkspace(const irlba_gb300_matrix* h) : my_h(h) {}
    const EigenMatrix_& realize(EigenMatrix_& buffer) {
        int64_t nr = 0, nc = 0;
        check(irlba_gb300_matrix_dims(my_h, &nr, &nc));
        std::vector<double> out(static_cast<size_t>(nr * nc));
        check(irlba_gb300_realize(my_h, out.data()));
        buffer.resize(nr, nc);
        for (int64_t c = 0; c < nc; ++c)
            for (int64_t r = 0; r < nr; ++r) buffer(r, c) = out[c * nr + r];
        return buffer;
    }

private:
    const irlba_gb300_matrix* my_h;
};

// Common base of the engine-backed matrices.
template <class EigenVector_, class EigenMatrix_>
class HandleMatrix : public Matrix<EigenVector_, EigenMatrix_> {
public:
    Index rows() const { return my_nrow; }
    Index cols() const { return my_ncol; }
    std::unique_ptr<Workspace<EigenVector_>> new_workspace() const {
        return std::make_unique<HandleWorkspace<EigenVector_>>(this->gpu_handle());
    }
    std::unique_ptr<AdjointWorkspace<EigenVector_>> new_adjoint_workspace() const {
        return std::make_unique<HandleAdjointWorkspace<EigenVector_>>(this->gpu_handle());
    }
    std::unique_ptr<RealizeWorkspace<EigenMatrix_>> new_realize_workspace() const {
        return std::make_unique<HandleRealizeWorkspace<EigenMatrix_>>(this->gpu_handle());
    }
    const irlba_gb300_matrix* gpu_handle() const override { return my_handle.get(); }

protected:
    Handle my_handle;
    Index my_nrow = 0, my_ncol = 0;
};

// A user-defined matrix whose products run on the device, e.g. a residual
// matrix that is never stored: the GPU form of a user's own Matrix subclass
// (Matrix/interface.hpp:141-223). product(adjoint, x, y, stream) enqueues
// y = A x (adjoint false; x of length cols()) or y = A^T x on the cudaStream_t
// `stream` and returns; x and y are device vectors of double (FP64 form) or
// float (FP32 form, see set_form()). A product that throws fails the running
// call.
template <class EigenVector_, class EigenMatrix_>
class DeviceMatrix final : public HandleMatrix<EigenVector_, EigenMatrix_> {
public:
    typedef std::function<void(bool adjoint, const void* x, void* y, void* stream)> Product;
    DeviceMatrix(Index nrow, Index ncol, Product product) : my_product(new Product(std::move(product))) {
        irlba_gb300_matrix* h = nullptr;
        check(irlba_gb300_matrix_create_device_operator(nrow, ncol, &DeviceMatrix::call, my_product.get(),
                                                        default_form(), &h));
        this->my_handle = adopt(h);
        this->my_nrow = nrow;
        this->my_ncol = ncol;
    }
    ~DeviceMatrix() { this->my_handle.reset(); }

private:
    static int32_t call(void* user, int32_t adjoint, const void* x, void* y, void* stream) {
        try {
            (*static_cast<Product*>(user))(adjoint != 0, x, y, stream);
            return 0;
        } catch (...) {
            return 1;
        }
    }
    std::unique_ptr<Product> my_product;
};

}  // namespace gpu

namespace gpu {

// Compressed sparse storage in Eigen's layout (Eigen::SparseMatrix and maps of
// it): valuePtr(), innerIndexPtr() and outerIndexPtr(), column-major unless the
// type's IsRowMajor is true. In Eigen's uncompressed mode innerNonZeroPtr() is
// not NULL and gives the entry count of each outer vector.
template <class T, class = void>
struct is_compressed_sparse : std::false_type {};
template <class T>
struct is_compressed_sparse<T, std::void_t<decltype(std::declval<const T&>().valuePtr()),
                                           decltype(std::declval<const T&>().innerIndexPtr()),
                                           decltype(std::declval<const T&>().outerIndexPtr())>> : std::true_type {};

template <class T, class = void>
struct has_inner_nonzeros : std::false_type {};
template <class T>
struct has_inner_nonzeros<T, std::void_t<decltype(std::declval<const T&>().innerNonZeroPtr())>> : std::true_type {};

// The entries of a compressed sparse matrix as the C ABI takes them: int64
// pointers over the outer dimension (columns, or rows when row-major), int32
// inner indices and the values, in either storage mode.
template <class S, class V>
void compressed_arrays(const S& m, std::vector<int64_t>& ptr, std::vector<int32_t>& idx, std::vector<V>& val) {
    const Index outer = is_row_major<S>::value ? m.rows() : m.cols();
    const auto* op = m.outerIndexPtr();
    const auto* ip = m.innerIndexPtr();
    const auto* vp = m.valuePtr();
    const decltype(op) counts = [&]() -> decltype(op) {
        if constexpr (has_inner_nonzeros<S>::value) return m.innerNonZeroPtr();
        else return nullptr;
    }();
    ptr.assign(static_cast<size_t>(outer) + 1, 0);
    for (Index o = 0; o < outer; ++o)
        ptr[o + 1] = ptr[o] + static_cast<int64_t>(counts ? counts[o] : op[o + 1] - op[o]);
    idx.resize(static_cast<size_t>(ptr[outer]));
    val.resize(static_cast<size_t>(ptr[outer]));
    for (Index o = 0; o < outer; ++o) {
        const int64_t src = static_cast<int64_t>(op[o]);
        for (int64_t k = 0; k < ptr[o + 1] - ptr[o]; ++k) {
            idx[ptr[o] + k] = static_cast<int32_t>(ip[src + k]);
            val[ptr[o] + k] = static_cast<V>(vp[src + k]);
        }
    }
}

}  // namespace gpu

// SimpleMatrix over a dense matrix or an Eigen-style compressed sparse matrix
// (simple.hpp:124-178 wraps either). The data are copied to the device at
// construction: dense input as it is, sparse input through the same device
// layout as ParallelSparseMatrix.
template <class EigenVector_, class EigenMatrix_, class Simple_>
class SimpleMatrix final : public gpu::HandleMatrix<EigenVector_, EigenMatrix_> {
public:
    SimpleMatrix(Simple_ matrix) : my_matrix(std::move(matrix)) {
        const auto& m = gpu::deref(my_matrix);
        typedef typename std::remove_cv<typename std::remove_reference<decltype(m)>::type>::type M;
        const bool rm = gpu::is_row_major<M>::value;
        irlba_gb300_matrix* h = nullptr;
        if constexpr (gpu::is_compressed_sparse<M>::value) {
            typedef typename std::remove_cv<typename std::remove_pointer<decltype(m.valuePtr())>::type>::type Scalar;
            std::vector<int64_t> ptr;
            std::vector<int32_t> idx;
            if (std::is_same<Scalar, float>::value) {
                std::vector<float> val;
                gpu::compressed_arrays(m, ptr, idx, val);
                gpu::check(irlba_gb300_matrix_create_sparse(m.rows(), m.cols(), val.data(), IRLBA_GB300_VALUE_F32,
                                                            idx.data(), ptr.data(), rm ? 0 : 1, gpu::default_form(), &h));
            } else {
                std::vector<double> val;
                gpu::compressed_arrays(m, ptr, idx, val);
                gpu::check(irlba_gb300_matrix_create_sparse(m.rows(), m.cols(), val.data(), IRLBA_GB300_VALUE_F64,
                                                            idx.data(), ptr.data(), rm ? 0 : 1, gpu::default_form(), &h));
            }
        } else {
            typedef typename std::remove_cv<typename std::remove_pointer<decltype(m.data())>::type>::type Scalar;
            const irlba_gb300_value_type vt =
                std::is_same<Scalar, float>::value ? IRLBA_GB300_VALUE_F32 : IRLBA_GB300_VALUE_F64;
            std::vector<double> conv;
            const void* data = m.data();
            int64_t ld = rm ? m.cols() : m.rows();
            bool unit_inner = true;
            if constexpr (gpu::has_strides<M>::value) {
                // Strided storage (a Map with an outer stride, a Block): the
                // engine reads it with the type's own leading dimension.
                ld = static_cast<int64_t>(m.outerStride());
                unit_inner = m.innerStride() == 1;
            }
            const bool convert = !std::is_same<Scalar, float>::value && !std::is_same<Scalar, double>::value;
            bool row_major = rm;
            if (convert || !unit_inner) {
                // Other scalar types, or a non-unit inner stride: copy to a
                // contiguous column-major FP64 array.
                conv.resize(static_cast<size_t>(m.rows() * m.cols()));
                for (Index c = 0; c < m.cols(); ++c)
                    for (Index r = 0; r < m.rows(); ++r)
                        conv[static_cast<size_t>(c * m.rows() + r)] = static_cast<double>(m(r, c));
                data = conv.data();
                ld = m.rows();
                row_major = false;
            }
            gpu::check(irlba_gb300_matrix_create_dense(m.rows(), m.cols(), data,
                                                       (convert || !unit_inner) ? IRLBA_GB300_VALUE_F64 : vt,
                                                       ld > 0 ? ld : 1, row_major ? 1 : 0, gpu::default_form(), &h));
        }
        this->my_handle = gpu::adopt(h);
        this->my_nrow = m.rows();
        this->my_ncol = m.cols();
    }

private:
    Simple_ my_matrix;
};

namespace gpu {

// The host thread partitions ParallelSparseMatrix reports for num_threads > 1
// (sparse.hpp:53-113; the device uses its own split, so these only keep the
// accessors' values): each thread gets an equal share of the nonzeros, the
// first (nnz % num_threads) threads one more. primary[t], primary[t + 1] bound
// thread t's primary elements (the last element whose cumulative count is
// within the thread's cumulative share); secondary[t], secondary[t + 1] bound
// its secondary elements (cumulative per-secondary counts, stepping past the
// share by at most one element); secondary_nonzero[t][c] is where thread t's
// secondary range starts within primary element c.
struct ThreadPartitions {
    std::vector<Index> primary, secondary;
    std::vector<std::vector<int64_t>> secondary_nonzero;
};

inline ThreadPartitions thread_partitions(Index primary_dim, Index secondary_dim, const int64_t* ptr,
                                          const int32_t* idx, int num_threads) {
    ThreadPartitions out;
    if (num_threads <= 1) return out;
    const int64_t total = ptr[primary_dim];
    const auto share_end = [&](int t) {  // cumulative nonzeros of threads 0..t
        const int64_t base = total / num_threads, extra = total % num_threads;
        return base * (t + 1) + std::min<int64_t>(t + 1, extra);
    };
    out.primary.assign(static_cast<size_t>(num_threads) + 1, 0);
    Index p = 0;
    for (int t = 0; t < num_threads; ++t) {
        const int64_t end = share_end(t);
        while (p < primary_dim && ptr[p + 1] <= end) ++p;
        out.primary[t + 1] = p;
    }
    std::vector<int64_t> per_secondary(static_cast<size_t>(secondary_dim), 0);
    for (int64_t k = 0; k < total; ++k) ++per_secondary[idx[k]];
    out.secondary.assign(static_cast<size_t>(num_threads) + 1, 0);
    Index q = 0;
    int64_t seen = 0;
    for (int t = 0; t < num_threads; ++t) {
        const int64_t end = share_end(t);
        while (q < secondary_dim && seen <= end) seen += per_secondary[q++];
        out.secondary[t + 1] = q;
    }
    out.secondary_nonzero.assign(static_cast<size_t>(num_threads) + 1,
                                 std::vector<int64_t>(static_cast<size_t>(primary_dim), 0));
    for (Index c = 0; c < primary_dim; ++c) {
        int64_t k = ptr[c];
        out.secondary_nonzero[0][c] = k;
        for (int t = 1; t <= num_threads; ++t) {
            while (k < ptr[c + 1] && idx[k] < out.secondary[t]) ++k;
            out.secondary_nonzero[t][c] = k;
        }
    }
    return out;
}

}  // namespace gpu

// ParallelSparseMatrix (sparse.hpp:469): compressed sparse column/row data.
// num_threads is accepted for interface parity; the device sets its own split,
// and the host partitions of the reference are kept for its accessors.
template <class EigenVector_, class EigenMatrix_, class ValueArray_, class IndexArray_, class PointerArray_>
class ParallelSparseMatrix final : public gpu::HandleMatrix<EigenVector_, EigenMatrix_> {
public:
    ParallelSparseMatrix() {}
    ParallelSparseMatrix(Index nrow, Index ncol, ValueArray_ x, IndexArray_ i, PointerArray_ p, bool column_major,
                         int num_threads)
        : my_values(std::move(x)), my_indices(std::move(i)), my_ptrs(std::move(p)), my_column_major(column_major),
          my_num_threads(num_threads) {
        const Index primary = column_major ? ncol : nrow;
        std::vector<int64_t> ptr(static_cast<size_t>(primary) + 1);
        for (Index k = 0; k <= primary; ++k) ptr[k] = static_cast<int64_t>(my_ptrs[k]);
        const int64_t nnz = ptr[primary];
        std::vector<int32_t> idx(static_cast<size_t>(nnz));
        for (int64_t k = 0; k < nnz; ++k) idx[k] = static_cast<int32_t>(my_indices[k]);
        typedef typename std::remove_cv<typename std::remove_reference<decltype(my_values[0])>::type>::type Scalar;
        std::vector<double> v64;
        std::vector<float> v32;
        const void* vals;
        irlba_gb300_value_type vt;
        if (std::is_same<Scalar, float>::value) {
            v32.resize(nnz);
            for (int64_t k = 0; k < nnz; ++k) v32[k] = static_cast<float>(my_values[k]);
            vals = v32.data();
            vt = IRLBA_GB300_VALUE_F32;
        } else {
            v64.resize(nnz);
            for (int64_t k = 0; k < nnz; ++k) v64[k] = static_cast<double>(my_values[k]);
            vals = v64.data();
            vt = IRLBA_GB300_VALUE_F64;
        }
        irlba_gb300_matrix* h = nullptr;
        gpu::check(irlba_gb300_matrix_create_sparse(nrow, ncol, vals, vt, idx.data(), ptr.data(), column_major ? 1 : 0,
                                                    gpu::default_form(), &h));
        this->my_handle = gpu::adopt(h);
        this->my_nrow = nrow;
        this->my_ncol = ncol;
        if (num_threads > 1) {
            gpu::ThreadPartitions parts =
                gpu::thread_partitions(primary, column_major ? nrow : ncol, ptr.data(), idx.data(), num_threads);
            my_primary_boundaries = std::move(parts.primary);
            my_secondary_boundaries = std::move(parts.secondary);
            for (const auto& starts : parts.secondary_nonzero)
                my_secondary_nonzero_boundaries.emplace_back(starts.begin(), starts.end());
        }
    }
    typedef typename std::remove_cv<
        typename std::remove_reference<decltype(std::declval<const PointerArray_&>()[0])>::type>::type PointerType;
    const ValueArray_& get_values() const { return my_values; }
    const IndexArray_& get_indices() const { return my_indices; }
    const PointerArray_& get_pointers() const { return my_ptrs; }
    bool get_column_major() const { return my_column_major; }
    int get_num_threads() const { return my_num_threads; }
    // Host thread partitions (sparse.hpp:521-553); set only when num_threads > 1.
    const std::vector<Index>& get_primary_boundaries() const { return my_primary_boundaries; }
    const std::vector<Index>& get_secondary_boundaries() const { return my_secondary_boundaries; }
    const std::vector<std::vector<PointerType>>& get_secondary_nonzero_boundaries() const {
        return my_secondary_nonzero_boundaries;
    }

private:
    std::vector<Index> my_primary_boundaries, my_secondary_boundaries;
    std::vector<std::vector<PointerType>> my_secondary_nonzero_boundaries;
    ValueArray_ my_values;
    IndexArray_ my_indices;
    PointerArray_ my_ptrs;
    bool my_column_major = false;
    int my_num_threads = 1;
};

// CenteredMatrix (centered.hpp:139-204).
template <class EigenVector_, class EigenMatrix_, class MatrixPointer_ = const Matrix<EigenVector_, EigenMatrix_>*,
          class CenterPointer_ = const EigenVector_*>
class CenteredMatrix final : public gpu::HandleMatrix<EigenVector_, EigenMatrix_> {
public:
    CenteredMatrix(MatrixPointer_ matrix, CenterPointer_ center) : my_matrix(std::move(matrix)), my_center(std::move(center)) {
        const auto& inner = gpu::deref(my_matrix);
        const irlba_gb300_matrix* ih = gpu::handle_or_host_operator<EigenVector_>(inner, my_products, my_inner_op);
        const auto& c = gpu::deref(my_center);
        my_seen.assign(c.data(), c.data() + c.size());
        if (static_cast<Index>(my_seen.size()) != inner.cols()) throw std::runtime_error("center has the wrong length");
        irlba_gb300_matrix* h = nullptr;
        gpu::check(irlba_gb300_matrix_center(ih, my_seen.data(), &h));
        this->my_handle = gpu::adopt(h);
        this->my_nrow = inner.rows();
        this->my_ncol = inner.cols();
    }

    ~CenteredMatrix() { this->my_handle.reset(); }

    // Like the reference's decorator, which reads the caller's centre vector
    // through its pointer at every product (centered.hpp:46-52,83-87), the
    // engine handle picks up the vector's current contents whenever it is
    // used (every compute/pca call and every workspace).
    const irlba_gb300_matrix* gpu_handle() const override {
        gpu::handle_of(gpu::deref(my_matrix));  // refreshes decorators nested inside
        gpu::refresh_vector(this->my_handle.get(), gpu::deref(my_center), my_seen);
        return this->my_handle.get();
    }

private:
    MatrixPointer_ my_matrix;
    CenterPointer_ my_center;
    mutable std::vector<double> my_seen;  // the contents last passed to the engine
    std::shared_ptr<void> my_products;  // host products of an inner matrix without an engine handle
    gpu::Handle my_inner_op;
};

// ScaledMatrix (scaled.hpp:195-268).
template <class EigenVector_, class EigenMatrix_, class MatrixPointer_ = const Matrix<EigenVector_, EigenMatrix_>*,
          class ScalePointer_ = const EigenVector_*>
class ScaledMatrix final : public gpu::HandleMatrix<EigenVector_, EigenMatrix_> {
public:
    ScaledMatrix(MatrixPointer_ matrix, ScalePointer_ scale, bool column, bool divide)
        : my_matrix(std::move(matrix)), my_scale(std::move(scale)) {
        const auto& inner = gpu::deref(my_matrix);
        const irlba_gb300_matrix* ih = gpu::handle_or_host_operator<EigenVector_>(inner, my_products, my_inner_op);
        const auto& s = gpu::deref(my_scale);
        my_seen.assign(s.data(), s.data() + s.size());
        if (static_cast<Index>(my_seen.size()) != (column ? inner.cols() : inner.rows()))
            throw std::runtime_error("scale has the wrong length");
        irlba_gb300_matrix* h = nullptr;
        gpu::check(irlba_gb300_matrix_scale(ih, my_seen.data(), column ? 1 : 0, divide ? 1 : 0, &h));
        this->my_handle = gpu::adopt(h);
        this->my_nrow = inner.rows();
        this->my_ncol = inner.cols();
    }

    ~ScaledMatrix() { this->my_handle.reset(); }

    // The scale vector is read at every use, as the reference's decorator
    // reads it through its pointer (scaled.hpp:52-69,106-123).
    const irlba_gb300_matrix* gpu_handle() const override {
        gpu::handle_of(gpu::deref(my_matrix));  // refreshes decorators nested inside
        gpu::refresh_vector(this->my_handle.get(), gpu::deref(my_scale), my_seen);
        return this->my_handle.get();
    }

private:
    MatrixPointer_ my_matrix;
    ScalePointer_ my_scale;
    mutable std::vector<double> my_seen;  // the contents last passed to the engine
    std::shared_ptr<void> my_products;  // host products of an inner matrix without an engine handle
    gpu::Handle my_inner_op;
};

// ---------------------------------------------------------------------------
// compute (compute.hpp:141-308) and overloads
// ---------------------------------------------------------------------------
namespace gpu {
template <class EigenMatrix_>
void fill_matrix(EigenMatrix_& out, Index nr, Index nc, const std::vector<double>& colmajor) {
    out.resize(nr, nc);
    for (Index c = 0; c < nc; ++c)
        for (Index r = 0; r < nr; ++r) out(r, c) = colmajor[static_cast<size_t>(c * nr + r)];
}
template <class EigenVector_>
void fill_vector(EigenVector_& out, const std::vector<double>& v, Index n) {
    out.resize(n);
    for (Index i = 0; i < n; ++i) out.data()[i] = v[i];
}
}  // namespace gpu

template <class Matrix_, class EigenMatrix_, class EigenVector_>
std::pair<bool, int> compute(const Matrix_& matrix, Index number, EigenMatrix_& outU, EigenMatrix_& outV,
                             EigenVector_& outD, const Options<EigenVector_>& options) {
    // A matrix without an engine handle (a user's own Matrix subclass) runs
    // with the loop on the device and its products called on the host.
    std::shared_ptr<void> products;
    gpu::Handle host_op;
    const irlba_gb300_matrix* h = gpu::handle_or_host_operator<EigenVector_>(matrix, products, host_op);
    const Index nr = matrix.rows(), nc = matrix.cols();
    const Index cap = std::max<Index>(std::min<Index>(number, std::min(nr, nc)), 0);
    std::vector<double> U(static_cast<size_t>(nr * cap)), V(static_cast<size_t>(nc * cap)), D(cap > 0 ? cap : 1);
    std::vector<double> init;
    irlba_gb300_options o = gpu::to_c(options, init);
    int64_t num = 0;
    int32_t conv = 0, iters = 0;
    const irlba_gb300_status st =
        irlba_gb300_compute(h, number, &o, U.data(), V.data(), D.data(), &num, &conv, &iters, nullptr);
    if (st != IRLBA_GB300_OK && products) {
        const std::string& why = static_cast<gpu::HostProducts<Matrix_, EigenVector_>*>(products.get())->error;
        if (!why.empty()) throw std::runtime_error(why);
    }
    gpu::check(st);
    gpu::fill_matrix(outU, nr, num, U);
    gpu::fill_matrix(outV, nc, num, V);
    gpu::fill_vector(outD, D, num);
    return std::make_pair(conv != 0, static_cast<int>(iters));
}

template <class EigenMatrix_, class EigenVector_>
struct Results {
    EigenMatrix_ U;
    EigenMatrix_ V;
    EigenVector_ D;
    int iterations;
    bool converged;
};

template <class EigenMatrix_ IRLBA_GB300_MATRIX_DEFAULT_ARG, class EigenVector_ IRLBA_GB300_VECTOR_DEFAULT_ARG,
          class Matrix_>
Results<EigenMatrix_, EigenVector_> compute(const Matrix_& matrix, Index number, const Options<EigenVector_>& options) {
    Results<EigenMatrix_, EigenVector_> output;
    const auto stats = compute(matrix, number, output.U, output.V, output.D, options);
    output.converged = stats.first;
    output.iterations = stats.second;
    return output;
}

template <class InputEigenMatrix_, class OutputEigenMatrix_, class EigenVector_>
std::pair<bool, int> compute_simple(const InputEigenMatrix_& matrix, Index number, OutputEigenMatrix_& outU,
                                    OutputEigenMatrix_& outV, EigenVector_& outD,
                                    const Options<EigenVector_>& options) {
    SimpleMatrix<EigenVector_, OutputEigenMatrix_, const InputEigenMatrix_*> wrapped(&matrix);
    return compute(wrapped, number, outU, outV, outD, options);
}

template <class OutputEigenMatrix_ IRLBA_GB300_MATRIX_DEFAULT_ARG, class EigenVector_ IRLBA_GB300_VECTOR_DEFAULT_ARG,
          class InputEigenMatrix_>
Results<OutputEigenMatrix_, EigenVector_> compute_simple(const InputEigenMatrix_& matrix, Index number,
                                                         const Options<EigenVector_>& options) {
    Results<OutputEigenMatrix_, EigenVector_> output;
    const auto stats = compute_simple(matrix, number, output.U, output.V, output.D, options);
    output.converged = stats.first;
    output.iterations = stats.second;
    return output;
}

// ---------------------------------------------------------------------------
// pca (pca.hpp:55-204)
// ---------------------------------------------------------------------------
template <class EigenMatrix_, class EigenVector_>
struct PcaResults {
    EigenMatrix_ scores;
    EigenMatrix_ rotation;
    EigenVector_ variances;
    int iterations;
    bool converged;
};

namespace gpu {
template <class OutputEigenMatrix_, class EigenVector_>
std::pair<bool, int> pca_on_handle(const irlba_gb300_matrix* h, Index nr, Index nc, bool center, bool scale,
                                   Index number, OutputEigenMatrix_& scores, OutputEigenMatrix_& rotation,
                                   EigenVector_& variances, const Options<EigenVector_>& options) {
    const Index cap = std::max<Index>(std::min<Index>(number, std::min(nr, nc)), 0);
    std::vector<double> S(static_cast<size_t>(nr * cap)), R(static_cast<size_t>(nc * cap)), var(cap > 0 ? cap : 1);
    std::vector<double> init;
    irlba_gb300_options o = to_c(options, init);
    int64_t num = 0;
    int32_t conv = 0, iters = 0;
    check(irlba_gb300_pca(h, center ? 1 : 0, scale ? 1 : 0, number, &o, S.data(), R.data(), var.data(), &num, &conv,
                          &iters, nullptr, nullptr, nullptr));
    fill_matrix(scores, nr, num, S);
    fill_matrix(rotation, nc, num, R);
    fill_vector(variances, var, num);
    return std::make_pair(conv != 0, static_cast<int>(iters));
}
}  // namespace gpu

template <class InputEigenMatrix_, class OutputEigenMatrix_, class EigenVector_>
std::pair<bool, int> pca(const InputEigenMatrix_& matrix, bool center, bool scale, Index number,
                         OutputEigenMatrix_& scores, OutputEigenMatrix_& rotation, EigenVector_& variances,
                         const Options<EigenVector_>& options) {
    SimpleMatrix<EigenVector_, OutputEigenMatrix_, const InputEigenMatrix_*> wrapped(&matrix);
    return gpu::pca_on_handle(wrapped.gpu_handle(), wrapped.rows(), wrapped.cols(), center, scale, number, scores,
                              rotation, variances, options);
}

template <class OutputEigenMatrix_ IRLBA_GB300_MATRIX_DEFAULT_ARG, class EigenVector_ IRLBA_GB300_VECTOR_DEFAULT_ARG,
          class InputEigenMatrix_>
PcaResults<OutputEigenMatrix_, EigenVector_> pca(const InputEigenMatrix_& matrix, bool center, bool scale,
                                                 Index number, const Options<EigenVector_>& options) {
    PcaResults<OutputEigenMatrix_, EigenVector_> output;
    const auto stats = pca(matrix, center, scale, number, output.scores, output.rotation, output.variances, options);
    output.converged = stats.first;
    output.iterations = stats.second;
    return output;
}

// Extension: pca() over an engine-backed base matrix (e.g. a ParallelSparseMatrix
// of cells x genes), with the column statistics computed on the device.
template <class EigenVector_, class EigenMatrix_, class OutputEigenMatrix_>
std::pair<bool, int> pca(const gpu::HandleMatrix<EigenVector_, EigenMatrix_>& matrix, bool center, bool scale,
                         Index number, OutputEigenMatrix_& scores, OutputEigenMatrix_& rotation,
                         EigenVector_& variances, const Options<EigenVector_>& options) {
    return gpu::pca_on_handle(matrix.gpu_handle(), matrix.rows(), matrix.cols(), center, scale, number, scores,
                              rotation, variances, options);
}

}  // namespace irlba

#endif
