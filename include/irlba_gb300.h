/*
 * irlba_gb300.h — C ABI of the GB300 (sm_103a) IRLBA engine.
 *
 * This is the only entry into the CUDA engine. Every function returns an
 * irlba_gb300_status; on failure, irlba_gb300_last_error() gives a message whose
 * wording follows the exception text CppIrlba throws for the same condition.
 * Plain pointers and sizes only. Host pointers unless a name says "device".
 *
 * Reference interfaces replaced (CppIrlba, paths relative to its project root):
 *   matrix handles      <- irlba::Matrix and subclasses   include/irlba/Matrix/interface.hpp:141-223
 *   sparse create       <- irlba::ParallelSparseMatrix    include/irlba/Matrix/sparse.hpp:469-471
 *   dense create        <- irlba::SimpleMatrix            include/irlba/Matrix/simple.hpp:124-178
 *   operator create     <- a user subclass of irlba::Matrix include/irlba/Matrix/interface.hpp:141-223
 *   center              <- irlba::CenteredMatrix          include/irlba/Matrix/centered.hpp:139-204
 *   scale               <- irlba::ScaledMatrix            include/irlba/Matrix/scaled.hpp:195-268
 *   multiply            <- Workspace::multiply            include/irlba/Matrix/interface.hpp:49
 *   adjoint_multiply    <- AdjointWorkspace::multiply     include/irlba/Matrix/interface.hpp:87
 *   realize             <- RealizeWorkspace::realize_copy include/irlba/Matrix/interface.hpp:125-130
 *   options             <- irlba::Options                 include/irlba/Options.hpp:19-83
 *   compute             <- irlba::compute                 include/irlba/compute.hpp:141-308
 *   pca                 <- irlba::pca                     include/irlba/pca.hpp:55-139
 *   orthogonalize       <- irlba::orthogonalize_vector    include/irlba/lanczos.hpp:17-21
 */
#ifndef IRLBA_GB300_H
#define IRLBA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    IRLBA_GB300_OK = 0,
    IRLBA_GB300_ERROR_INVALID_ARGUMENT = 1, /* messages as the reference's std::runtime_error */
    IRLBA_GB300_ERROR_CUDA = 2,             /* a CUDA call failed (no GPU, out of memory, ...) */
    IRLBA_GB300_ERROR_NUMERICAL = 3,        /* e.g. starting vector near the null space */
    IRLBA_GB300_ERROR_UNSUPPORTED = 4       /* e.g. a gradient through an unfused decorator chain */
} irlba_gb300_status;

typedef enum {
    IRLBA_GB300_VALUE_F32 = 0,
    IRLBA_GB300_VALUE_F64 = 1
} irlba_gb300_value_type;

/* Arithmetic form of the Lanczos loop. */
typedef enum {
    /* FP64 matrix values, basis, matvecs, recurrence and restart (matches the reference). */
    IRLBA_GB300_FORM_FP64 = 0,
    /* FP32 matrix values, basis and matvecs with FP32 accumulation; FP64 for the
     * reorthogonalization coefficients and norms, the bidiagonal recurrence
     * (alpha/beta), the restart small SVD and the residual convergence test. */
    IRLBA_GB300_FORM_FP32_FP64STEPS = 1
} irlba_gb300_form;

/* Mirrors irlba::Options (Options.hpp:19-83); same names, meanings and defaults.
 * `initial` is the optional start vector (length = columns of the matrix), or NULL. */
typedef struct {
    double invariant_subspace_tolerance;   /* -1 -> eps^0.8 */
    double convergence_tolerance;          /* 1e-5 */
    double singular_value_ratio_tolerance; /* -1 -> convergence_tolerance */
    int32_t extra_work;                    /* 7 */
    int32_t max_iterations;                /* 1000 */
    int32_t exact_for_small_matrix;        /* 1 */
    int32_t exact_for_large_number;        /* 1 */
    int32_t cap_number;                    /* 0 */
    int32_t reserved0;
    uint64_t seed;                         /* std::mt19937_64::default_seed = 5489 */
    const double* initial;                 /* NULL = random normals from `seed` */
    int64_t initial_size;
} irlba_gb300_options;

/* Per-call statistics (not part of the reference's Results). */
typedef struct {
    int64_t matvecs;          /* multiply + adjoint_multiply calls */
    int64_t lanczos_steps;
    int64_t restarts;
    int64_t careful_restarts; /* restarts re-run to refill an invariant subspace */
    double seconds_total;     /* host wall time of the call */
    double device_ms;         /* CUDA-event time of the call on its stream */
    int64_t kernel_launches;  /* kernels this library launched during the call */
    int64_t svd_sweeps;       /* Jacobi sweeps of the restart SVDs, summed */
} irlba_gb300_stats;

/* Opaque matrix handle: a base matrix or a centre/scale decorator over one. */
typedef struct irlba_gb300_matrix irlba_gb300_matrix;

void irlba_gb300_default_options(irlba_gb300_options* options);
const char* irlba_gb300_last_error(void);
/* Number of CUDA devices visible, or -1 if the runtime cannot be queried. */
int irlba_gb300_device_count(void);

/* ParallelSparseMatrix(nrow, ncol, x, i, p, column_major, num_threads) (sparse.hpp:469).
 * values: nnz entries of value_type; indices: int32 row (column_major) or column
 * indices, sorted within each primary element; pointers: int64, length primary+1.
 * The data are copied to the device. `form` fixes the stored value precision. */
irlba_gb300_status irlba_gb300_matrix_create_sparse(int64_t nrow, int64_t ncol, const void* values,
                                                    irlba_gb300_value_type value_type, const int32_t* indices,
                                                    const int64_t* pointers, int32_t column_major,
                                                    irlba_gb300_form form, irlba_gb300_matrix** out);

/* Where irlba_gb300_matrix_create_sparse builds its device layout: on the GPU
 * from the uploaded compressed arrays (default; needs about twice the matrix
 * size of device memory while it runs, and sorted rows, else it uses the
 * host), or on the host (on = 0). Both give the same layout. */
void irlba_gb300_set_device_ingest(int32_t on);

/* Launch shape of the sparse products of FP32-form matrices created after
 * this call: 0 = 256-thread CTAs; 1 = 256 threads, six CTAs per SM; 2 (the
 * default) = 512 threads, three CTAs per SM. A tuning switch: results agree to
 * rounding. */
void irlba_gb300_set_spmv_shape(int32_t shape);

/* Copies between pageable host memory and the device of at least `min_bytes`
 * (default 16 MiB; < 0: never) run through pinned staging buffers of
 * `slice_bytes` each (default 8 MiB; <= 0 keeps the current size), filled and
 * drained by up to eight host threads. Smaller copies, and copies of pinned
 * host memory, are plain cudaMemcpyAsync calls. Results are the same. */
void irlba_gb300_set_staging(int64_t min_bytes, int64_t slice_bytes);

/* SimpleMatrix over a dense matrix (simple.hpp:124-178); column-major unless
 * row_major != 0; `ld` is the leading dimension. Copied to the device. */
irlba_gb300_status irlba_gb300_matrix_create_dense(int64_t nrow, int64_t ncol, const void* values,
                                                   irlba_gb300_value_type value_type, int64_t ld,
                                                   int32_t row_major, irlba_gb300_form form,
                                                   irlba_gb300_matrix** out);

/* A user-defined matrix: the counterpart of a user subclass of irlba::Matrix
 * (Matrix/interface.hpp:141-223), e.g. a residual matrix that is never stored.
 * The engine runs its whole IRLBA loop (and any CenteredMatrix / ScaledMatrix
 * over it, fused into one elementwise pass after each product) on the device
 * and calls `product` for each Workspace::multiply (adjoint = 0: y = A x, x of
 * length ncol, y of length nrow) and AdjointWorkspace::multiply (adjoint = 1:
 * y = A^T x). Both functions return 0 on success; any other value makes the
 * running call fail with IRLBA_GB300_ERROR_INVALID_ARGUMENT ("user-defined
 * product failed"). `user` is passed through untouched. Products are issued
 * one at a time; `y` arrives dirty and must be fully overwritten, and `x` must
 * not be modified. pca() (which needs the stored columns for its statistics),
 * the differentiation form and irlba_gb300_spmv_device reject these handles. */

/* Device product: x and y are device vectors of the form's type (double for
 * IRLBA_GB300_FORM_FP64, float for IRLBA_GB300_FORM_FP32_FP64STEPS). The
 * function enqueues its work on `stream` (a cudaStream_t) and returns without
 * waiting for it; it may be called on more than one of the engine's streams,
 * always ordered after the producer of x and before the consumer of y. */
typedef int32_t (*irlba_gb300_device_product)(void* user, int32_t adjoint, const void* x, void* y, void* stream);

/* Host product: x and y are FP64 host vectors; the engine copies x out of and
 * y back into device memory around each call (one synchronization per
 * product: correct but not fast). */
typedef int32_t (*irlba_gb300_host_product)(void* user, int32_t adjoint, const double* x, double* y);

irlba_gb300_status irlba_gb300_matrix_create_device_operator(int64_t nrow, int64_t ncol,
                                                             irlba_gb300_device_product product, void* user,
                                                             irlba_gb300_form form, irlba_gb300_matrix** out);
irlba_gb300_status irlba_gb300_matrix_create_host_operator(int64_t nrow, int64_t ncol,
                                                           irlba_gb300_host_product product, void* user,
                                                           irlba_gb300_form form, irlba_gb300_matrix** out);

/* CenteredMatrix(inner, center) (centered.hpp:152): column centring, center has
 * length ncol. The inner handle must outlive the new one. */
irlba_gb300_status irlba_gb300_matrix_center(const irlba_gb300_matrix* inner, const double* center,
                                             irlba_gb300_matrix** out);

/* ScaledMatrix(inner, scale, column, divide) (scaled.hpp:420). scale has length
 * ncol (column != 0) or nrow. The inner handle must outlive the new one. */
irlba_gb300_status irlba_gb300_matrix_scale(const irlba_gb300_matrix* inner, const double* scale, int32_t column,
                                            int32_t divide, irlba_gb300_matrix** out);

irlba_gb300_status irlba_gb300_matrix_destroy(irlba_gb300_matrix* matrix);
irlba_gb300_status irlba_gb300_matrix_dims(const irlba_gb300_matrix* matrix, int64_t* nrow, int64_t* ncol);

/* Workspace::multiply: output (length nrow) = A * right (length ncol). The output
 * is fully overwritten, whatever it held. Host buffers. */
irlba_gb300_status irlba_gb300_multiply(const irlba_gb300_matrix* matrix, const double* right, double* output);
/* AdjointWorkspace::multiply: output (length ncol) = A^T * right (length nrow). */
irlba_gb300_status irlba_gb300_adjoint_multiply(const irlba_gb300_matrix* matrix, const double* right,
                                                double* output);
/* RealizeWorkspace::realize_copy: column-major nrow x ncol dense copy. */
irlba_gb300_status irlba_gb300_realize(const irlba_gb300_matrix* matrix, double* output);

/* irlba::compute(matrix, number, outU, outV, outD, options) (compute.hpp:141-308).
 * U: nrow x number, V: ncol x number (column-major), D: number. If cap_number
 * lowers `number`, *out_number says how many were written. Returns converged and
 * the restart iteration count as the reference's std::pair. */
irlba_gb300_status irlba_gb300_compute(const irlba_gb300_matrix* matrix, int64_t number,
                                       const irlba_gb300_options* options, double* U, double* V, double* D,
                                       int64_t* out_number, int32_t* converged, int32_t* iterations,
                                       irlba_gb300_stats* stats);

/* irlba::pca(matrix, center, scale, number, scores, rotation, variances, options)
 * (pca.hpp:55-139) on a base (undecorated) matrix whose rows are observations.
 * Column means and standard deviations are computed on the device; centring and
 * scaling are deferred into the matvecs. scores: nrow x number; rotation:
 * ncol x number; variances: number. center_out / scale_out (length ncol) may be
 * NULL. */
irlba_gb300_status irlba_gb300_pca(const irlba_gb300_matrix* matrix, int32_t center, int32_t scale, int64_t number,
                                   const irlba_gb300_options* options, double* scores, double* rotation,
                                   double* variances, int64_t* out_number, int32_t* converged, int32_t* iterations,
                                   double* center_out, double* scale_out, irlba_gb300_stats* stats);

/* orthogonalize_vector(mat, vec, ncols, tmp) (lanczos.hpp:17-21) on device memory:
 * vec -= Q[:, :ncols] (Q[:, :ncols]^T vec), Q column-major L x ldq-strided,
 * FP64. `stream` is a cudaStream_t (NULL = legacy default stream). Scratch for
 * the partial dot products is allocated by the library per call. */
irlba_gb300_status irlba_gb300_orthogonalize_vector_device(const double* Q, int64_t L, int64_t ldq, int64_t ncols,
                                                           double* vec, void* stream);

/* Same as irlba_gb300_orthogonalize_vector_device, but allocates nothing: for
 * callers that cannot call cudaMalloc/cudaFree (code living inside another
 * framework's memory budget, or latency-critical loops where an allocation
 * would synchronize the device). No counterpart in the reference. Scratch is a
 * fixed 1 MiB device array per GPU, held until the process exits; the first
 * call on a device looks up its address (make it before any stream capture).
 * The call synchronizes `stream` before it returns. Calls that overlap on the
 * GPU race on the shared scratch. Needs
 * 128 + round_up(max(ncols, 1), 32) + min(ceil(L / 256), 1216) * max(ncols, 1)
 * <= 131072 doubles (any L for ncols <= 107); larger requests return
 * IRLBA_GB300_ERROR_INVALID_ARGUMENT. */
irlba_gb300_status irlba_gb300_orthogonalize_vector_device_noalloc(const double* Q, int64_t L, int64_t ldq,
                                                                   int64_t ncols, double* vec, void* stream);

/* ---- Extensions without a counterpart in the reference --------------------- */

/* irlba_gb300_compute with U (nrow x number), V (ncol x number) and D (number)
 * in device memory, issued on `stream` (a cudaStream_t; NULL = an internal
 * stream). The call returns when the results are complete. */
irlba_gb300_status irlba_gb300_compute_device(const irlba_gb300_matrix* matrix, int64_t number,
                                              const irlba_gb300_options* options, double* U_device,
                                              double* V_device, double* D_device, int64_t* out_number,
                                              int32_t* converged, int32_t* iterations, irlba_gb300_stats* stats,
                                              void* stream);

/* irlba_gb300_pca with scores (nrow x number), rotation (ncol x number) and
 * variances (number) in device memory, issued on `stream` (NULL = internal). */
irlba_gb300_status irlba_gb300_pca_device(const irlba_gb300_matrix* matrix, int32_t center, int32_t scale,
                                          int64_t number, const irlba_gb300_options* options, double* scores_device,
                                          double* rotation_device, double* variances_device, int64_t* out_number,
                                          int32_t* converged, int32_t* iterations, irlba_gb300_stats* stats,
                                          void* stream);

/* One direction of the raw sparse product of an undecorated matrix on device
 * vectors: y = A x (adjoint = 0) or y = A^T x. Vectors are FP64 for FP64-form
 * matrices and FP32 for the FP32 form. Asynchronous on `stream`. */
irlba_gb300_status irlba_gb300_spmv_device(const irlba_gb300_matrix* matrix, int32_t adjoint, const void* x,
                                           void* y, void* stream);

/* Replaces the centre vector of a CenteredMatrix handle or the scale vector of
 * a ScaledMatrix handle (same length as at creation). Replaces the pointer
 * semantics of the reference's decorators, which read the caller's vector at
 * every product (centered.hpp:139-160, scaled.hpp:195-223). */
irlba_gb300_status irlba_gb300_matrix_set_vector(irlba_gb300_matrix* matrix, const double* values);

/* update_k of the device restart step (compute.hpp:78-111, irlba::update_k)
 * evaluated on the GPU for `count` argument quadruples args[4i..4i+3] =
 * (k, requested, n_converged, work); out[i] receives the next k. Host arrays.
 * Exposed so the device arithmetic can be checked against the reference's
 * known answers (tests/src/compute.cpp:52-76). */
irlba_gb300_status irlba_gb300_update_k_device(const int32_t* args, int64_t count, int32_t* out);

/* The restart step's basis rotation (compute.hpp:268-280: V <- V BV,
 * W <- W BU) on device memory: out[:, :k] = Q[:, :w] R[:w, :k], and
 * out[:, k] = fcol / *fnorm when fcol is not NULL (fnorm a device pointer).
 * Q, out and fcol are FP64 (fp64 = 1) or FP32 (fp64 = 0) column-major arrays;
 * R is FP64; out may be Q. engine 1 runs the tensor-core kernels (BF16 slice
 * products to FP32 or FP64 accuracy; w, k <= 64, otherwise
 * IRLBA_GB300_ERROR_UNSUPPORTED), engine 0 the CUDA-core kernels. Returns when
 * the rotation is complete. Exposed so the rotation kernels can be checked
 * against each other and an FP64 product. */
irlba_gb300_status irlba_gb300_rotate_device(int32_t fp64, const void* Q, int64_t L, int64_t ldq, int32_t w,
                                             const double* R, int32_t ldr, int32_t k, void* out, int64_t ldo,
                                             const void* fcol, const double* fnorm, int32_t engine, void* stream);

/* Engine of the restart rotations of later compute calls with a working
 * subspace of at most 64 columns: 1 = tensor cores (default), 0 = CUDA cores. */
void irlba_gb300_set_rotation_engine(int32_t engine);

/* Dictionary coding of FP32-form sparse matrices created afterwards (0, the
 * default, keeps the plain layout): with 1, a matrix with at most 2,048
 * distinct values keeps each value as a 16-bit code into a table of the exact
 * values for the products (4 bytes per entry moved instead of 6; results
 * unchanged). irlba_gb300_matrix_layout reports value_bytes = 2 for a coded
 * matrix. */
void irlba_gb300_set_value_coding(int32_t on);

/* Stored layout of an undecorated matrix, for byte accounting. */
irlba_gb300_status irlba_gb300_matrix_layout(const irlba_gb300_matrix* matrix, int64_t* nnz, int32_t* value_bytes,
                                             int32_t* index_bytes_mul, int32_t* index_bytes_adj,
                                             int32_t* panels_mul, int32_t* panels_adj);

/* Per-kernel-class CUDA-event timing of compute calls, off by default.
 * Classes: 0 SpMV multiply, 1 SpMV adjoint, 2 reorthogonalization,
 * 3 restart (small SVD), 4 rotation, 5 other. */
void irlba_gb300_set_profiling(int32_t on);
void irlba_gb300_last_profile(double* ms, int64_t* launches);

/* Kernels launched by this library since the process started. */
int64_t irlba_gb300_launch_count(void);

/* Bytes this library copied host-to-device and device-to-host since the
 * process started (either pointer may be NULL). */
void irlba_gb300_transfer_bytes(int64_t* h2d, int64_t* d2h);

/* ------------------------------------------------------------------------
 * Differentiation form. No counterpart in the reference (irlba::compute has
 * no derivative). For the top-k SVD A' ~ U diag(S) V^T computed on `matrix`
 * (an undecorated matrix or its centre/scale chain) and the cotangents gU
 * (m x k), gS (k), gV (n x k) of a scalar loss, the gradient with respect to
 * A' is the rank-2k product Z1 Z2^T. U, V, gU, gV are column-major (ld m / n)
 * FP64 device arrays, S and gS FP64 device vectors; gU, gS or gV may be NULL
 * (zero). The in-subspace terms are Townsend's F-matrix terms; the terms in
 * the orthogonal complement of U and V are solved exactly by shifted
 * conjugate gradients on the device to relative residual cg_tol (which needs
 * S[k-1] above the (k+1)-th singular value); cg_tol < 0 uses the rank-k
 * projection terms (I - UU^T) gU S^-1 V^T + U S^-1 gV^T (I - VV^T) instead,
 * exact only when A' has rank k. k <= 64.
 * ---------------------------------------------------------------------- */

/* Z1 (m x 2k) and Z2 (n x 2k), row-major FP64 device arrays. */
irlba_gb300_status irlba_gb300_svd_adjoint_factors(const irlba_gb300_matrix* matrix, int64_t k, const double* U,
                                                   const double* S, const double* V, const double* gU,
                                                   const double* gS, const double* gV, double cg_tol,
                                                   int32_t cg_max_iter, double* Z1, double* Z2,
                                                   int32_t* cg_iterations, void* stream);

/* grad = Z1 Z2^T as a dense m x n device array of `type` (row-major when
 * row_major, else column-major; leading dimension ld). */
irlba_gb300_status irlba_gb300_svd_adjoint_dense(int64_t m, int64_t n, int64_t k, const double* Z1, const double* Z2,
                                                 void* grad, int64_t ld, int32_t row_major,
                                                 irlba_gb300_value_type type, void* stream);

/* Gradient with respect to the stored values of a sparse input (the same
 * compressed layout as irlba_gb300_matrix_create_sparse, as device arrays):
 * Z1 Z2^T sampled on the sparsity pattern (SDDMM) and carried back through the
 * chain of `matrix`: column scaling divides (or multiplies) by the scale, a
 * constant centre adds nothing. statistics = 1 treats the centre and scale as
 * pca()'s column means and standard deviations of these values
 * (pca.hpp:85-109) and adds their derivatives. grad_values has the input's
 * value type. */
irlba_gb300_status irlba_gb300_svd_adjoint_sparse(const irlba_gb300_matrix* matrix, int64_t k, const double* Z1,
                                                  const double* Z2, const int64_t* pointers, const int32_t* indices,
                                                  const void* values, irlba_gb300_value_type type,
                                                  int32_t column_major, int32_t statistics, void* grad_values,
                                                  void* stream);

/* ------------------------------------------------------------------------
 * Batched form. No counterpart in the reference, which solves one matrix per
 * irlba::pca call (pca.hpp:55-139): a batch holds many independent sparse
 * matrices on the device and solves them all with the same arguments, as a
 * loop of irlba::pca(matrix_j, center, scale, number, options) would, in one
 * persistent kernel launch replayed from a captured CUDA graph (one CTA per
 * matrix, largest first; FP32 matrices and bases with FP64 recurrence, small
 * SVD and convergence test). Large matrices are shared by a team of CTAs (a
 * thread-block cluster). The gather schedule of each matrix's SpMVs (lanes per
 * row, L2 prefetch distance) is picked by an autotuner that times the
 * candidates on the device.
 * Matrices whose iterations hit an invariant subspace, or whose arguments need
 * the exact SVD or a working subspace above 32, are solved by the
 * single-matrix FP32 form instead (status IRLBA_GB300_BATCH_SINGLE).
 * ---------------------------------------------------------------------- */
typedef struct irlba_gb300_batch irlba_gb300_batch;

enum {
    IRLBA_GB300_BATCH_OK = 0,      /* solved by the batched kernel */
    IRLBA_GB300_BATCH_SINGLE = 1,  /* solved by the single-matrix engine */
    IRLBA_GB300_BATCH_FAILED = 2   /* the single-matrix engine raised an error */
};

typedef struct {
    int32_t status;          /* IRLBA_GB300_BATCH_* */
    int32_t converged;
    int32_t iterations;      /* restart iterations, as Results::iterations */
    int32_t group_mul;       /* lanes per row of the multiply SpMV */
    int32_t group_adj;       /* lanes per row of the adjoint SpMV */
    int32_t prefetch_mul;    /* row batches prefetched into L2 ahead, multiply */
    int32_t prefetch_adj;    /* same, adjoint */
    int32_t error;           /* irlba_gb300_status of a failed single-matrix solve */
    int32_t reserved0;
    int64_t lanczos_steps;
    int64_t svd_sweeps;
    double ms;               /* device time of this matrix on its CTA */
} irlba_gb300_batch_info;

typedef struct {
    double device_ms;        /* CUDA-event time of the graph launch */
    double tune_ms;          /* autotuner time in this call (0 when cached) */
    double single_ms;        /* time spent in single-matrix solves */
    int64_t kernel_launches; /* kernels this library launched during the call */
    int32_t graph_captured;  /* 1 if this call captured a new graph */
    int32_t single;          /* matrices solved by the single-matrix engine */
    int32_t ctas;            /* CTAs of the persistent launch */
    int32_t team;            /* CTAs per team (a thread-block cluster) */
    int32_t joint;           /* matrices solved by a whole team */
    int32_t reserved0;
    int64_t nnz;             /* stored entries over all matrices (one direction) */
    int64_t lanczos_steps;   /* summed over the batched matrices */
} irlba_gb300_batch_stats;

/* count matrices; matrix j is nrow[j] x ncol[j] in compressed form (as
 * irlba_gb300_matrix_create_sparse), values FP32 or FP64 (stored as FP32). */
irlba_gb300_status irlba_gb300_batch_create(int32_t count, const int64_t* nrow, const int64_t* ncol,
                                            const void* const* values, irlba_gb300_value_type value_type,
                                            const int32_t* const* indices, const int64_t* const* pointers,
                                            int32_t column_major, irlba_gb300_batch** out);
irlba_gb300_status irlba_gb300_batch_destroy(irlba_gb300_batch* batch);

/* Runs the autotuner now (otherwise the first solve does): `repeats` timed
 * SpMVs per candidate schedule (lanes per row 4/8/16/32 x L2 prefetch
 * distance 0/1/3 row batches) and direction. */
irlba_gb300_status irlba_gb300_batch_tune(irlba_gb300_batch* batch, int32_t repeats, void* stream);
/* Teams of CTAs (thread-block clusters of `team` = 1, 2, 4 or 8 CTAs; 0, the
 * default, picks per call the size with the smallest estimated makespan). A
 * team solves each of the `joint` largest matrices together and the others
 * one matrix per CTA; joint < 0 (default) picks the matrices whose cost
 * exceeds half of the average per-CTA load. */
irlba_gb300_status irlba_gb300_batch_set_team(irlba_gb300_batch* batch, int32_t team, int32_t joint);
/* Lanes per row chosen for each matrix (arrays of `count`, either may be NULL). */
irlba_gb300_status irlba_gb300_batch_groups(const irlba_gb300_batch* batch, int32_t* group_mul,
                                            int32_t* group_adj);
/* Fixes the lanes per row (4, 8, 16 or 32) instead of tuning; NULL keeps a direction's choice. */
irlba_gb300_status irlba_gb300_batch_set_groups(irlba_gb300_batch* batch, const int32_t* group_mul,
                                                const int32_t* group_adj);

/* pca() of every matrix, results kept on the device (fetch them with
 * irlba_gb300_batch_result / _result_device). Issued on `stream` (NULL = an
 * internal stream); returns when all results are complete. */
irlba_gb300_status irlba_gb300_batch_pca(irlba_gb300_batch* batch, int32_t center, int32_t scale, int64_t number,
                                         const irlba_gb300_options* options, irlba_gb300_batch_stats* stats,
                                         void* stream);

/* Results of matrix `index` of the last batch_pca, copied to host memory:
 * scores (nrow x number), rotation (ncol x number), variances (number),
 * center and scale (ncol, when requested); any pointer may be NULL. */
irlba_gb300_status irlba_gb300_batch_result(const irlba_gb300_batch* batch, int32_t index, double* scores,
                                            double* rotation, double* variances, double* center, double* scale,
                                            irlba_gb300_batch_info* info);
/* Device addresses of the same results (valid until the next batch_pca or destroy). */
irlba_gb300_status irlba_gb300_batch_result_device(const irlba_gb300_batch* batch, int32_t index,
                                                   const double** scores, const double** rotation,
                                                   const double** variances);

#ifdef __cplusplus
}
#endif

#endif /* IRLBA_GB300_H */
