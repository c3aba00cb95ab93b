// Kernel launchers of the GB300 IRLBA engine (host-callable, C++ linkage).
#pragma once

#include "common.cuh"

namespace irlba_gb300 {

// Threads per CTA of the SpMV kernels.
constexpr int kSpmvThreads = 256;

// One gather direction of a sparse operator, stored as a "panel CSR":
// the input vector x (length ncols) is split into npanels column panels of
// panel_width entries; segment (p, r) holds the entries of output row r whose
// column falls in panel p, in panel-major order. Output
//   y[r] = sum_p sum_{s in segment(p, r)} val[s] * x[p * panel_width + idx[s]].
// staged = 1: the panel of x is copied to shared memory and idx16 holds the
// column offset within the panel (u16). staged = 0: a single panel, x is
// gathered from global memory, idx32 holds the column.
struct DirPlanDev {
    int64_t nrows = 0;
    int64_t ncols = 0;
    int64_t nnz = 0;
    int32_t npanels = 1;
    int32_t staged = 0;
    int64_t panel_width = 0;
    int64_t nseg = 0;
    const int64_t* segptr = nullptr;   // nseg + 1
    const uint16_t* idx16 = nullptr;
    const int32_t* idx32 = nullptr;
    const void* val = nullptr;
    int32_t val_f64 = 0;
    int32_t nblocks = 0;
    const int64_t* block_seg = nullptr;  // nblocks + 1 segment boundaries per CTA
    size_t smem_bytes = 0;
    int32_t group_lanes = 32;            // lanes per segment: 4, 8, 16 or 32
    int32_t shape = 0;                   // launch shape of the kernel (see spmv_shape_threads)
    // Dictionary-coded values (FP32 staged plans with at most kMaxDict distinct
    // values): entry i's value is dict[code[i]], the dictionary staged in shared
    // memory at float offset dict_offset (smem_bytes includes it). NULL: val.
    const uint16_t* code = nullptr;
    const float* dict = nullptr;
    int32_t ndict = 0;
    int32_t dict_offset = 0;
};
// Largest dictionary of a coded plan.
constexpr int32_t kMaxDict = 2048;
// Threads per CTA of an SpMV launch shape.
int spmv_shape_threads(int shape);

// Fused prologue/epilogue of a matvec (deferred centring and scaling, and the
// Lanczos axpy). With acc the raw sparse product of row r:
//   v = acc
//   if (beta && !center_after) v -= *beta * (cvec ? cvec[r] : 1)
//   if (oscale)               v = odivide ? v / oscale[r] : v * oscale[r]
//   if (beta && center_after)  v -= *beta * (cvec ? cvec[r] : 1)
//   if (alpha)                v -= *alpha * q[r]
// The prologue scales x while staging: x'[c] = idivide ? x[c] / iscale[c] : x[c] * iscale[c].
template <typename T>
struct Epilogue {
    const double* beta = nullptr;
    const T* cvec = nullptr;
    int32_t center_after = 0;
    const T* oscale = nullptr;
    int32_t odivide = 0;
    const double* alpha = nullptr;
    const T* q = nullptr;
    const T* iscale = nullptr;
    int32_t idivide = 0;
};

template <typename T>
void launch_spmv(const DirPlanDev& p, const T* x, T* y, T* partial, const Epilogue<T>& e, const int32_t* abort,
                 cudaStream_t stream);

// The epilogue alone, applied in place to y (the raw product of a user-defined
// operator); a no-op when e has no beta, oscale or alpha.
template <typename T>
void launch_epilogue(T* y, int64_t nrows, const Epilogue<T>& e, const int32_t* abort, cudaStream_t stream);

// Launch configuration helpers (dynamic shared-memory limits, occupancy, grids).
cudaError_t spmv_configure(size_t max_smem);
int spmv_blocks_per_sm(bool staged, bool vf64, bool tf64, size_t smem, int group, int shape = 0, bool coded = false);
cudaError_t rotate_configure(size_t max_smem);
// The restart rotations on the tensor cores (rotate_tc.cu): w, k <= 64, FP32
// (three BF16 slices) and FP64 (seven) forms; out may be Q (rows are read
// before they are written). error_flag NULL: a module-wide flag.
cudaError_t rotate_tc_configure(size_t max_smem);
bool rotate_tc32_available();
bool rotate_tc64_available();
size_t rotate_tc32_smem_bytes();
size_t rotate_tc64_smem_bytes();
void launch_rotate_tc32(const float* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                        float* out, int64_t ldo, const float* fcol, const double* fnorm, const int32_t* abort,
                        int32_t* error_flag, int sms, cudaStream_t stream);
void launch_rotate_tc64(const double* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                        double* out, int64_t ldo, const double* fcol, const double* fnorm, const int32_t* abort,
                        int32_t* error_flag, int sms, cudaStream_t stream);
// Engine of the restart rotations with w, k <= 64: 1 = tensor cores (default), 0 = CUDA cores.
void set_rotate_engine(int engine);
int rotate_engine();
// 1 if a tensor-core rotation since the last call gave up on a bounded wait
// (its output is invalid), 0 if none did, -1 if the flag could not be read.
int rotate_tc_take_error();
int cgs_update_grid(int64_t L);
int cgs_dot_grid(int64_t L);

// out = prologue-scaled copy of x (used when x is not staged in shared memory).
template <typename T>
void launch_scale_vector(const T* x, const T* s, int32_t divide, int64_t n, T* out, cudaStream_t stream);

// t[j] = sum_r Q[r, j] v[r] for j < c (FP64 accumulation); part: >= grid*c scratch.
template <typename T>
void launch_cgs_dot(const T* Q, int64_t L, int64_t ldq, int32_t c, const T* v, double* part, double* t, Ctrl* ctrl,
                    cudaStream_t stream);

// v -= Q[:, :c] t; then norm = ||v|| -> *norm_out (FP64); flags invariant if
// check_eps and norm < ctrl->eps; null_start is raised instead when
// check_null. When write_B >= 0, B[write_B] = *b_value (a device scalar) first.
template <typename T>
void launch_cgs_update(const T* Q, int64_t L, int64_t ldq, int32_t c, const double* t, T* v, double* part,
                       double* norm_out, int32_t check_eps, int32_t check_null, Ctrl* ctrl, cudaStream_t stream);

// v *= 1 / *norm; Q[:, col] = v (col >= 0); beta_out = sum f(v[i]) g[i] where
// f applies the optional scale vector s (divide or multiply) and g is the
// optional centre vector (NULL = 1). When bpos >= 0 also writes B[bpos] = S and
// B[bpos + ldb] = R_F (the bidiagonal entries of the step).
template <typename T>
void launch_normalize(T* v, int64_t L, const double* norm, T* qcol, const T* fscale, int32_t fdivide,
                      const T* gvec, double* beta_out, double* part, double* B, int64_t bpos, int64_t ldb,
                      Ctrl* ctrl, cudaStream_t stream);

// beta_out = sum f(x[i]) g[i] (no normalization).
template <typename T>
void launch_beta(const T* x, int64_t L, const T* fscale, int32_t fdivide, const T* gvec, double* beta_out,
                 double* part, Ctrl* ctrl, cudaStream_t stream);

// out[:, :k] = Q[:, :w] R[:, :k] row by row (in place allowed when out == Q);
// R is FP64 column-major w x w (ld ldr). If fcol != NULL also sets
// out[:, k] = fcol / *fnorm.
template <typename T>
void launch_rotate(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k, T* out,
                   int64_t ldo, const T* fcol, const double* fnorm, const int32_t* abort, cudaStream_t stream);

// Same, on the CUDA cores whatever the rotation engine setting.
template <typename T>
void launch_rotate_cores(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                         T* out, int64_t ldo, const T* fcol, const double* fnorm, const int32_t* abort,
                         cudaStream_t stream);

// Same, writing FP64 output (the final U and V).
template <typename T>
void launch_rotate_out(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                       double* out, int64_t ldo, cudaStream_t stream);

// Elementwise copy with conversion.
template <typename A, typename B>
void launch_convert(const A* in, B* out, int64_t n, cudaStream_t stream);

// Dense column-major realization of one direction plan (rows x cols of the plan).
void launch_realize(const DirPlanDev& p, double* out, int64_t ld, int32_t transpose, cudaStream_t stream);

// Centre / scale applied to a realized column-major m x n matrix.
void launch_realize_ops(double* A, int64_t m, int64_t n, const double* center, const double* scale,
                        int32_t scale_column, int32_t scale_divide, int32_t center_outer, cudaStream_t stream);

// Column sums and sums of squared deviations of the matrix whose gather plan
// over features is `p` (rows of p = features): mean[f] = sum / nobs,
// var[f] = (sum (x - mean)^2 + (nobs - nnz_f) mean^2) / (nobs - 1).
void launch_feature_stats(const DirPlanDev& p, int64_t nobs, int32_t center, int32_t scale, double* center_out,
                          double* scale_out, double* scratch, cudaStream_t stream);

// Restart of the IRLBA loop on the device (compute.hpp:225-293): SVD of B,
// convergence test, update_k, and B rebuilt for the next Lanczos run.
struct RestartArgs {
    double* B;          // work x work, column-major
    double* BS;         // work
    double* BU;         // work x work
    double* BV;         // work x work
    double* prevS;      // work
    double* res;        // work
    double* scratch;    // >= restart_smem_bytes(work) bytes, used when they exceed shared memory
    int32_t work;
    int32_t k;          // start column of the run that produced B
    int32_t requested;
    int32_t iter;
    double tol;
    double svtol;
    Ctrl* ctrl;
};
void launch_restart(const RestartArgs& a, cudaStream_t stream, size_t max_smem);
// The convergence test, update_k and the rebuild of B alone, given BS, BU, BV.
void launch_restart_tail(const RestartArgs& a, cudaStream_t stream);
// out[i] = the restart kernel's update_k(args[4i], args[4i+1], args[4i+2], args[4i+3])
// (k, requested, n_converged, work), compute.hpp:78-111.
void launch_update_k(const int32_t* args, int64_t count, int32_t* out, cudaStream_t stream);
size_t restart_smem_bytes(int work);
cudaError_t restart_configure(size_t max_smem);

// Thin SVD of a dense column-major m x n matrix with m >= n (one-sided Jacobi):
// U m x n, S n (descending), V n x n. scratch >= m*n + n*n doubles.
void launch_dense_svd(const double* A, int64_t m, int64_t n, double* U, double* S, double* V, double* scratch,
                      Ctrl* ctrl, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Batched form (batch.cu): one persistent launch solves many independent
// centred/scaled sparse PCAs in the FP32 form, one team of CTAs per problem.
// ---------------------------------------------------------------------------
// One gather direction of one problem: plain CSR over `rows` output entries.
// Row 0 of ptr starts at a multiple of 4 entries (16-byte aligned values).
struct BatchDir {
    int64_t rows = 0;
    int64_t cols = 0;                  // length of the gathered vector
    const int64_t* ptr = nullptr;      // rows + 1 absolute offsets into idx / val
    const void* idx = nullptr;         // u16 columns when staged, int32 otherwise
    const float* val = nullptr;
    int32_t staged = 0;                // gathered vector copied to shared memory
    int32_t group = 32;                // lanes per row: 4, 8, 16 or 32
    int32_t prefetch = 0;              // row batches bulk-prefetched into L2 ahead (0 = off)
    int32_t idx_bytes = 2;             // 2 (u16, staged) or 4 (int32)
};

struct BatchProblem {
    int64_t m = 0, n = 0;              // rows (observations), columns (features)
    BatchDir mul;                      // rows = m, gathers x (n)
    BatchDir adj;                      // rows = n, gathers y (m)
    float* V = nullptr;                // n x work, ld ldv
    int64_t ldv = 0;
    float* W = nullptr;                // m x work, ld ldw
    int64_t ldw = 0;
    float* F = nullptr;                // n
    float* Wn = nullptr;               // m
    float* xs = nullptr;               // n: scaled x when the multiply is not staged
    float* center = nullptr;           // n, FP32 copies used by the matvecs
    float* scale = nullptr;            // n
    double* center64 = nullptr;        // n, FP64 column statistics (outputs)
    double* scale64 = nullptr;         // n
    const double* init = nullptr;      // n, start vector
    double* scores = nullptr;          // m x number (ld m)
    double* rotation = nullptr;        // n x number (ld n)
    double* variances = nullptr;       // number
};

struct BatchParams {
    int32_t number = 0;
    int32_t work = 0;
    int32_t max_iter = 0;
    int32_t center = 0;
    int32_t scale = 0;
    double tol = 0;
    double svtol = 0;
    double eps = 0;
};

// status: 0 = finished (converged or out of iterations), 2 = a Lanczos norm
// fell below the invariant-subspace tolerance (re-solved by the caller).
struct BatchResult {
    int32_t status = 0;
    int32_t converged = 0;
    int32_t iterations = 0;
    int32_t svd_sweeps = 0;
    int64_t steps = 0;
    uint64_t t_start = 0;              // %globaltimer (ns) when the CTA took the problem
    uint64_t t_end = 0;
};

// ---------------------------------------------------------------------------
// Device-side ingestion (ingest.cu): compressed arrays -> gather plans.
// ---------------------------------------------------------------------------
// flags[1] index out of range, flags[2] unsorted row (pointers checked by the caller).
void launch_validate(int64_t rows, int64_t cols, int64_t nnz, const int64_t* ptr, const int32_t* idx,
                     int32_t* flags, cudaStream_t s);
// Exclusive scan of n int64 (out may alias in); *total = sum; scratch >= scan_scratch_elems(n).
size_t scan_scratch_elems(int64_t n);
void launch_exclusive_scan(const int64_t* in, int64_t n, int64_t* out, int64_t* total, int64_t* scratch,
                           cudaStream_t s);
// Stable transpose over chunks of input rows (chunk_rows: nchunks + 1 boundaries).
void launch_transpose_count(const int64_t* ptr, const int32_t* idx, const int64_t* chunk_rows, int nchunks,
                            int64_t cols, int32_t* count, cudaStream_t s);
void launch_transpose_totals(const int32_t* count, int nchunks, int64_t cols, int64_t* tot, cudaStream_t s);
void launch_transpose_cursors(const int32_t* count, int nchunks, int64_t cols, const int64_t* tptr, int64_t* cursor,
                              cudaStream_t s);
void launch_transpose_scatter(const int64_t* ptr, const int32_t* idx, const void* val, bool in_f64,
                              const int64_t* chunk_rows, int nchunks, int64_t cols, int64_t* cursor, int32_t* tidx,
                              void* tval, bool out_f64, cudaStream_t s);
// Panel layout of sorted rows: counts per (panel, row), then the panel-major copy.
void launch_panel_count(int64_t rows, int32_t npanels, int64_t pw, const int64_t* ptr, const int32_t* idx,
                        int64_t* cnt, cudaStream_t s);
void launch_panel_scatter(int64_t rows, int32_t npanels, int64_t pw, const int64_t* ptr, const int32_t* idx,
                          const void* val, bool in_f64, const int64_t* segptr, uint16_t* idx16, void* vout,
                          bool out_f64, cudaStream_t s);
void launch_copy_entries(int64_t nnz, const int32_t* idx, const void* val, bool in_f64, uint16_t* idx16,
                         int32_t* idx32, void* vout, bool out_f64, cudaStream_t s);
void launch_block_seg(const int64_t* segptr, int64_t nseg, int64_t cost, int64_t nblocks, int64_t* bseg,
                      cudaStream_t s);
// Value dictionary (ingest.cu): hash set of 2^log2h slots (zeroed by the
// caller), count of distinct values (overflow set beyond maxd or when full),
// compaction into codes and dictionary, and the encoding of a value array.
void launch_dict_insert(const float* val, int64_t n, unsigned long long* slots, int log2h, uint32_t* count,
                        int32_t* overflow, uint32_t maxd, cudaStream_t s);
void launch_dict_compact(const unsigned long long* slots, int log2h, uint16_t* slot_code, float* dict,
                         cudaStream_t s);
size_t dict_encode_smem(int log2h);
void launch_dict_encode(const float* val, int64_t n, const unsigned long long* slots, const uint16_t* slot_code,
                        int log2h, uint16_t* code, cudaStream_t s);

// ---------------------------------------------------------------------------
// Differentiation form (adjoint.cu). Blocks are row-major FP64 with k <= 64
// columns; Z1 and Z2 have kk = 2k <= 128.
// ---------------------------------------------------------------------------
constexpr int kAdjointMaxK = 64;
// Y (plan rows x k) = plan * X (plan cols x k), k <= 128.
void launch_spmm(const DirPlanDev& p, const double* X, int k, double* Y, cudaStream_t s);
// Partial-buffer length (in units of k*k doubles) the reductions below need.
int gram_parts(int64_t L);
// out (k x k, [a * k + b]) = P^T Q over L rows; part >= gram_parts(L) * k * k doubles.
void launch_gram(const double* P, const double* Q, int64_t L, int k, double* part, double* out, cudaStream_t s);
// out[c] = sum_r w(r) P[r, c] (Q ? Q[r, c] : 1), k <= 128; part >= gram_parts(L) * k doubles.
void launch_coldot(const double* P, const double* Q, const double* weight, int64_t L, int k, double* part, double* out,
                   cudaStream_t s);
// out = alpha * A R + beta * diag(bs) B (per column); out may alias B.
void launch_block_update(int64_t L, int ka, int kout, const double* A, int64_t lda, const double* R, double alpha,
                         const double* B, int64_t ldb, const double* bs, double beta, double* out, int64_t ldo,
                         cudaStream_t s);
void launch_rank1(int64_t L, int k, const double* a, const double* b, double coef, double* Y, cudaStream_t s);
void launch_scale_rows(int64_t L, int k, const double* X, const double* sv, int divide, double* out, cudaStream_t s);
void launch_cg_step(int64_t L, int k, const double* alpha, const double* P, const double* Q, double* X, double* R,
                    cudaStream_t s);
void launch_cg_dir(int64_t L, int k, const double* beta, const double* R, double* P, cudaStream_t s);
// Device-side CG scalars (k <= kAdjointMaxK): st[0] columns active, st[1]
// non-positive curvature met, st[2] iterations with an active column.
void launch_cg_init(int k, const double* rr0, double* rr, double* bnorm, int32_t* active, int32_t* st,
                    cudaStream_t s);
void launch_cg_alpha(int k, const double* pq, const double* rr, const int32_t* active, double* alpha, int32_t* st,
                     cudaStream_t s);
void launch_cg_beta(int k, const double* rn, double* rr, const double* bnorm, double tol, int32_t* active,
                    double* beta, int32_t* st, cudaStream_t s);

void launch_shift(int64_t L, int k, const double* shift, const double* P, const double* W, double* Q, cudaStream_t s);
void launch_to_rows(int64_t L, int k, const double* src, int64_t ld, double* out, cudaStream_t s);
// d[r] = coef * X[r, :] . (Y ? Y[r, :] : y)
void launch_rowdot(int64_t L, int k, const double* X, const double* Y, const double* y, double coef, double* d,
                   cudaStream_t s);
void launch_outer(int64_t m, int64_t n, int kk, const double* Z1, const double* Z2, void* G, int64_t ldg,
                  int row_major, int f64, cudaStream_t s);
void launch_sddmm(int64_t nprimary, const int64_t* ptr, const int32_t* idx, const void* vals, int f64,
                  int column_major, const double* Z1, const double* Z2, int kk, const double* f, const double* cmean,
                  const double* c, const double* qf, void* grad, cudaStream_t s);

constexpr int kBatchMaxWork = 32;
// Largest gathered vector that a batched SpMV stages in shared memory (floats).
int64_t batch_stage_limit();
// Dynamic shared memory of the batched kernels for a given largest staged vector.
size_t batch_smem_bytes(int64_t max_staged);
cudaError_t batch_configure(size_t max_smem_optin);
// Teams of `team` CTAs (a thread-block cluster; 1, 2, 4 or 8) that can be
// resident at once with `smem` bytes of dynamic shared memory (0 on error).
int batch_max_teams(int team, size_t smem);
// `teams` teams of `team` CTAs take the `count` problems of `order` in turn:
// the first n_joint each by a whole team, the rest one CTA each.
void launch_batch_pca(int team, const BatchProblem* probs, const int32_t* order, int32_t count, int32_t n_joint,
                      const BatchParams& prm, BatchResult* results, uint32_t* queue, int teams, size_t smem,
                      cudaStream_t stream);
// Autotuner probe: CTAs take the problems in `order` and time `reps` SpMVs of
// each (direction adjoint, `group` lanes per row, `prefetch` row batches of L2
// prefetch), writing the best time in SM cycles to cycles_out[problem]. Uses
// the problems' xs/Wn/F as scratch.
void launch_batch_spmv_probe(const BatchProblem* probs, const int32_t* order, int32_t count, int32_t adjoint,
                             int32_t group, int32_t prefetch, int32_t reps, uint64_t* cycles_out, int grid,
                             size_t smem, cudaStream_t stream);

}  // namespace irlba_gb300
