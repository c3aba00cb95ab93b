// Device kernels of the differentiation form (truncated-SVD adjoint).
//
// The adjoint of A -> (U, S, V) (top-k SVD) is assembled as a rank-2k product
// dL/dA = Z1 Z2^T (Z1 m x 2k, Z2 n x 2k, row-major FP64); building Z1 and Z2
// needs small Gram matrices, products of the operator with k-column blocks
// (SpMM over the engine's gather plans) and per-column conjugate-gradient
// updates. The gradient is then either the dense product Z1 Z2^T or, for a
// sparse input, its values on the sparsity pattern (SDDMM) carried back
// through pca()'s column centring and scaling. All block arrays here are
// row-major with k <= 64 columns (kk = 2k <= 128 for Z1, Z2; the SpMM and the
// column reductions take up to 128 columns).

#include "kernels.cuh"

namespace irlba_gb300 {

namespace {

constexpr int kT = 256;

// Y (rows x k) = plan * X (cols x k), k <= 128; one warp per output row, lane
// l accumulates columns l, l + 32, l + 64, l + 96; the row's entries are
// broadcast 32 at a time.
template <typename VT>
__global__ void __launch_bounds__(kT) spmm_kernel(const DirPlanDev p, const double* __restrict__ X, int k,
                                                  double* __restrict__ Y) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const VT* __restrict__ val = static_cast<const VT*>(p.val);
    for (int64_t r = gw; r < p.nrows; r += nw) {
        double acc[4] = {0, 0, 0, 0};
        for (int32_t pn = 0; pn < p.npanels; ++pn) {
            const int64_t seg = pn * p.nrows + r;
            const int64_t b = p.segptr[seg], e = p.segptr[seg + 1];
            const int64_t base = pn * p.panel_width;
            for (int64_t s0 = b; s0 < e; s0 += 32) {
                const int64_t s = s0 + lane;
                double v = 0;
                int64_t c = 0;
                if (s < e) {
                    v = static_cast<double>(val[s]);
                    c = p.staged ? base + p.idx16[s] : static_cast<int64_t>(p.idx32[s]);
                }
                const int cnt = static_cast<int>(e - s0 < 32 ? e - s0 : 32);
                for (int t = 0; t < cnt; ++t) {
                    const double vt = __shfl_sync(0xffffffffu, v, t);
                    const int64_t ct = __shfl_sync(0xffffffffu, c, t);
                    const double* xr = X + ct * k;
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (lane + 32 * q < k) acc[q] = fma(vt, xr[lane + 32 * q], acc[q]);
                }
            }
        }
        double* yr = Y + r * k;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (lane + 32 * q < k) yr[lane + 32 * q] = acc[q];
    }
}

// Partial Gram matrices: part[blk][a * k + b] = sum over the block's rows of
// P[r, a] Q[r, b] (P, Q: L x k row-major). 16 x 16 threads, 4 x 4 entries each.
__global__ void __launch_bounds__(kT) gram_kernel(const double* __restrict__ P, const double* __restrict__ Q,
                                                  int64_t L, int k, int64_t rows_per_block, double* part) {
    __shared__ double sp[16][64];
    __shared__ double sq[16][64];
    const int tid = threadIdx.x;
    const int ta = tid / 16, tb = tid % 16;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0;
    const int64_t r0 = blockIdx.x * rows_per_block;
    const int64_t r1 = min(L, r0 + rows_per_block);
    for (int64_t rb = r0; rb < r1; rb += 16) {
        for (int e = tid; e < 16 * 64; e += kT) {
            const int rr = e / 64, cc = e % 64;
            const int64_t r = rb + rr;
            const bool ok = r < r1 && cc < k;
            sp[rr][cc] = ok ? P[r * k + cc] : 0.0;
            sq[rr][cc] = ok ? Q[r * k + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int rr = 0; rr < 16; ++rr) {
            double pa[4], qb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                pa[i] = sp[rr][ta * 4 + i];
                qb[i] = sq[rr][tb * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(pa[i], qb[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int a = ta * 4 + i, b = tb * 4 + j;
            if (a < k && b < k) part[blockIdx.x * static_cast<int64_t>(k) * k + a * k + b] = acc[i][j];
        }
}

// Partial column reductions (k <= 128): part[blk][c] = sum over the block's
// rows of w(r) * P[r, c] * (Q ? Q[r, c] : 1), w(r) = weight ? weight[r] : 1.
__global__ void __launch_bounds__(kT) coldot_kernel(const double* __restrict__ P, const double* __restrict__ Q,
                                                    const double* __restrict__ weight, int64_t L, int k,
                                                    int64_t rows_per_block, double* part) {
    __shared__ double red[4][128];
    const int c0 = threadIdx.x % 64, rg = threadIdx.x / 64;
    const int64_t r0 = blockIdx.x * rows_per_block;
    const int64_t r1 = min(L, r0 + rows_per_block);
    for (int c = c0; c < 128; c += 64) {
        double acc = 0;
        if (c < k) {
            for (int64_t r = r0 + rg; r < r1; r += 4) {
                double v = P[r * k + c];
                if (Q) v *= Q[r * k + c];
                if (weight) v *= weight[r];
                acc += v;
            }
        }
        red[rg][c] = acc;
    }
    __syncthreads();
    if (rg == 0)
        for (int c = c0; c < k; c += 64)
            part[blockIdx.x * static_cast<int64_t>(k) + c] = ((red[0][c] + red[1][c]) + red[2][c]) + red[3][c];
}

// out[e] = sum_p part[p * len + e] (fixed order).
__global__ void sum_partials_kernel(const double* __restrict__ part, int nparts, int64_t len, double* __restrict__ out) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < len;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double s = 0;
        for (int p = 0; p < nparts; ++p) s += part[p * len + e];
        out[e] = s;
    }
}

// out[r, c] = alpha * sum_j A[r, j] R[j, c] + beta * (bs ? bs[c] : 1) * B[r, c]
// for c < kout; A (L x ka, ld lda), B and out (ld ldb, ldo). out may alias B.
__global__ void __launch_bounds__(kT) block_update_kernel(int64_t L, int ka, int kout, const double* __restrict__ A,
                                                          int64_t lda, const double* __restrict__ R, double alpha,
                                                          const double* B, int64_t ldb, const double* __restrict__ bs,
                                                          double beta, double* out, int64_t ldo) {
    __shared__ double sR[64 * 64];
    if (A && R) {
        for (int e = threadIdx.x; e < ka * kout; e += kT) sR[e] = R[e];
    }
    __syncthreads();
    const int64_t total = L * kout;
    for (int64_t e = blockIdx.x * static_cast<int64_t>(kT) + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * kT) {
        const int64_t r = e / kout;
        const int c = static_cast<int>(e % kout);
        double v = 0;
        if (A && R) {
            const double* ar = A + r * lda;
            for (int j = 0; j < ka; ++j) v = fma(ar[j], sR[j * kout + c], v);
            v *= alpha;
        }
        if (B) v += beta * (bs ? bs[c] : 1.0) * B[r * ldb + c];
        out[r * ldo + c] = v;
    }
}

// Y[r, c] += coef * (a ? a[r] : 1) * b[c]
__global__ void rank1_kernel(int64_t L, int k, const double* __restrict__ a, const double* __restrict__ b, double coef,
                             double* Y) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < L * k;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = e / k;
        const int c = static_cast<int>(e % k);
        Y[e] += coef * (a ? a[r] : 1.0) * b[c];
    }
}

// out[r, :] = X[r, :] / s[r] (divide) or * s[r]
__global__ void scale_rows_kernel(int64_t L, int k, const double* __restrict__ X, const double* __restrict__ s,
                                  int divide, double* out) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < L * k;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = e / k;
        out[e] = divide ? X[e] / s[r] : X[e] * s[r];
    }
}

// Per-column CG updates: X += alpha * P; R -= alpha * Q (alpha per column).
__global__ void cg_step_kernel(int64_t L, int k, const double* __restrict__ alpha, const double* __restrict__ P,
                               const double* __restrict__ Q, double* X, double* R) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < L * k;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double a = alpha[e % k];
        X[e] = fma(a, P[e], X[e]);
        R[e] = fma(-a, Q[e], R[e]);
    }
}

// P = R + beta * P (beta per column).
__global__ void cg_dir_kernel(int64_t L, int k, const double* __restrict__ beta, const double* __restrict__ R,
                              double* P) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < L * k;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        P[e] = fma(beta[e % k], P[e], R[e]);
}

// Q = shift * P - W (shift per column).
__global__ void shift_kernel(int64_t L, int k, const double* __restrict__ shift, const double* __restrict__ P,
                             const double* __restrict__ W, double* Q) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < L * k;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        Q[e] = shift[e % k] * P[e] - W[e];
}

// CG scalars of the shifted complement solves, kept on the device so the
// iterations run without a host round trip. st: [0] columns still active,
// [1] a non-positive curvature was met, [2] iterations that had an active
// column. One CTA of at least k threads.
__global__ void cg_init_kernel(int k, const double* __restrict__ rr0, double* rr, double* bnorm, int32_t* active,
                               int32_t* st) {
    const int j = threadIdx.x;
    int a = 0;
    if (j < k) {
        rr[j] = rr0[j];
        bnorm[j] = sqrt(rr0[j]);
        a = bnorm[j] > 0;
        active[j] = a;
    }
    a = __syncthreads_or(a);
    if (j == 0) {
        st[0] = a;
        st[1] = 0;
        st[2] = 0;
    }
}

// alpha_j = rr_j / (p_j . q_j) for the active columns, 0 otherwise.
__global__ void cg_alpha_kernel(int k, const double* __restrict__ pq, const double* __restrict__ rr,
                                const int32_t* __restrict__ active, double* alpha, int32_t* st) {
    const int j = threadIdx.x;
    if (j == 0 && st[0]) st[2] += 1;
    if (j >= k) return;
    double a = 0;
    if (active[j]) {
        if (pq[j] > 0) a = rr[j] / pq[j];
        else st[1] = 1;
    }
    alpha[j] = a;
}

// Columns with ||r_j|| <= tol ||b_j|| stop; beta_j = rn_j / rr_j for the rest.
__global__ void cg_beta_kernel(int k, const double* __restrict__ rn, double* rr, const double* __restrict__ bnorm,
                               double tol, int32_t* active, double* beta, int32_t* st) {
    const int j = threadIdx.x;
    int a = 0;
    if (j < k) {
        a = active[j];
        if (a && sqrt(rn[j]) <= tol * bnorm[j]) a = 0;
        active[j] = a;
        beta[j] = a ? rn[j] / rr[j] : 0.0;
        rr[j] = rn[j];
    }
    a = __syncthreads_or(a);
    if (j == 0) st[0] = a;
}

// Column-major (ld) -> row-major (L x k) copy, optional; NULL source gives zeros.
__global__ void to_rows_kernel(int64_t L, int k, const double* __restrict__ src, int64_t ld, double* out) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < L * k;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = e / k;
        const int c = static_cast<int>(e % k);
        out[e] = src ? src[r + c * ld] : 0.0;
    }
}

// d[r] = coef * sum_c X[r, c] * (Y ? Y[r, c] : y[c]) (row-wise dot, X and Y L x k).
__global__ void rowdot_kernel(int64_t L, int k, const double* __restrict__ X, const double* __restrict__ Y,
                              const double* __restrict__ y, double coef, double* d) {
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < L;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double s = 0;
        for (int c = 0; c < k; ++c) s = fma(X[r * k + c], Y ? Y[r * k + c] : y[c], s);
        d[r] = coef * s;
    }
}

// Dense gradient G = Z1 Z2^T (m x n) from row-major Z1 (m x kk), Z2 (n x kk):
// 64 x 64 output tiles, 16 x 16 threads with 4 x 4 outputs, kk in chunks of 16.
template <typename GT>
__global__ void __launch_bounds__(kT) outer_kernel(int64_t m, int64_t n, int kk, const double* __restrict__ Z1,
                                                   const double* __restrict__ Z2, GT* __restrict__ G, int64_t ldg,
                                                   int row_major) {
    __shared__ double s1[16][65];
    __shared__ double s2[16][65];
    const int tid = threadIdx.x;
    // Consecutive threads walk the contiguous dimension of G.
    const int ti = row_major ? tid / 16 : tid % 16;
    const int tj = row_major ? tid % 16 : tid / 16;
    const int64_t i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0;
    for (int l0 = 0; l0 < kk; l0 += 16) {
        for (int e = tid; e < 64 * 16; e += kT) {
            const int rr = e / 16, ll = e % 16;
            const int64_t i = i0 + rr, j = j0 + rr;
            const int l = l0 + ll;
            s1[ll][rr] = (i < m && l < kk) ? Z1[i * kk + l] : 0.0;
            s2[ll][rr] = (j < n && l < kk) ? Z2[j * kk + l] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int ll = 0; ll < 16; ++ll) {
            double x[4], y[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                x[a] = s1[ll][ti + 16 * a];
                y[a] = s2[ll][tj + 16 * a];
            }
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = fma(x[a], y[b], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int64_t i = i0 + ti + 16 * a, j = j0 + tj + 16 * b;
            if (i < m && j < n) {
                if (row_major) G[i * ldg + j] = static_cast<GT>(acc[a][b]);
                else G[i + j * ldg] = static_cast<GT>(acc[a][b]);
            }
        }
}

// Sparse gradient on the input's pattern (SDDMM). Warp per primary element p;
// the primary factor row is staged in shared memory, each lane takes one stored
// entry and forms its 2k-term dot product. With j the column of the entry:
//   g = (t - cmean[j]) * f[j] - (qf ? (A - c[j]) * f[j] * qf[j] : 0)
// where t = Z1[row] . Z2[j], f = 1 / scale (or 1), cmean = column sums of
// Z1 Z2^T over m (or 0), qf = q / ((m - 1) scale) for the scale statistics.
template <typename VT>
__global__ void __launch_bounds__(kT) sddmm_kernel(int64_t nprimary, const int64_t* __restrict__ ptr,
                                                   const int32_t* __restrict__ idx, const VT* __restrict__ vals,
                                                   int column_major, const double* __restrict__ Z1,
                                                   const double* __restrict__ Z2, int kk,
                                                   const double* __restrict__ f, const double* __restrict__ cmean,
                                                   const double* __restrict__ c, const double* __restrict__ qf,
                                                   VT* __restrict__ grad) {
    __shared__ double zp[kT / 32][128];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t gw = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const double* Zp_all = column_major ? Z2 : Z1;
    const double* Zq_all = column_major ? Z1 : Z2;
    for (int64_t p = gw; p < nprimary; p += nw) {
        for (int l = lane; l < kk; l += 32) zp[w][l] = Zp_all[p * kk + l];
        __syncwarp();
        const int64_t b = ptr[p], e = ptr[p + 1];
        for (int64_t s = b + lane; s < e; s += 32) {
            const int64_t q = idx[s];
            const double* zq = Zq_all + q * kk;
            double t = 0;
            for (int l = 0; l < kk; ++l) t = fma(zp[w][l], zq[l], t);
            const int64_t j = column_major ? p : q;
            double g = t;
            if (cmean) g -= cmean[j];
            if (f) g *= f[j];
            if (qf) g -= (static_cast<double>(vals[s]) - (c ? c[j] : 0.0)) * (f ? f[j] : 1.0) * qf[j];
            grad[s] = static_cast<VT>(g);
        }
        __syncwarp();
    }
}

int grid_of(int64_t work, int threads, int cap) {
    int64_t g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return static_cast<int>(g);
}

}  // namespace

void launch_spmm(const DirPlanDev& p, const double* X, int k, double* Y, cudaStream_t s) {
    if (p.nrows == 0) return;
    const int grid = grid_of(p.nrows * 32, kT, 152 * 16);
    if (p.val_f64) spmm_kernel<double><<<grid, kT, 0, s>>>(p, X, k, Y);
    else spmm_kernel<float><<<grid, kT, 0, s>>>(p, X, k, Y);
    count_launch();
}

int gram_parts(int64_t L) { return grid_of(L, 1024, 152 * 2); }

void launch_gram(const double* P, const double* Q, int64_t L, int k, double* part, double* out, cudaStream_t s) {
    const int parts = gram_parts(L);
    const int64_t rows = (L + parts - 1) / parts;
    gram_kernel<<<parts, kT, 0, s>>>(P, Q, L, k, rows < 1 ? 1 : rows, part);
    sum_partials_kernel<<<grid_of(static_cast<int64_t>(k) * k, kT, 64), kT, 0, s>>>(part, parts,
                                                                                static_cast<int64_t>(k) * k, out);
    count_launch(2);
}

void launch_coldot(const double* P, const double* Q, const double* weight, int64_t L, int k, double* part, double* out,
                   cudaStream_t s) {
    const int parts = gram_parts(L);
    const int64_t rows = (L + parts - 1) / parts;
    coldot_kernel<<<parts, kT, 0, s>>>(P, Q, weight, L, k, rows < 1 ? 1 : rows, part);
    sum_partials_kernel<<<1, 128, 0, s>>>(part, parts, k, out);
    count_launch(2);
}

void launch_block_update(int64_t L, int ka, int kout, const double* A, int64_t lda, const double* R, double alpha,
                         const double* B, int64_t ldb, const double* bs, double beta, double* out, int64_t ldo,
                         cudaStream_t s) {
    if (L == 0 || kout == 0) return;
    block_update_kernel<<<grid_of(L * kout, kT, 152 * 8), kT, 0, s>>>(L, ka, kout, A, lda, R, alpha, B, ldb, bs,
                                                                      beta, out, ldo);
    count_launch();
}

void launch_rank1(int64_t L, int k, const double* a, const double* b, double coef, double* Y, cudaStream_t s) {
    if (L == 0) return;
    rank1_kernel<<<grid_of(L * k, kT, 152 * 8), kT, 0, s>>>(L, k, a, b, coef, Y);
    count_launch();
}

void launch_scale_rows(int64_t L, int k, const double* X, const double* sv, int divide, double* out, cudaStream_t s) {
    if (L == 0) return;
    scale_rows_kernel<<<grid_of(L * k, kT, 152 * 8), kT, 0, s>>>(L, k, X, sv, divide, out);
    count_launch();
}

void launch_cg_step(int64_t L, int k, const double* alpha, const double* P, const double* Q, double* X, double* R,
                    cudaStream_t s) {
    cg_step_kernel<<<grid_of(L * k, kT, 152 * 8), kT, 0, s>>>(L, k, alpha, P, Q, X, R);
    count_launch();
}

void launch_cg_init(int k, const double* rr0, double* rr, double* bnorm, int32_t* active, int32_t* st,
                    cudaStream_t s) {
    cg_init_kernel<<<1, kAdjointMaxK, 0, s>>>(k, rr0, rr, bnorm, active, st);
    count_launch();
}

void launch_cg_alpha(int k, const double* pq, const double* rr, const int32_t* active, double* alpha, int32_t* st,
                     cudaStream_t s) {
    cg_alpha_kernel<<<1, kAdjointMaxK, 0, s>>>(k, pq, rr, active, alpha, st);
    count_launch();
}

void launch_cg_beta(int k, const double* rn, double* rr, const double* bnorm, double tol, int32_t* active,
                    double* beta, int32_t* st, cudaStream_t s) {
    cg_beta_kernel<<<1, kAdjointMaxK, 0, s>>>(k, rn, rr, bnorm, tol, active, beta, st);
    count_launch();
}

void launch_cg_dir(int64_t L, int k, const double* beta, const double* R, double* P, cudaStream_t s) {
    cg_dir_kernel<<<grid_of(L * k, kT, 152 * 8), kT, 0, s>>>(L, k, beta, R, P);
    count_launch();
}

void launch_shift(int64_t L, int k, const double* shift, const double* P, const double* W, double* Q, cudaStream_t s) {
    shift_kernel<<<grid_of(L * k, kT, 152 * 8), kT, 0, s>>>(L, k, shift, P, W, Q);
    count_launch();
}

void launch_to_rows(int64_t L, int k, const double* src, int64_t ld, double* out, cudaStream_t s) {
    if (L == 0) return;
    to_rows_kernel<<<grid_of(L * k, kT, 152 * 8), kT, 0, s>>>(L, k, src, ld, out);
    count_launch();
}

void launch_rowdot(int64_t L, int k, const double* X, const double* Y, const double* y, double coef, double* d,
                   cudaStream_t s) {
    if (L == 0) return;
    rowdot_kernel<<<grid_of(L, kT, 152 * 8), kT, 0, s>>>(L, k, X, Y, y, coef, d);
    count_launch();
}

void launch_outer(int64_t m, int64_t n, int kk, const double* Z1, const double* Z2, void* G, int64_t ldg,
                  int row_major, int f64, cudaStream_t s) {
    if (m == 0 || n == 0) return;
    const dim3 grid(static_cast<unsigned>((m + 63) / 64), static_cast<unsigned>((n + 63) / 64));
    if (f64) outer_kernel<double><<<grid, kT, 0, s>>>(m, n, kk, Z1, Z2, static_cast<double*>(G), ldg, row_major);
    else outer_kernel<float><<<grid, kT, 0, s>>>(m, n, kk, Z1, Z2, static_cast<float*>(G), ldg, row_major);
    count_launch();
}

void launch_sddmm(int64_t nprimary, const int64_t* ptr, const int32_t* idx, const void* vals, int f64,
                  int column_major, const double* Z1, const double* Z2, int kk, const double* f, const double* cmean,
                  const double* c, const double* qf, void* grad, cudaStream_t s) {
    if (nprimary == 0) return;
    const int grid = grid_of(nprimary * 32, kT, 152 * 16);
    if (f64)
        sddmm_kernel<double><<<grid, kT, 0, s>>>(nprimary, ptr, idx, static_cast<const double*>(vals), column_major,
                                                 Z1, Z2, kk, f, cmean, c, qf, static_cast<double*>(grad));
    else
        sddmm_kernel<float><<<grid, kT, 0, s>>>(nprimary, ptr, idx, static_cast<const float*>(vals), column_major, Z1,
                                                Z2, kk, f, cmean, c, qf, static_cast<float*>(grad));
    count_launch();
}

}  // namespace irlba_gb300
