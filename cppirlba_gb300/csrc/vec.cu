// Tall-skinny kernels of the IRLBA loop:
//  * classical Gram-Schmidt reorthogonalization, orthogonalize_vector in
//    CppIrlba's lanczos.hpp:17-21 (t = Q^T v; v -= Q t), as two passes over Q:
//    a GEMV-transpose with per-CTA partials reduced by the last CTA in a fixed
//    order, then the GEMV update fused with the norm of the result;
//  * normalization of a Lanczos vector fused with the centring scalar of the
//    next matvec and the bidiagonal entries (lanczos.hpp:85-86,108-113,131-134);
//  * the restart rotations V <- V BV, W <- W BU (compute.hpp:268-280) and the
//    output assembly (compute.hpp:298-305);
//  * realization and PCA column statistics (pca.hpp:85-109).
// Coefficients and norms accumulate in FP64 in both precision forms: in the FP32
// form each lane sums 16 FP32 products (the dot pass) or one row's products (the
// update pass) before adding them to an FP64 total.

#include <type_traits>

#include "kernels.cuh"

namespace irlba_gb300 {

namespace {

constexpr int kThreads = 256;
constexpr int kDotRows = 1024;     // rows of v staged per sub-chunk of the GEMV-transpose pass
constexpr int kDotUnit = 256;      // granularity of its row ranges
constexpr int kDotMaxRanges = 1216;  // upper bound of its row ranges (gridDim.x)
constexpr int kMaxCols = 1024;     // basis columns held in shared memory

int grid_for(int64_t n, int threads, int cap) {
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return static_cast<int>(g);
}

// ---------------------------------------------------------------------------
// t = Q[:, :c]^T v
// ---------------------------------------------------------------------------
// Grid: x = row ranges, y = groups of (threads / 32) columns; one warp per
// (range, column). gridDim.x is sized so the whole grid is one wave of resident
// CTAs, and each range is a balanced run of 256-row units processed in
// sub-chunks of kDotRows rows (v staged in shared memory per sub-chunk). Lanes
// keep their FP64 accumulators across the whole range, so the FP64 shuffle
// reduction runs once per (range, column): on GB300, whose FP64 rate is about
// 1/60 of its FP32 rate, per-sub-chunk reductions made the FP64 pipe a
// co-bottleneck of this memory-bound pass. The last CTA reduces the per-range
// partials with one warp per column (lane-strided, then a shuffle tree): the
// summation order is fixed, so results are bit-reproducible.
template <typename T>
__global__ void __launch_bounds__(kThreads) cgs_dot_kernel(const T* __restrict__ Q, int64_t L, int64_t ldq, int32_t c,
                                                           const T* __restrict__ v, double* __restrict__ part,
                                                           double* __restrict__ t, Ctrl* ctrl) {
    __shared__ T vs[kDotRows];
    __shared__ bool is_last;
    if (ctrl->abort) return;
    const int64_t units = (L + kDotUnit - 1) / kDotUnit;
    const int64_t u0 = units * blockIdx.x / gridDim.x, u1 = units * (blockIdx.x + 1) / gridDim.x;
    const int64_t rbeg = u0 * kDotUnit, rend = (u1 * kDotUnit < L) ? u1 * kDotUnit : L;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int j = static_cast<int>(blockIdx.y) * nw + warp;
    double acc = 0;
    for (int64_t r0 = rbeg; r0 < rend; r0 += kDotRows) {
        const int rows = static_cast<int>((rend - r0 < kDotRows ? rend - r0 : static_cast<int64_t>(kDotRows)));
        __syncthreads();  // the previous sub-chunk's readers are done with vs
        for (int i = threadIdx.x; i < rows; i += blockDim.x) vs[i] = v[r0 + i];
        __syncthreads();
        if (j < c) {
            const T* __restrict__ q = Q + j * ldq + r0;
            int i = lane;
            // 16-product partials: 16 loads in flight per lane and one
            // conversion and FP64 add per 16 products (the FP64 pipe, at about
            // 1/60 of the FP32 rate on GB300, otherwise co-limits this pass).
            for (; i + 15 * 32 < rows; i += 16 * 32) {
                T s = 0;
#pragma unroll
                for (int u = 0; u < 16; ++u) s += q[i + u * 32] * vs[i + u * 32];
                acc += static_cast<double>(s);
            }
            {
                T s = 0;
                for (; i < rows; i += 32) s += q[i] * vs[i];
                acc += static_cast<double>(s);
            }
        }
    }
    acc = warp_sum(acc);
    if (j < c && lane == 0) part[static_cast<int64_t>(blockIdx.x) * c + j] = acc;

    if (last_block(&ctrl->ticket[kTicketDot], &is_last)) {
        const int chunks = static_cast<int>(gridDim.x);
        for (int jj = warp; jj < c; jj += nw) {
            double s = 0;
            for (int b = lane; b < chunks; b += 32) s += __ldcg(part + static_cast<int64_t>(b) * c + jj);
            s = warp_sum(s);
            if (lane == 0) t[jj] = s;
        }
        if (threadIdx.x == 0) ctrl->ticket[kTicketDot] = 0;
    }
}

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    typedef float4 V;
    static constexpr int N = 4;
};
template <>
struct Vec16<double> {
    typedef double2 V;
    static constexpr int N = 2;
};

template <typename T>
__device__ __forceinline__ void vec16_fma(T* s, const float4& x, T tj) {
    s[0] += x.x * tj;
    s[1] += x.y * tj;
    s[2] += x.z * tj;
    s[3] += x.w * tj;
}
template <typename T>
__device__ __forceinline__ void vec16_fma(T* s, const double2& x, T tj) {
    s[0] += x.x * tj;
    s[1] += x.y * tj;
}
__device__ __forceinline__ double vec16_update(float4& x, const float* s) {
    x.x -= s[0];
    x.y -= s[1];
    x.z -= s[2];
    x.w -= s[3];
    double q = static_cast<double>(x.x) * static_cast<double>(x.x);
    q += static_cast<double>(x.y) * static_cast<double>(x.y);
    q += static_cast<double>(x.z) * static_cast<double>(x.z);
    q += static_cast<double>(x.w) * static_cast<double>(x.w);
    return q;
}
__device__ __forceinline__ double vec16_update(double2& x, const double* s) {
    x.x -= s[0];
    x.y -= s[1];
    return x.x * x.x + x.y * x.y;
}
template <typename T>
__device__ __forceinline__ void vec16_dot(T& s, const float4& a, const float4& b) {
    s += a.x * b.x;
    s += a.y * b.y;
    s += a.z * b.z;
    s += a.w * b.w;
}
template <typename T>
__device__ __forceinline__ void vec16_dot(T& s, const double2& a, const double2& b) {
    s += a.x * b.x;
    s += a.y * b.y;
}

// The dot pass with 16-byte loads (four FP32 or two FP64 rows per lane and
// load, eight loads in flight per lane: 4 KB per warp), for a 16-byte aligned Q
// and v with ldq a multiple of the vector width. Same ranges, accumulation
// structure and final reduction as cgs_dot_kernel; each FP64 add takes a
// partial sum of 32 FP32 products or 16 FP64 products. Used for the FP64 form.
template <typename T>
__global__ void __launch_bounds__(kThreads) cgs_dot_vec_kernel(const T* __restrict__ Q, int64_t L, int64_t ldq,
                                                               int32_t c, const T* __restrict__ v,
                                                               double* __restrict__ part, double* __restrict__ t,
                                                               Ctrl* ctrl) {
    typedef typename Vec16<T>::V V;
    constexpr int N = Vec16<T>::N;
    constexpr int kU = 8;                       // vectors in flight per lane
    constexpr int kRows = 32 * kU * N * 2;      // rows of v staged per sub-chunk
    __shared__ __align__(16) T vs[kRows];
    __shared__ bool is_last;
    if (ctrl->abort) return;
    const int64_t units = (L + kDotUnit - 1) / kDotUnit;
    const int64_t u0 = units * blockIdx.x / gridDim.x, u1 = units * (blockIdx.x + 1) / gridDim.x;
    const int64_t rbeg = u0 * kDotUnit, rend = (u1 * kDotUnit < L) ? u1 * kDotUnit : L;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int j = static_cast<int>(blockIdx.y) * nw + warp;
    double acc = 0;
    for (int64_t r0 = rbeg; r0 < rend; r0 += kRows) {
        const int rows = static_cast<int>((rend - r0 < kRows ? rend - r0 : static_cast<int64_t>(kRows)));
        __syncthreads();  // the previous sub-chunk's readers are done with vs
        for (int i = threadIdx.x; i < rows; i += blockDim.x) vs[i] = v[r0 + i];
        __syncthreads();
        if (j < c) {
            const V* __restrict__ q4 = reinterpret_cast<const V*>(Q + j * ldq + r0);
            const V* v4 = reinterpret_cast<const V*>(vs);
            const int nvec = rows / N;
            int i = lane;
            for (; i + (kU - 1) * 32 < nvec; i += kU * 32) {
                V a[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) a[u] = q4[i + u * 32];
                T sum = 0;
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const V b = v4[i + u * 32];
                    vec16_dot<T>(sum, a[u], b);
                }
                acc += static_cast<double>(sum);
            }
            T sum = 0;
            for (; i < nvec; i += 32) vec16_dot<T>(sum, q4[i], v4[i]);
            for (int rr = nvec * N + lane; rr < rows; rr += 32) sum += Q[j * ldq + r0 + rr] * vs[rr];
            acc += static_cast<double>(sum);
        }
    }
    acc = warp_sum(acc);
    if (j < c && lane == 0) part[static_cast<int64_t>(blockIdx.x) * c + j] = acc;

    if (last_block(&ctrl->ticket[kTicketDot], &is_last)) {
        const int chunks = static_cast<int>(gridDim.x);
        for (int jj = warp; jj < c; jj += nw) {
            double s = 0;
            for (int b = lane; b < chunks; b += 32) s += __ldcg(part + static_cast<int64_t>(b) * c + jj);
            s = warp_sum(s);
            if (lane == 0) t[jj] = s;
        }
        if (threadIdx.x == 0) ctrl->ticket[kTicketDot] = 0;
    }
}

// Sum of count partials by the whole CTA in a fixed order (thread-strided, then
// the block tree); the result is valid in thread 0.
__device__ __forceinline__ double reduce_partials(const double* part, int count, double* red) {
    double s = 0;
    for (int b = threadIdx.x; b < count; b += blockDim.x) s += __ldcg(part + b);
    return block_sum(s, red);
}

// ---------------------------------------------------------------------------
// v -= Q[:, :c] t ; norm = ||v||
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads) cgs_update_kernel(const T* __restrict__ Q, int64_t L, int64_t ldq,
                                                              int32_t c, const double* __restrict__ t,
                                                              T* __restrict__ v, double* __restrict__ part,
                                                              double* norm_out, int32_t check_eps, int32_t check_null,
                                                              Ctrl* ctrl) {
    __shared__ T ts[kMaxCols];
    __shared__ double red[32];
    __shared__ bool is_last;
    if (ctrl->abort) return;
    // The first kMaxCols coefficients are staged; any beyond are read from t.
    const int cs = c < kMaxCols ? c : kMaxCols;
    for (int j = threadIdx.x; j < cs; j += blockDim.x) ts[j] = static_cast<T>(t[j]);
    __syncthreads();

    double sq = 0;
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < L;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        T s = 0;
        const T* __restrict__ q = Q + r;
        int j = 0;
        for (; j + 3 < cs; j += 4) {
            const T q0 = q[j * ldq], q1 = q[(j + 1) * ldq], q2 = q[(j + 2) * ldq], q3 = q[(j + 3) * ldq];
            s += q0 * ts[j];
            s += q1 * ts[j + 1];
            s += q2 * ts[j + 2];
            s += q3 * ts[j + 3];
        }
        for (; j < cs; ++j) s += q[j * ldq] * ts[j];
        for (; j < c; ++j) s += q[j * ldq] * static_cast<T>(__ldg(t + j));
        const T nv = v[r] - s;
        v[r] = nv;
        sq += static_cast<double>(nv) * static_cast<double>(nv);
    }
    const double bs = block_sum(sq, red);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;

    if (last_block(&ctrl->ticket[kTicketUpdate], &is_last)) {
        const double s = reduce_partials(part, static_cast<int>(gridDim.x), red);
        if (threadIdx.x == 0) {
            const double nrm = sqrt(s);
            *norm_out = nrm;
            if (check_null && nrm < ctrl->eps) {
                ctrl->null_start = 1;
                ctrl->abort = 1;
            } else if (check_eps && nrm < ctrl->eps) {
                ctrl->invariant = 1;
                ctrl->abort = 1;
            }
            ctrl->ticket[kTicketUpdate] = 0;
        }
    }
}

// The update pass with four FP32 or two FP64 consecutive rows per thread: one
// 16-byte load per basis column and eight columns in flight, so a warp keeps
// 4 KB of loads outstanding (the form above keeps 512 B, too few to cover
// HBM latency at full bandwidth). Columns run from the last to the first: the
// dot pass just before read the basis column group by column group, so its
// last columns are the ones still in L2 when this pass starts. Each row's
// products are therefore summed in descending column order (the form above
// sums ascending; v differs by rounding only). Needs ldq a multiple of the row
// count and 16-byte aligned Q and v; rows past the last full group are done by
// the first CTA.
template <typename T>
__global__ void __launch_bounds__(kThreads) cgs_update_vec_kernel(const T* __restrict__ Q, int64_t L, int64_t ldq,
                                                                  int32_t c, const double* __restrict__ t,
                                                                  T* __restrict__ v, double* __restrict__ part,
                                                                  double* norm_out, int32_t check_eps,
                                                                  int32_t check_null, Ctrl* ctrl) {
    typedef typename Vec16<T>::V V;
    constexpr int N = Vec16<T>::N;
    __shared__ T ts[kMaxCols];
    __shared__ double red[32];
    __shared__ bool is_last;
    if (ctrl->abort) return;
    const int cs = c < kMaxCols ? c : kMaxCols;
    for (int j = threadIdx.x; j < cs; j += blockDim.x) ts[j] = static_cast<T>(t[j]);
    __syncthreads();

    double sq = 0;
    const int64_t nv = L / N;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < nv;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = g * N;
        T s[N];
#pragma unroll
        for (int u = 0; u < N; ++u) s[u] = 0;
        const T* __restrict__ q = Q + r;
        int j = c - 1;
        for (; j >= cs; --j) vec16_fma<T>(s, *reinterpret_cast<const V*>(q + j * ldq), static_cast<T>(__ldg(t + j)));
        for (; j >= 7; j -= 8) {
            V x[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) x[u] = *reinterpret_cast<const V*>(q + (j - u) * ldq);
#pragma unroll
            for (int u = 0; u < 8; ++u) vec16_fma<T>(s, x[u], ts[j - u]);
        }
        for (; j >= 0; --j) vec16_fma<T>(s, *reinterpret_cast<const V*>(q + j * ldq), ts[j]);
        V x = *reinterpret_cast<V*>(v + r);
        sq += vec16_update(x, s);
        *reinterpret_cast<V*>(v + r) = x;
    }
    if (blockIdx.x == 0)
        for (int64_t r = nv * N + threadIdx.x; r < L; r += blockDim.x) {
            T s = 0;
            for (int j = 0; j < c; ++j) s += Q[r + j * ldq] * (j < cs ? ts[j] : static_cast<T>(__ldg(t + j)));
            const T nvv = v[r] - s;
            v[r] = nvv;
            sq += static_cast<double>(nvv) * static_cast<double>(nvv);
        }
    const double bs = block_sum(sq, red);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;

    if (last_block(&ctrl->ticket[kTicketUpdate], &is_last)) {
        const double tot = reduce_partials(part, static_cast<int>(gridDim.x), red);
        if (threadIdx.x == 0) {
            const double nrm = sqrt(tot);
            *norm_out = nrm;
            if (check_null && nrm < ctrl->eps) {
                ctrl->null_start = 1;
                ctrl->abort = 1;
            } else if (check_eps && nrm < ctrl->eps) {
                ctrl->invariant = 1;
                ctrl->abort = 1;
            }
            ctrl->ticket[kTicketUpdate] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// v /= norm; qcol = v; beta = sum f(v) g; B entries.
// ---------------------------------------------------------------------------
template <typename T, bool NORMALIZE>
__global__ void __launch_bounds__(kThreads) normalize_kernel(T* __restrict__ v, int64_t L, const double* norm,
                                                             T* __restrict__ qcol, const T* __restrict__ fscale,
                                                             int32_t fdivide, const T* __restrict__ gvec,
                                                             double* beta_out, double* __restrict__ part, double* B,
                                                             int64_t bpos, int64_t ldb, Ctrl* ctrl) {
    __shared__ double red[32];
    __shared__ bool is_last;
    if (ctrl->abort) return;
    T inv = 1;
    if (NORMALIZE) inv = static_cast<T>(1.0 / *norm);
    double acc = 0;
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < L;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        T x = v[r];
        if (NORMALIZE) {
            x = x * inv;
            v[r] = x;
            if (qcol) qcol[r] = x;
        }
        if (beta_out) {
            T f = x;
            if (fscale) f = fdivide ? f / fscale[r] : f * fscale[r];
            if (gvec) acc += static_cast<double>(f * gvec[r]);
            else acc += static_cast<double>(f);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && B && bpos >= 0) {
        B[bpos] = ctrl->S;
        B[bpos + ldb] = ctrl->R_F;
    }
    if (!beta_out) return;
    const double bs = block_sum(acc, red);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (last_block(&ctrl->ticket[kTicketNormalize], &is_last)) {
        const double s = reduce_partials(part, static_cast<int>(gridDim.x), red);
        if (threadIdx.x == 0) {
            *beta_out = s;
            ctrl->ticket[kTicketNormalize] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// out[:, :k] = Q[:, :w] R[:, :k] (+ out[:, k] = fcol / fnorm)
// ---------------------------------------------------------------------------
template <typename T, typename O, int WMAX>
__global__ void __launch_bounds__(128) rotate_kernel(const T* Q, int64_t L, int64_t ldq, int32_t w,
                                                     const double* __restrict__ R, int32_t ldr, int32_t k, O* out,
                                                     int64_t ldo, const T* __restrict__ fcol,
                                                     const double* fnorm, const int32_t* abort) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // Rs[j * k + i] = R[j, i] for j < w, zero for w <= j < WMAX.
    T* Rs = reinterpret_cast<T*>(smem_raw);
    if (abort && *abort) return;
    for (int idx = threadIdx.x; idx < WMAX * k; idx += blockDim.x) {
        const int j = idx / k, i = idx % k;
        Rs[idx] = j < w ? static_cast<T>(R[j + static_cast<int64_t>(i) * ldr]) : T(0);
    }
    __syncthreads();
    T finv = 0;
    if (fcol) finv = static_cast<T>(1.0 / *fnorm);
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < L;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        T row[WMAX];
#pragma unroll
        for (int j = 0; j < WMAX; ++j) row[j] = (j < w) ? Q[r + j * ldq] : T(0);
        for (int i = 0; i < k; ++i) {
            T s = 0;
#pragma unroll
            for (int j = 0; j < WMAX; ++j) s += row[j] * Rs[j * k + i];
            out[r + i * ldo] = static_cast<O>(s);
        }
        if (fcol) out[r + static_cast<int64_t>(k) * ldo] = static_cast<O>(fcol[r] * finv);
    }
}

// FP32 rotation with the whole output row in registers: for each input column
// j, one float4 shared-memory broadcast feeds four FMAs (the scalar form above
// spends one shared load per FMA). R is zero-padded to WMAX x WMAX.
template <int WMAX>
__global__ void __launch_bounds__(128) rotate_f32_tiled_kernel(const float* Q, int64_t L, int64_t ldq, int32_t w,
                                                               const double* __restrict__ R, int32_t ldr, int32_t k,
                                                               float* out, int64_t ldo, const float* __restrict__ fcol,
                                                               const double* fnorm, const int32_t* abort) {
    __shared__ __align__(16) float4 Rs4[WMAX * (WMAX / 4)];
    if (abort && *abort) return;
    float* Rs = reinterpret_cast<float*>(Rs4);
    for (int idx = threadIdx.x; idx < WMAX * WMAX; idx += blockDim.x) {
        const int j = idx / WMAX, i = idx % WMAX;
        Rs[idx] = (j < w && i < k) ? static_cast<float>(R[j + static_cast<int64_t>(i) * ldr]) : 0.0f;
    }
    __syncthreads();
    float finv = 0;
    if (fcol) finv = static_cast<float>(1.0 / *fnorm);
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < L;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float row[WMAX];
#pragma unroll
        for (int j = 0; j < WMAX; ++j) row[j] = (j < w) ? Q[r + j * ldq] : 0.0f;
        float acc[WMAX];
#pragma unroll
        for (int i = 0; i < WMAX; ++i) acc[i] = 0.0f;
#pragma unroll
        for (int j = 0; j < WMAX; ++j) {
            const float rj = row[j];
#pragma unroll
            for (int i4 = 0; i4 < WMAX / 4; ++i4) {
                const float4 c = Rs4[j * (WMAX / 4) + i4];
                acc[4 * i4 + 0] += rj * c.x;
                acc[4 * i4 + 1] += rj * c.y;
                acc[4 * i4 + 2] += rj * c.z;
                acc[4 * i4 + 3] += rj * c.w;
            }
        }
#pragma unroll
        for (int i = 0; i < WMAX; ++i)
            if (i < k) out[r + i * ldo] = acc[i];
        if (fcol) out[r + static_cast<int64_t>(k) * ldo] = fcol[r] * finv;
    }
}

// FP32 rotation as a tiled GEMM for w, k <= 64. A CTA takes 128 rows at a
// time and stages Q[rows, :w] in shared memory first, so the outputs may
// overwrite Q (in place) and the fcol column may be one of the inputs. Each
// of the 256 threads forms rows {4 tx .. 4 tx + 3, 64 + 4 tx .. 64 + 4 tx + 3}
// x columns {4 ty .. 4 ty + 3}: per input column, three 16-byte shared loads
// (conflict-free for the rows, broadcast for R) feed 32 FMAs.
constexpr int kRotTileRows = 128;
constexpr size_t kRotGemmSmem = sizeof(float) * (64 * 64 + 64 * kRotTileRows);

__device__ __forceinline__ float4 load4_guarded(const float* src, int64_t r, int64_t L) {
    if (r + 3 < L) return *reinterpret_cast<const float4*>(src);
    float4 v;
    v.x = r < L ? src[0] : 0.0f;
    v.y = r + 1 < L ? src[1] : 0.0f;
    v.z = r + 2 < L ? src[2] : 0.0f;
    v.w = r + 3 < L ? src[3] : 0.0f;
    return v;
}

__device__ __forceinline__ void store4_guarded(float* dst, int64_t r, int64_t L, float a, float b, float c, float d) {
    if (r + 3 < L) {
        *reinterpret_cast<float4*>(dst) = make_float4(a, b, c, d);
        return;
    }
    if (r < L) dst[0] = a;
    if (r + 1 < L) dst[1] = b;
    if (r + 2 < L) dst[2] = c;
}

__global__ void __launch_bounds__(256) rotate_f32_gemm_kernel(const float* Q, int64_t L, int64_t ldq, int32_t w,
                                                             const double* __restrict__ R, int32_t ldr, int32_t k,
                                                             float* out, int64_t ldo, const float* __restrict__ fcol,
                                                             const double* fnorm, const int32_t* abort) {
    extern __shared__ __align__(16) float rsm[];
    float* Rs = rsm;                // Rs[j * 64 + i]
    float* Qs = rsm + 64 * 64;      // Qs[j * kRotTileRows + row]
    if (abort && *abort) return;
    for (int idx = threadIdx.x; idx < 64 * 64; idx += blockDim.x) {
        const int j = idx / 64, i = idx % 64;
        Rs[idx] = (j < w && i < k) ? static_cast<float>(R[j + static_cast<int64_t>(i) * ldr]) : 0.0f;
    }
    const float finv = fcol ? static_cast<float>(1.0 / *fnorm) : 0.0f;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    for (int64_t r0 = blockIdx.x * static_cast<int64_t>(kRotTileRows); r0 < L;
         r0 += static_cast<int64_t>(gridDim.x) * kRotTileRows) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < w * (kRotTileRows / 4); idx += blockDim.x) {
            const int j = idx / (kRotTileRows / 4), q = idx % (kRotTileRows / 4);
            const int64_t r = r0 + 4 * q;
            *reinterpret_cast<float4*>(Qs + j * kRotTileRows + 4 * q) = load4_guarded(Q + r + j * ldq, r, L);
        }
        __syncthreads();
        float acc[8][4];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
        for (int j = 0; j < w; ++j) {
            const float4 q0 = *reinterpret_cast<const float4*>(Qs + j * kRotTileRows + 4 * tx);
            const float4 q1 = *reinterpret_cast<const float4*>(Qs + j * kRotTileRows + 64 + 4 * tx);
            const float4 rr = *reinterpret_cast<const float4*>(Rs + j * 64 + 4 * ty);
            const float qa[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
            const float rb[4] = {rr.x, rr.y, rr.z, rr.w};
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(qa[a], rb[b], acc[a][b]);
        }
        if (fcol)
            for (int idx = threadIdx.x; idx < kRotTileRows; idx += blockDim.x) {
                const int64_t r = r0 + idx;
                if (r < L) out[r + static_cast<int64_t>(k) * ldo] = fcol[r] * finv;
            }
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int col = 4 * ty + b;
            if (col < k) {
                const int64_t ra = r0 + 4 * tx, rb2 = r0 + 64 + 4 * tx;
                store4_guarded(out + ra + col * ldo, ra, L, acc[0][b], acc[1][b], acc[2][b], acc[3][b]);
                store4_guarded(out + rb2 + col * ldo, rb2, L, acc[4][b], acc[5][b], acc[6][b], acc[7][b]);
            }
        }
    }
}

// The same FP32 rotation with the Q tiles streamed through two shared-memory
// buffers by cp.async (16-byte copies completing in the background), so the
// next tile's loads overlap this tile's products, and with the column groups
// at or past k idle (k = 50 of 64 leaves three of sixteen groups without
// products). Needs ldq % 4 == 0 and a 16-byte aligned Q; the last, partial
// tile is loaded with guarded plain loads. Every CTA reads all rows of a tile
// into shared memory before it writes any output row of that tile, so out
// may be Q itself.
constexpr size_t kRotPipeSmem = sizeof(float) * (64 * 64 + 2 * 64 * kRotTileRows);

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__global__ void __launch_bounds__(256) rotate_f32_pipe_kernel(const float* Q, int64_t L, int64_t ldq, int32_t w,
                                                             const double* __restrict__ R, int32_t ldr, int32_t k,
                                                             float* out, int64_t ldo, const float* __restrict__ fcol,
                                                             const double* fnorm, const int32_t* abort) {
    extern __shared__ __align__(16) float rsm[];
    float* Rs = rsm;                // Rs[j * 64 + i]
    float* Qb = rsm + 64 * 64;      // two tiles, Qb[buf][j * kRotTileRows + row]
    if (abort && *abort) return;
    const int64_t ntiles = (L + kRotTileRows - 1) / kRotTileRows;
    auto issue = [&](int64_t tile, int buf) {
        const int64_t r0 = tile * kRotTileRows;
        float* dst = Qb + buf * (64 * kRotTileRows);
        if (r0 + kRotTileRows <= L) {
            for (int idx = threadIdx.x; idx < w * (kRotTileRows / 4); idx += blockDim.x) {
                const int j = idx / (kRotTileRows / 4), q = idx % (kRotTileRows / 4);
                cp_async16(dst + j * kRotTileRows + 4 * q, Q + r0 + 4 * q + j * ldq);
            }
        } else {
            for (int idx = threadIdx.x; idx < w * (kRotTileRows / 4); idx += blockDim.x) {
                const int j = idx / (kRotTileRows / 4), q = idx % (kRotTileRows / 4);
                const int64_t r = r0 + 4 * q;
                *reinterpret_cast<float4*>(dst + j * kRotTileRows + 4 * q) = load4_guarded(Q + r + j * ldq, r, L);
            }
        }
        cp_async_commit();
    };
    int64_t tile = blockIdx.x;
    if (tile < ntiles) issue(tile, 0);
    for (int idx = threadIdx.x; idx < 64 * 64; idx += blockDim.x) {
        const int j = idx / 64, i = idx % 64;
        Rs[idx] = (j < w && i < k) ? static_cast<float>(R[j + static_cast<int64_t>(i) * ldr]) : 0.0f;
    }
    const float finv = fcol ? static_cast<float>(1.0 / *fnorm) : 0.0f;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const bool cols = 4 * ty < k;
    int buf = 0;
    for (; tile < ntiles; tile += gridDim.x) {
        const int64_t next = tile + gridDim.x;
        if (next < ntiles) issue(next, buf ^ 1);
        else cp_async_commit();
        cp_async_wait_prev();
        __syncthreads();
        const float* Qs = Qb + buf * (64 * kRotTileRows);
        const int64_t r0 = tile * kRotTileRows;
        float acc[8][4];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
        if (cols) {
            for (int j = 0; j < w; ++j) {
                const float4 q0 = *reinterpret_cast<const float4*>(Qs + j * kRotTileRows + 4 * tx);
                const float4 q1 = *reinterpret_cast<const float4*>(Qs + j * kRotTileRows + 64 + 4 * tx);
                const float4 rr = *reinterpret_cast<const float4*>(Rs + j * 64 + 4 * ty);
                const float qa[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
                const float rb[4] = {rr.x, rr.y, rr.z, rr.w};
#pragma unroll
                for (int a = 0; a < 8; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(qa[a], rb[b], acc[a][b]);
            }
        }
        if (fcol)
            for (int idx = threadIdx.x; idx < kRotTileRows; idx += blockDim.x) {
                const int64_t r = r0 + idx;
                if (r < L) out[r + static_cast<int64_t>(k) * ldo] = fcol[r] * finv;
            }
        if (cols) {
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int col = 4 * ty + b;
                if (col < k) {
                    const int64_t ra = r0 + 4 * tx, rb2 = r0 + 64 + 4 * tx;
                    store4_guarded(out + ra + col * ldo, ra, L, acc[0][b], acc[1][b], acc[2][b], acc[3][b]);
                    store4_guarded(out + rb2 + col * ldo, rb2, L, acc[4][b], acc[5][b], acc[6][b], acc[7][b]);
                }
            }
        }
        // Every thread is done with this buffer before the next issue refills it.
        __syncthreads();
        buf ^= 1;
    }
    cp_async_wait_all();
}

// Rotations with more than 128 basis columns: tmp (rows x k, ld rows) =
// Q[r0 : r0 + rows, :w] R[:w, :k] with 32 x 32 output tiles and 32-column
// steps through w in shared memory; then tmp is copied over out (in place is
// safe: every read of the chunk's rows happens in the product kernel).
template <typename T>
__global__ void __launch_bounds__(256) rotate_chunk_kernel(const T* __restrict__ Q, int64_t r0, int64_t rows,
                                                           int64_t ldq, int32_t w, const double* __restrict__ R,
                                                           int32_t ldr, int32_t k, T* __restrict__ tmp) {
    __shared__ T Qs[32][33];
    __shared__ T Rs[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;      // 32 x 8 threads, 4 outputs each
    const int64_t rb = static_cast<int64_t>(blockIdx.x) * 32;
    const int cb = blockIdx.y * 32;
    T acc[4] = {0, 0, 0, 0};
    for (int j0 = 0; j0 < w; j0 += 32) {
        for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
            const int a = t % 32, b = t / 32;                          // a: row / j, b: j / column
            const int64_t r = rb + a;
            Qs[b][a] = (r < rows && j0 + b < w) ? Q[r0 + r + static_cast<int64_t>(j0 + b) * ldq] : T(0);
            Rs[b][a] = (j0 + a < w && cb + b < k) ? static_cast<T>(R[(j0 + a) + static_cast<int64_t>(cb + b) * ldr])
                                                  : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
            const T q = Qs[j][tx];
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] += q * Rs[ty + 8 * u][j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t r = rb + tx;
        const int c = cb + ty + 8 * u;
        if (r < rows && c < k) tmp[r + static_cast<int64_t>(c) * rows] = acc[u];
    }
}

template <typename T, typename O>
__global__ void rotate_chunk_store_kernel(const T* __restrict__ tmp, int64_t r0, int64_t rows, int32_t k, O* out,
                                          int64_t ldo, const T* __restrict__ fcol, const double* fnorm) {
    const T finv = fcol ? static_cast<T>(1.0 / *fnorm) : T(0);
    const int64_t total = rows * (k + (fcol ? 1 : 0));
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = e % rows, c = e / rows;
        if (c < k) out[r0 + r + c * ldo] = static_cast<O>(tmp[r + c * rows]);
        else out[r0 + r + static_cast<int64_t>(k) * ldo] = static_cast<O>(fcol[r0 + r] * finv);
    }
}

template <typename T, typename O>
static void rotate_wide(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                        O* out, int64_t ldo, const T* fcol, const double* fnorm, cudaStream_t stream) {
    if (L == 0 || (k == 0 && !fcol)) return;
    // Chunks of rows whose product fits a 256 MB stream-ordered temporary.
    const int64_t kk = k > 0 ? k : 1;
    const int64_t chunk = std::max<int64_t>(32, std::min<int64_t>(L, (int64_t(256) << 20) / (sizeof(T) * kk)));
    void* tmp = nullptr;
    if (cudaMallocAsync(&tmp, sizeof(T) * kk * chunk, stream) != cudaSuccess) return;
    for (int64_t r0 = 0; r0 < L; r0 += chunk) {
        const int64_t rows = std::min(chunk, L - r0);
        if (k > 0) {
            dim3 grid(static_cast<unsigned>((rows + 31) / 32), static_cast<unsigned>((k + 31) / 32));
            rotate_chunk_kernel<T><<<grid, 256, 0, stream>>>(Q, r0, rows, ldq, w, R, ldr, k, static_cast<T*>(tmp));
            count_launch();
        }
        rotate_chunk_store_kernel<T, O><<<grid_for(rows * (k + 1), 256, 152 * 16), 256, 0, stream>>>(
            static_cast<const T*>(tmp), r0, rows, k, out, ldo, fcol, fnorm);
        count_launch();
    }
    cudaFreeAsync(tmp, stream);
}

static bool g_rotate_pipe_ok = false;

template <typename T, typename O>
void rotate_dispatch(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k, O* out,
                     int64_t ldo, const T* fcol, const double* fnorm, const int32_t* abort, cudaStream_t stream,
                     bool allow_tc = true) {
    if (w > 128) {
        // Wide bases skip the abort check: the engine only rotates after a
        // restart whose control block it has read (abort clear).
        rotate_wide<T, O>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, stream);
        return;
    }
    // Tensor cores (BF16 slice products, FP32 or FP64 accuracy) for the
    // restart rotations; the CUDA-core kernels below otherwise.
    if constexpr (std::is_same<T, O>::value) {
        if (allow_tc && w >= 1 && w <= 64 && k <= 64 && rotate_engine() == 1) {
            if constexpr (std::is_same<T, float>::value) {
                if (rotate_tc32_available()) {
                    launch_rotate_tc32(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort, nullptr, 0, stream);
                    return;
                }
            } else {
                if (rotate_tc64_available()) {
                    launch_rotate_tc64(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort, nullptr, 0, stream);
                    return;
                }
            }
        }
    }
    if constexpr (std::is_same<T, float>::value && std::is_same<O, float>::value) {
        const bool aligned = ldq % 4 == 0 && ldo % 4 == 0 && reinterpret_cast<uintptr_t>(Q) % 16 == 0 &&
                             reinterpret_cast<uintptr_t>(out) % 16 == 0;
        if (w <= 64 && k <= 64 && aligned) {
            const int64_t tiles = (L + kRotTileRows - 1) / kRotTileRows;
            if (g_rotate_pipe_ok) {
                const int grid = static_cast<int>(tiles < 152 * 2 ? (tiles < 1 ? 1 : tiles) : 152 * 2);
                rotate_f32_pipe_kernel<<<grid, 256, kRotPipeSmem, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol,
                                                                            fnorm, abort);
            } else {
                const int grid = static_cast<int>(tiles < 152 * 4 ? (tiles < 1 ? 1 : tiles) : 152 * 4);
                rotate_f32_gemm_kernel<<<grid, 256, kRotGemmSmem, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol,
                                                                            fnorm, abort);
            }
            count_launch();
            return;
        }
        if (w <= 64) {
            const int grid = grid_for(L, 128, 152 * 16);
            if (w <= 16) {
                rotate_f32_tiled_kernel<16><<<grid, 128, 0, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort);
            } else if (w <= 32) {
                rotate_f32_tiled_kernel<32><<<grid, 128, 0, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort);
            } else {
                rotate_f32_tiled_kernel<64><<<grid, 128, 0, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort);
            }
            count_launch();
            return;
        }
    }
    const int grid = grid_for(L, 128, 152 * 8);
    const int kk = k > 0 ? k : 1;
    if (w <= 16) {
        rotate_kernel<T, O, 16><<<grid, 128, sizeof(T) * 16 * kk, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort); count_launch();
    } else if (w <= 32) {
        rotate_kernel<T, O, 32><<<grid, 128, sizeof(T) * 32 * kk, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort); count_launch();
    } else if (w <= 64) {
        rotate_kernel<T, O, 64><<<grid, 128, sizeof(T) * 64 * kk, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort); count_launch();
    } else {
        rotate_kernel<T, O, 128><<<grid, 128, sizeof(T) * 128 * kk, stream>>>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort); count_launch();
    }
}

template <typename A, typename B>
__global__ void convert_kernel(const A* __restrict__ in, B* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<B>(in[i]);
}

// Scatter of a direction plan into a dense column-major matrix. The plan's rows
// are matrix rows (transpose = 0) or matrix columns (transpose = 1).
template <typename VT>
__global__ void realize_kernel(const DirPlanDev p, double* out, int64_t ld, int32_t transpose) {
    const VT* val = static_cast<const VT*>(p.val);
    for (int64_t seg = blockIdx.x; seg < p.nseg; seg += gridDim.x) {
        const int64_t panel = seg / p.nrows, row = seg % p.nrows;
        for (int64_t s = p.segptr[seg] + threadIdx.x; s < p.segptr[seg + 1]; s += blockDim.x) {
            const int64_t col = p.staged ? panel * p.panel_width + p.idx16[s] : p.idx32[s];
            const double v = static_cast<double>(val[s]);
            if (transpose) out[row * ld + col] = v;
            else out[col * ld + row] = v;
        }
    }
}

__global__ void realize_ops_kernel(double* A, int64_t m, int64_t n, const double* center, const double* scale,
                                   int32_t scale_column, int32_t scale_divide, int32_t center_outer) {
    const int64_t total = m * n;
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = e % m, c = e / m;
        double v = A[e];
        if (center && !center_outer) v -= center[c];
        if (scale) {
            const double s = scale_column ? scale[c] : scale[r];
            v = scale_divide ? v / s : v * s;
        }
        if (center && center_outer) v -= center[c];
        A[e] = v;
    }
}

// Per-feature sums over segments of a plan whose rows are features.
template <typename VT>
__global__ void feature_sums_kernel(const DirPlanDev p, const double* mean, double* out_sum, double* out_cnt) {
    const VT* val = static_cast<const VT*>(p.val);
    __shared__ double red[32];
    for (int64_t f = blockIdx.x; f < p.nrows; f += gridDim.x) {
        double acc = 0, cnt = 0;
        for (int32_t pnl = 0; pnl < p.npanels; ++pnl) {
            const int64_t seg = pnl * p.nrows + f;
            const int64_t b = p.segptr[seg], en = p.segptr[seg + 1];
            if (threadIdx.x == 0) cnt += static_cast<double>(en - b);
            for (int64_t s = b + threadIdx.x; s < en; s += blockDim.x) {
                const double x = static_cast<double>(val[s]);
                if (mean) {
                    const double d = x - mean[f];
                    acc += d * d;
                } else {
                    acc += x;
                }
            }
        }
        const double tot = block_sum(acc, red);
        if (threadIdx.x == 0) {
            out_sum[f] = tot;
            if (out_cnt) out_cnt[f] = cnt;
        }
        __syncthreads();
    }
}

__global__ void feature_finalize_kernel(int64_t nf, int64_t nobs, int32_t center, int32_t scale, const double* sum,
                                        const double* cnt, const double* ssd, double* center_out, double* scale_out,
                                        double* mean_tmp, int32_t stage) {
    for (int64_t f = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; f < nf;
         f += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (stage == 0) {
            const double mean = center ? sum[f] / static_cast<double>(nobs) : 0.0;
            mean_tmp[f] = mean;
            if (center) center_out[f] = mean;
        } else {
            const double mean = mean_tmp[f];
            const double var = ssd[f] + (static_cast<double>(nobs) - cnt[f]) * mean * mean;
            scale_out[f] = var != 0 ? sqrt(var / static_cast<double>(nobs - 1)) : 1.0;
        }
    }
}

}  // namespace

// Row ranges of the GEMV-transpose pass for c columns: one wave of resident
// CTAs over all column groups, at most one range per 256-row unit and at most
// kDotMaxRanges (the bound cgs_dot_grid() reports for scratch sizing).
template <typename T, bool VEC>
static int cgs_dot_ranges(int64_t L, int32_t c) {
    static const int per_sm = [] {
        int b = 0;
        const cudaError_t e = VEC ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, cgs_dot_vec_kernel<T>, kThreads, 0)
                                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, cgs_dot_kernel<T>, kThreads, 0);
        if (e != cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 1;
        }
        return b;
    }();
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms < 1) {
        cudaGetLastError();
        sms = 152;
    }
    const int groups = (c + kThreads / 32 - 1) / (kThreads / 32);
    int64_t g = static_cast<int64_t>(sms) * per_sm / groups;
    const int64_t units = (L + kDotUnit - 1) / kDotUnit;
    if (g > units) g = units;
    if (g > kDotMaxRanges) g = kDotMaxRanges;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

template <typename T>
void launch_cgs_dot(const T* Q, int64_t L, int64_t ldq, int32_t c, const T* v, double* part, double* t, Ctrl* ctrl,
                    cudaStream_t stream) {
    if (c <= 0 || L == 0) return;
    constexpr int N = Vec16<T>::N;
    // The 16-byte form for FP64 (measured: FP64-form CGS 323 -> 316 ms per
    // solve on the 2,000 x 1.3M matrix); the FP32 form keeps the scalar form's
    // 16 loads in flight (137 ms against 140 ms with the 16-byte form).
    const bool vec = std::is_same<T, double>::value && ldq % N == 0 && reinterpret_cast<uintptr_t>(Q) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(v) % 16 == 0;
    const unsigned groups = static_cast<unsigned>((c + kThreads / 32 - 1) / (kThreads / 32));
    if (vec) {
        const dim3 grid(static_cast<unsigned>(cgs_dot_ranges<T, true>(L, c)), groups);
        cgs_dot_vec_kernel<T><<<grid, kThreads, 0, stream>>>(Q, L, ldq, c, v, part, t, ctrl);
    } else {
        const dim3 grid(static_cast<unsigned>(cgs_dot_ranges<T, false>(L, c)), groups);
        cgs_dot_kernel<T><<<grid, kThreads, 0, stream>>>(Q, L, ldq, c, v, part, t, ctrl);
    }
    count_launch();
}

int cgs_update_grid(int64_t L) { return grid_for(L, kThreads, 152 * 8); }
int cgs_dot_grid(int64_t L) {
    const int64_t units = (L + kDotUnit - 1) / kDotUnit;
    return static_cast<int>(units < kDotMaxRanges ? units : kDotMaxRanges);
}

template <typename T>
void launch_cgs_update(const T* Q, int64_t L, int64_t ldq, int32_t c, const double* t, T* v, double* part,
                       double* norm_out, int32_t check_eps, int32_t check_null, Ctrl* ctrl, cudaStream_t stream) {
    constexpr int N = Vec16<T>::N;
    const bool vec = ldq % N == 0 && reinterpret_cast<uintptr_t>(Q) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(v) % 16 == 0 && L >= N;
    if (vec) {
        cgs_update_vec_kernel<T><<<grid_for(L / N, kThreads, 152 * 8), kThreads, 0, stream>>>(
            Q, L, ldq, c, t, v, part, norm_out, check_eps, check_null, ctrl);
    } else {
        cgs_update_kernel<T><<<cgs_update_grid(L), kThreads, 0, stream>>>(Q, L, ldq, c, t, v, part, norm_out,
                                                                         check_eps, check_null, ctrl);
    }
    count_launch();
}

template <typename T>
void launch_normalize(T* v, int64_t L, const double* norm, T* qcol, const T* fscale, int32_t fdivide, const T* gvec,
                      double* beta_out, double* part, double* B, int64_t bpos, int64_t ldb, Ctrl* ctrl,
                      cudaStream_t stream) {
    normalize_kernel<T, true><<<cgs_update_grid(L), kThreads, 0, stream>>>(v, L, norm, qcol, fscale, fdivide, gvec,
                                                                          beta_out, part, B, bpos, ldb, ctrl); count_launch();
}

template <typename T>
void launch_beta(const T* x, int64_t L, const T* fscale, int32_t fdivide, const T* gvec, double* beta_out,
                 double* part, Ctrl* ctrl, cudaStream_t stream) {
    normalize_kernel<T, false><<<cgs_update_grid(L), kThreads, 0, stream>>>(const_cast<T*>(x), L, nullptr, nullptr,
                                                                           fscale, fdivide, gvec, beta_out, part,
                                                                           nullptr, -1, 0, ctrl); count_launch();
}

template <typename T>
void launch_rotate(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k, T* out,
                   int64_t ldo, const T* fcol, const double* fnorm, const int32_t* abort, cudaStream_t stream) {
    if (L == 0 || (k == 0 && !fcol)) return;
    rotate_dispatch<T, T>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort, stream);
}

template <typename T>
void launch_rotate_cores(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                         T* out, int64_t ldo, const T* fcol, const double* fnorm, const int32_t* abort,
                         cudaStream_t stream) {
    if (L == 0 || (k == 0 && !fcol)) return;
    rotate_dispatch<T, T>(Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort, stream, false);
}

template <typename T>
void launch_rotate_out(const T* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                       double* out, int64_t ldo, cudaStream_t stream) {
    if (L == 0 || k == 0) return;
    rotate_dispatch<T, double>(Q, L, ldq, w, R, ldr, k, out, ldo, static_cast<const T*>(nullptr), nullptr, nullptr,
                               stream);
}

template <typename T, typename O>
cudaError_t rotate_configure_one(size_t max_smem) {
    const int b = static_cast<int>(max_smem);
    cudaError_t e = cudaFuncSetAttribute(rotate_kernel<T, O, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(rotate_kernel<T, O, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(rotate_kernel<T, O, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(rotate_kernel<T, O, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return e;
}

cudaError_t rotate_configure(size_t max_smem) {
    cudaError_t e = rotate_configure_one<float, float>(max_smem);
    if (e == cudaSuccess && max_smem >= kRotPipeSmem) {
        e = cudaFuncSetAttribute(rotate_f32_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kRotPipeSmem));
        g_rotate_pipe_ok = e == cudaSuccess;
    }
    if (e == cudaSuccess) e = rotate_configure_one<double, double>(max_smem);
    if (e == cudaSuccess) e = rotate_configure_one<float, double>(max_smem);
    return e;
}

template <typename A, typename B>
void launch_convert(const A* in, B* out, int64_t n, cudaStream_t stream) {
    if (n == 0) return;
    convert_kernel<A, B><<<grid_for(n, 256, 152 * 16), 256, 0, stream>>>(in, out, n); count_launch();
}

void launch_realize(const DirPlanDev& p, double* out, int64_t ld, int32_t transpose, cudaStream_t stream) {
    if (p.nseg == 0) return;
    const int grid = static_cast<int>(std::min<int64_t>(p.nseg, 152 * 64));
    if (p.val_f64) {
        realize_kernel<double><<<grid, 128, 0, stream>>>(p, out, ld, transpose);
    } else {
        realize_kernel<float><<<grid, 128, 0, stream>>>(p, out, ld, transpose);
    }
    count_launch();
}

void launch_realize_ops(double* A, int64_t m, int64_t n, const double* center, const double* scale,
                        int32_t scale_column, int32_t scale_divide, int32_t center_outer, cudaStream_t stream) {
    if (m * n == 0) return;
    realize_ops_kernel<<<grid_for(m * n, 256, 152 * 16), 256, 0, stream>>>(A, m, n, center, scale, scale_column,
                                                                         scale_divide, center_outer); count_launch();
}

// scratch: 4 * nrows doubles.
void launch_feature_stats(const DirPlanDev& p, int64_t nobs, int32_t center, int32_t scale, double* center_out,
                          double* scale_out, double* scratch, cudaStream_t stream) {
    const int64_t nf = p.nrows;
    if (nf == 0) return;
    double* sum = scratch;
    double* cnt = scratch + nf;
    double* ssd = scratch + 2 * nf;
    double* mean = scratch + 3 * nf;
    const int grid = static_cast<int>(std::min<int64_t>(nf, 152 * 16));
    if (p.val_f64) {
        feature_sums_kernel<double><<<grid, 256, 0, stream>>>(p, nullptr, sum, cnt);
    } else {
        feature_sums_kernel<float><<<grid, 256, 0, stream>>>(p, nullptr, sum, cnt);
    }
    count_launch();
    feature_finalize_kernel<<<grid_for(nf, 256, 1024), 256, 0, stream>>>(nf, nobs, center, scale, sum, cnt, ssd,
                                                                         center_out, scale_out, mean, 0); count_launch();
    if (scale) {
        if (p.val_f64) {
            feature_sums_kernel<double><<<grid, 256, 0, stream>>>(p, mean, ssd, nullptr);
        } else {
            feature_sums_kernel<float><<<grid, 256, 0, stream>>>(p, mean, ssd, nullptr);
        }
        count_launch();
        feature_finalize_kernel<<<grid_for(nf, 256, 1024), 256, 0, stream>>>(nf, nobs, center, scale, sum, cnt, ssd,
                                                                             center_out, scale_out, mean, 1); count_launch();
    }
}

#define IRLBA_INST(T)                                                                                               \
    template void launch_cgs_dot<T>(const T*, int64_t, int64_t, int32_t, const T*, double*, double*, Ctrl*,         \
                                    cudaStream_t);                                                                  \
    template void launch_cgs_update<T>(const T*, int64_t, int64_t, int32_t, const double*, T*, double*, double*,   \
                                       int32_t, int32_t, Ctrl*, cudaStream_t);                                      \
    template void launch_normalize<T>(T*, int64_t, const double*, T*, const T*, int32_t, const T*, double*,         \
                                      double*, double*, int64_t, int64_t, Ctrl*, cudaStream_t);                     \
    template void launch_beta<T>(const T*, int64_t, const T*, int32_t, const T*, double*, double*, Ctrl*,           \
                                 cudaStream_t);                                                                     \
    template void launch_rotate<T>(const T*, int64_t, int64_t, int32_t, const double*, int32_t, int32_t, T*,        \
                                   int64_t, const T*, const double*, const int32_t*, cudaStream_t);                 \
    template void launch_rotate_out<T>(const T*, int64_t, int64_t, int32_t, const double*, int32_t, int32_t,       \
                                       double*, int64_t, cudaStream_t);                                             \
    template void launch_rotate_cores<T>(const T*, int64_t, int64_t, int32_t, const double*, int32_t, int32_t, T*,  \
                                         int64_t, const T*, const double*, const int32_t*, cudaStream_t);
IRLBA_INST(float)
IRLBA_INST(double)
#undef IRLBA_INST

template void launch_convert<float, double>(const float*, double*, int64_t, cudaStream_t);
template void launch_convert<double, float>(const double*, float*, int64_t, cudaStream_t);
template void launch_convert<double, double>(const double*, double*, int64_t, cudaStream_t);
template void launch_convert<float, float>(const float*, float*, int64_t, cudaStream_t);

}  // namespace irlba_gb300
