// Batched form: many PCAs of uneven size in one persistent launch.
//
// Each CTA pulls problems from a device queue (largest first) and runs the whole
// centred/scaled PCA of one problem: column statistics (pca.hpp:85-109), the
// IRLBA restart loop of compute.hpp:141-308 with Lanczos bidiagonalization
// (lanczos.hpp:54-143), full Gram-Schmidt reorthogonalization, the one-sided
// Jacobi SVD of B, the convergence test, update_k, the basis rotation and the
// output assembly (compute.hpp:298-305, pca.hpp:128-136). The arithmetic is the
// engine's FP32 form: FP32 matrix values, bases and matvecs; FP64 coefficient
// and norm accumulation, recurrence, small SVD and convergence test. Every
// synchronization is a __syncthreads of the CTA; no CTA waits on another.
//
// Shared memory holds a persistent block (B, singular values, reduction slots)
// and a union region that is either the staged gathered vector of an SpMV or,
// during a restart, the Jacobi work arrays and the left/right singular vectors.
//
// A problem whose Lanczos vector falls into an invariant subspace (a norm below
// the invariant-subspace tolerance) stops with status 2; the host re-solves it
// with the single-problem engine, which refills from the host random engine as
// the reference does (lanczos.hpp:101-106,124-129).

#include "jacobi.cuh"
#include "kernels.cuh"
#include "segdot.cuh"

namespace irlba_gb300 {

namespace {

constexpr int kBT = 512;                   // threads per CTA
constexpr int kBW = kBT / 32;              // warps per CTA
constexpr int kWM = kBatchMaxWork;         // largest working subspace
constexpr int64_t kStageFloats = 50176;    // 196 KiB of staged vector

struct Persist {
    double B[kWM * kWM];
    double BS[kWM];
    double prevS[kWM];
    double res[kWM];
    double t[kWM];
    double norms[kWM];
    double pairs[3 * (kWM / 2)];
    double red[kBW * kWM];
    float t32[kWM];
    float R32[kWM * kWM];
    int order[kWM];
    int flags[8];
    int next;
};
constexpr size_t kPersistBytes = (sizeof(Persist) + 127) / 128 * 128;
constexpr size_t kJacobiBytes = 4 * sizeof(double) * kWM * kWM;

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Sum over the CTA in a fixed order; every thread gets the value.
__device__ double cta_sum(double v, Persist& ps) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) ps.red[warp] = v;
    __syncthreads();
    double r = 0;
#pragma unroll
    for (int w = 0; w < kBW; ++w) r += ps.red[w];
    __syncthreads();
    return r;
}

// Bulk prefetch of bytes [a, a + n) into L2 (no registers, no shared memory);
// the range is widened to 16-byte boundaries, which stay inside the pooled
// allocations (16-byte aligned, padded).
__device__ __forceinline__ void prefetch_l2(const void* a, size_t n) {
    uintptr_t b = reinterpret_cast<uintptr_t>(a) & ~static_cast<uintptr_t>(15);
    const uintptr_t e = (reinterpret_cast<uintptr_t>(a) + n + 15) & ~static_cast<uintptr_t>(15);
    for (; b < e; b += 32768) {
        const uint32_t sz = static_cast<uint32_t>(e - b < 32768 ? e - b : 32768);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b), "r"(sz) : "memory");
    }
}

// Values and indices of rows [ra, rb) of d into L2.
__device__ __forceinline__ void prefetch_rows(const BatchDir& d, int64_t ra, int64_t rb) {
    const int64_t b = d.ptr[ra], e = d.ptr[rb];
    if (e <= b) return;
    prefetch_l2(d.val + b, sizeof(float) * static_cast<size_t>(e - b));
    prefetch_l2(static_cast<const char*>(d.idx) + b * d.idx_bytes, static_cast<size_t>(d.idx_bytes) * (e - b));
}

// y[r] = epi(sum_s val[s] x[idx[s]]) over the rows of d, G lanes per row:
//   epi(v) = ((v - beta * (cvec ? cvec[r] : 1)) / (oscale ? oscale[r] : 1)) - alpha q[r]
template <bool STAGED, int G>
__device__ void spmv_rows(const BatchDir& d, const float* xs, const float* xg, float* __restrict__ y, float beta,
                          const float* cvec, const float* oscale, float alpha, const float* q) {
    constexpr int kGroups = kBT / G;
    const int gid = threadIdx.x / G;
    const int gl = threadIdx.x % G;
    Gather<float, STAGED> g;
    g.xs = xs;
    g.x = xg;
    const int64_t rows = d.rows;
    // Thread 0 keeps the L2 `prefetch` row batches ahead of the groups.
    const int pf = d.prefetch;
    if (pf > 0 && threadIdx.x == 0) prefetch_rows(d, 0, min(rows, static_cast<int64_t>(pf + 1) * kGroups));
    int64_t r = gid;
    int64_t b = 0, e = 0;
    if (r < rows) {
        b = d.ptr[r];
        e = d.ptr[r + 1];
    }
    for (int64_t r0 = 0; r0 < rows; r0 += kGroups) {
        if (pf > 0 && threadIdx.x == 0) {
            const int64_t ra = r0 + static_cast<int64_t>(pf + 1) * kGroups;
            if (ra < rows) prefetch_rows(d, ra, min(rows, ra + kGroups));
        }
        const int64_t rn = r + kGroups;
        int64_t nb = 0, ne = 0;
        if (rn < rows) {
            nb = d.ptr[rn];
            ne = d.ptr[rn + 1];
        }
        float acc = 0;
        if (r < rows) acc = segment_dot<float, float, STAGED, G>(d.val, d.idx, g, b, e, gl);
        acc = group_sum<G>(acc);
        if (gl == 0 && r < rows) {
            float v = acc - (cvec ? beta * cvec[r] : beta);
            if (oscale) v /= oscale[r];
            if (q) v -= alpha * q[r];
            y[r] = v;
        }
        r = rn;
        b = nb;
        e = ne;
    }
}

template <bool STAGED>
__device__ void spmv_dispatch(const BatchDir& d, const float* xs, const float* xg, float* y, float beta,
                              const float* cvec, const float* oscale, float alpha, const float* q) {
    switch (d.group) {
        case 4: spmv_rows<STAGED, 4>(d, xs, xg, y, beta, cvec, oscale, alpha, q); break;
        case 8: spmv_rows<STAGED, 8>(d, xs, xg, y, beta, cvec, oscale, alpha, q); break;
        case 16: spmv_rows<STAGED, 16>(d, xs, xg, y, beta, cvec, oscale, alpha, q); break;
        default: spmv_rows<STAGED, 32>(d, xs, xg, y, beta, cvec, oscale, alpha, q); break;
    }
}

// One direction: stage (or scale into global scratch) the gathered vector,
// then the row products. Returns after a CTA barrier.
__device__ void batch_spmv(const BatchDir& d, const float* x, const float* xscale, float* xscratch, float* stage,
                           float* y, float beta, const float* cvec, const float* oscale, float alpha, const float* q) {
    if (d.staged) {
        for (int64_t c = threadIdx.x; c < d.cols; c += kBT) {
            float v = x[c];
            if (xscale) v /= xscale[c];
            stage[c] = v;
        }
        __syncthreads();
        spmv_dispatch<true>(d, stage, nullptr, y, beta, cvec, oscale, alpha, q);
    } else {
        const float* xg = x;
        if (xscale) {
            for (int64_t c = threadIdx.x; c < d.cols; c += kBT) xscratch[c] = x[c] / xscale[c];
            __syncthreads();
            xg = xscratch;
        }
        spmv_dispatch<false>(d, nullptr, xg, y, beta, cvec, oscale, alpha, q);
    }
    __syncthreads();
}

// t[j] = sum_r Q[r, j] v[r] for j < c: FP32 products summed 8 rows at a time,
// then FP64 (the FP32 form's reorthogonalization coefficients).
__device__ void cta_dot(const float* __restrict__ Q, int64_t L, int64_t ldq, int c, const float* __restrict__ v,
                        Persist& ps) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc[kWM];
    float part[kWM];
#pragma unroll
    for (int j = 0; j < kWM; ++j) {
        acc[j] = 0;
        part[j] = 0;
    }
    int cnt = 0;
    for (int64_t r = threadIdx.x; r < L; r += kBT) {
        const float vr = v[r];
#pragma unroll
        for (int j = 0; j < kWM; ++j)
            if (j < c) part[j] = fmaf(Q[r + j * ldq], vr, part[j]);
        if (++cnt == 8) {
#pragma unroll
            for (int j = 0; j < kWM; ++j) {
                acc[j] += static_cast<double>(part[j]);
                part[j] = 0;
            }
            cnt = 0;
        }
    }
#pragma unroll
    for (int j = 0; j < kWM; ++j) acc[j] += static_cast<double>(part[j]);
#pragma unroll
    for (int j = 0; j < kWM; ++j) {
        if (j < c) {
            const double s = warp_sum(acc[j]);
            if (lane == 0) ps.red[warp * kWM + j] = s;
        }
    }
    __syncthreads();
    if (threadIdx.x < c) {
        double s = 0;
#pragma unroll
        for (int w = 0; w < kBW; ++w) s += ps.red[w * kWM + threadIdx.x];
        ps.t[threadIdx.x] = s;
        ps.t32[threadIdx.x] = static_cast<float>(s);
    }
    __syncthreads();
}

// Reorthogonalize v against Q[:, :c] (classical Gram-Schmidt, one pass as in
// lanczos.hpp:27-44) and return ||v|| in FP64.
__device__ double cta_cgs(const float* __restrict__ Q, int64_t L, int64_t ldq, int c, float* __restrict__ v,
                          Persist& ps) {
    if (c > 0) cta_dot(Q, L, ldq, c, v, ps);
    double sq = 0;
    for (int64_t r = threadIdx.x; r < L; r += kBT) {
        float s = 0;
        for (int j = 0; j < c; ++j) s = fmaf(Q[r + j * ldq], ps.t32[j], s);
        const float nv = v[r] - s;
        v[r] = nv;
        sq += static_cast<double>(nv) * static_cast<double>(nv);
    }
    return sqrt(cta_sum(sq, ps));
}

// v /= norm; qcol = v. Returns sum_r v[r] (the centring scalar of the next
// adjoint) when want_sum.
__device__ double cta_normalize(float* __restrict__ v, int64_t L, double norm, float* __restrict__ qcol,
                                bool want_sum, Persist& ps) {
    const float inv = static_cast<float>(1.0 / norm);
    double acc = 0;
    for (int64_t r = threadIdx.x; r < L; r += kBT) {
        const float x = v[r] * inv;
        v[r] = x;
        qcol[r] = x;
        acc += static_cast<double>(x);
    }
    if (!want_sum) {
        __syncthreads();
        return 0.0;
    }
    return cta_sum(acc, ps);
}

// R32[j][i] = M[j + i * w] for j < w, i < k (FP64 column-major -> FP32).
__device__ void load_rotation(const double* M, int w, int k, Persist& ps) {
    for (int e = threadIdx.x; e < kWM * kWM; e += kBT) {
        const int j = e / kWM, i = e % kWM;
        ps.R32[e] = (j < w && i < k) ? static_cast<float>(M[j + i * w]) : 0.0f;
    }
    __syncthreads();
}

// Q[:, :k] = Q[:, :w] R (in place, one row per thread); Q[:, k] = fcol * finv.
__device__ void cta_rotate(float* Q, int64_t L, int64_t ldq, int w, int k, const float* fcol, float finv,
                           const Persist& ps) {
    for (int64_t r = threadIdx.x; r < L; r += kBT) {
        float row[kWM];
#pragma unroll
        for (int j = 0; j < kWM; ++j) row[j] = j < w ? Q[r + j * ldq] : 0.0f;
        float acc[kWM];
#pragma unroll
        for (int i = 0; i < kWM; ++i) acc[i] = 0;
#pragma unroll
        for (int j = 0; j < kWM; ++j) {
            const float rj = row[j];
#pragma unroll
            for (int i = 0; i < kWM; ++i) acc[i] = fmaf(rj, ps.R32[j * kWM + i], acc[i]);
        }
#pragma unroll
        for (int i = 0; i < kWM; ++i)
            if (i < k) Q[r + i * ldq] = acc[i];
        if (fcol) Q[r + static_cast<int64_t>(k) * ldq] = fcol[r] * finv;
    }
    __syncthreads();
}

// Column means and standard deviations over the feature rows of the adjoint
// CSR (pca.hpp:85-109): implicit zeros enter the variance analytically, and a
// zero-variance column keeps a scale of 1. One warp per feature.
__device__ void column_stats(const BatchProblem& P, bool center, bool scale) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t m = P.m;
    for (int64_t f = warp; f < P.n; f += kBW) {
        const int64_t b = P.adj.ptr[f], e = P.adj.ptr[f + 1];
        double s = 0;
        for (int64_t i = b + lane; i < e; i += 32) s += static_cast<double>(P.adj.val[i]);
        s = warp_sum(s);
        const double mean = center ? s / static_cast<double>(m) : 0.0;
        if (lane == 0 && center) {
            P.center64[f] = mean;
            P.center[f] = static_cast<float>(mean);
        }
        if (scale) {
            double d2 = 0;
            for (int64_t i = b + lane; i < e; i += 32) {
                const double d = static_cast<double>(P.adj.val[i]) - mean;
                d2 += d * d;
            }
            d2 = warp_sum(d2);
            const double var = d2 + static_cast<double>(m - (e - b)) * mean * mean;
            const double sd = var != 0 ? sqrt(var / static_cast<double>(m - 1)) : 1.0;
            if (lane == 0) {
                P.scale64[f] = sd;
                P.scale[f] = static_cast<float>(sd);
            }
        }
    }
    __syncthreads();
}

__device__ void solve_problem(const BatchProblem& P, const BatchParams& prm, BatchResult* result, Persist& ps,
                              unsigned char* uni) {
    const int64_t m = P.m, n = P.n;
    const int w = prm.work, req = prm.number;
    const bool center = prm.center != 0, scale = prm.scale != 0;
    float* stage = reinterpret_cast<float*>(uni);
    double* G = reinterpret_cast<double*>(uni);
    double* Vj = G + w * w;
    double* BU = Vj + w * w;
    double* BV = BU + w * w;

    if (center || scale) column_stats(P, center, scale);
    const float* cvec = center ? P.center : nullptr;
    const float* svec = scale ? P.scale : nullptr;

    // Start vector (compute.hpp:179-190), normalized in FP64.
    {
        double s = 0;
        for (int64_t c = threadIdx.x; c < n; c += kBT) s += P.init[c] * P.init[c];
        const double nrm = sqrt(cta_sum(s, ps));
        for (int64_t c = threadIdx.x; c < n; c += kBT) P.V[c] = static_cast<float>(P.init[c] / nrm);
    }
    for (int e = threadIdx.x; e < kWM * kWM; e += kBT) ps.B[e] = 0.0;
    for (int e = threadIdx.x; e < kWM; e += kBT) ps.prevS[e] = 0.0;
    __syncthreads();

    // multiply: y = A (x / s) - (c . (x / s)) - alpha q   (centered.hpp, scaled.hpp)
    auto multiply = [&](const float* x, float* y, float alpha, const float* q) {
        double b = 0;
        if (cvec) {
            for (int64_t c = threadIdx.x; c < n; c += kBT) {
                const float xv = svec ? x[c] / svec[c] : x[c];
                b += static_cast<double>(xv) * static_cast<double>(cvec[c]);
            }
            b = cta_sum(b, ps);
        }
        batch_spmv(P.mul, x, svec, P.xs, stage, y, static_cast<float>(b), nullptr, nullptr, alpha, q);
    };
    // adjoint: out = (A^T y - (sum y) c) / s - alpha q
    auto adjoint = [&](const float* y, float* out, double ysum, float alpha, const float* q) {
        batch_spmv(P.adj, y, nullptr, nullptr, stage, out, cvec ? static_cast<float>(ysum) : 0.0f, cvec, svec, alpha,
                   q);
    };

    const double eps = prm.eps;
    int iter = 0, k = 0, status = 0, sweeps = 0;
    bool converged = false;
    int64_t steps = 0;
    for (; iter < prm.max_iter; ++iter) {
        // Lanczos bidiagonalization from column k (lanczos.hpp:54-143).
        multiply(P.V + k * P.ldv, P.Wn, 0.0f, nullptr);
        double S = cta_cgs(P.W, m, P.ldw, k, P.Wn, ps);
        if (S < eps) {
            status = 2;
            break;
        }
        double ysum = cta_normalize(P.Wn, m, S, P.W + k * P.ldw, cvec != nullptr, ps);
        double R_F = 0;
        for (int j = k; j < w; ++j) {
            adjoint(P.Wn, P.F, ysum, static_cast<float>(S), P.V + j * P.ldv);
            R_F = cta_cgs(P.V, n, P.ldv, j + 1, P.F, ps);
            if (j + 1 < w) {
                if (R_F < eps) {
                    status = 2;
                    break;
                }
                cta_normalize(P.F, n, R_F, P.V + (j + 1) * P.ldv, false, ps);
                if (threadIdx.x == 0) {
                    ps.B[j + j * w] = S;
                    ps.B[j + (j + 1) * w] = R_F;
                }
                multiply(P.V + (j + 1) * P.ldv, P.Wn, static_cast<float>(R_F), P.W + j * P.ldw);
                S = cta_cgs(P.W, m, P.ldw, j + 1, P.Wn, ps);
                if (S < eps) {
                    status = 2;
                    break;
                }
                ysum = cta_normalize(P.Wn, m, S, P.W + (j + 1) * P.ldw, cvec != nullptr, ps);
            } else if (threadIdx.x == 0) {
                ps.B[j + j * w] = S;
            }
        }
        if (status) break;
        steps += w - k;
        __syncthreads();

        // Restart (compute.hpp:225-293): SVD of B, convergence test, update_k.
        for (int e = threadIdx.x; e < w * w; e += kBT) {
            G[e] = ps.B[e];
            Vj[e] = ((e / w) == (e % w)) ? 1.0 : 0.0;
        }
        __syncthreads();
        jacobi::jacobi_sweeps(G, w, w, Vj, &ps.flags[0], &ps.flags[1], &ps.flags[2], ps.norms, ps.pairs);
        sweeps += ps.flags[0];
        jacobi::finish_svd(G, w, w, Vj, ps.BS, BU, w, BV, w, ps.norms, ps.order);
        if (threadIdx.x == 0) {
            int conv = 0, n_conv = 0;
            if (ps.B[(w - 1) + (w - 1) * w] == 0.0) {
                conv = 1;
            } else {
                for (int j = 0; j < w; ++j) ps.res[j] = R_F * BU[(w - 1) + j * w];
                if (iter > 0) {
                    double smax = ps.BS[0];
                    for (int j = 1; j < w; ++j) smax = ps.BS[j] > smax ? ps.BS[j] : smax;
                    const double threshold = smax * prm.tol;
                    for (int j = 0; j < w; ++j)
                        if (fabs(ps.res[j]) <= threshold && fabs(ps.BS[j] - ps.prevS[j]) / ps.BS[j] <= prm.svtol)
                            ++n_conv;
                    if (n_conv >= req) conv = 1;
                }
            }
            ps.flags[3] = conv;
            ps.flags[4] = conv ? k : jacobi::update_k_dev(k, req, n_conv, w);
            if (!conv)
                for (int j = 0; j < w; ++j) ps.prevS[j] = ps.BS[j];
        }
        __syncthreads();
        if (ps.flags[3]) {
            converged = true;
            break;
        }
        const int kn = ps.flags[4];
        // V[:, :kn] = V BV[:, :kn], V[:, kn] = F / ||F||, W[:, :kn] = W BU[:, :kn]
        // (compute.hpp:268-280); B = diag(S[:kn]) with residuals in column kn.
        load_rotation(BV, w, kn, ps);
        cta_rotate(P.V, n, P.ldv, w, kn, P.F, static_cast<float>(1.0 / R_F), ps);
        load_rotation(BU, w, kn, ps);
        cta_rotate(P.W, m, P.ldw, w, kn, nullptr, 0.0f, ps);
        for (int e = threadIdx.x; e < w * w; e += kBT) ps.B[e] = 0.0;
        __syncthreads();
        if (threadIdx.x < kn) {
            ps.B[threadIdx.x + threadIdx.x * w] = ps.BS[threadIdx.x];
            ps.B[threadIdx.x + kn * w] = ps.res[threadIdx.x];
        }
        __syncthreads();
        k = kn;
    }

    if (status == 0) {
        // scores = W BU[:, :r] diag(S), rotation = V BV[:, :r],
        // variances = S^2 / (m - 1) when n > 1 (compute.hpp:298-305, pca.hpp:130-136).
        for (int64_t e = threadIdx.x; e < m * req; e += kBT) {
            const int64_t r = e % m;
            const int i = static_cast<int>(e / m);
            double s = 0;
            for (int j = 0; j < w; ++j) s += static_cast<double>(P.W[r + j * P.ldw]) * BU[j + i * w];
            P.scores[e] = s * ps.BS[i];
        }
        for (int64_t e = threadIdx.x; e < n * req; e += kBT) {
            const int64_t r = e % n;
            const int i = static_cast<int>(e / n);
            double s = 0;
            for (int j = 0; j < w; ++j) s += static_cast<double>(P.V[r + j * P.ldv]) * BV[j + i * w];
            P.rotation[e] = s;
        }
        for (int i = threadIdx.x; i < req; i += kBT)
            P.variances[i] = n > 1 ? ps.BS[i] * ps.BS[i] / static_cast<double>(m - 1) : ps.BS[i];
    }
    if (threadIdx.x == 0) {
        result->status = status;
        result->converged = converged ? 1 : 0;
        result->iterations = converged ? iter + 1 : iter;
        result->svd_sweeps = sweeps;
        result->steps = steps;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kBT, 1) batch_pca_kernel(const BatchProblem* __restrict__ probs,
                                                           const int32_t* __restrict__ order, int32_t count,
                                                           BatchParams prm, BatchResult* results, uint32_t* queue) {
    extern __shared__ __align__(128) unsigned char smem[];
    Persist& ps = *reinterpret_cast<Persist*>(smem);
    unsigned char* uni = smem + kPersistBytes;
    while (true) {
        if (threadIdx.x == 0) ps.next = static_cast<int>(atomicAdd(queue, 1u));
        __syncthreads();
        const int i = ps.next;
        __syncthreads();
        if (i >= count) break;
        const int p = order[i];
        const uint64_t t0 = global_ns();
        solve_problem(probs[p], prm, results + p, ps, uni);
        if (threadIdx.x == 0) {
            results[p].t_start = t0;
            results[p].t_end = global_ns();
        }
    }
}

// Autotuner probe: each CTA times `reps` SpMVs (staging included) of the
// problems it takes, in the given order, and keeps the best time in SM cycles.
__global__ void __launch_bounds__(kBT, 1) batch_spmv_probe_kernel(const BatchProblem* __restrict__ probs,
                                                                  const int32_t* __restrict__ order, int32_t count,
                                                                  int32_t adjoint, int32_t group, int32_t prefetch,
                                                                  int32_t reps, uint64_t* cycles_out) {
    extern __shared__ __align__(128) unsigned char smem[];
    float* stage = reinterpret_cast<float*>(smem + kPersistBytes);
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        const BatchProblem& P = probs[order[i]];
        BatchDir d = adjoint ? P.adj : P.mul;
        d.group = group;
        d.prefetch = prefetch;
        float* x = adjoint ? P.Wn : P.xs;
        float* y = adjoint ? P.F : P.Wn;
        for (int64_t c = threadIdx.x; c < d.cols; c += kBT) x[c] = 1.0f;
        __syncthreads();
        uint64_t best = ~0ull;
        for (int rep = 0; rep < reps; ++rep) {
            __syncthreads();
            const uint64_t t0 = clock64();
            batch_spmv(d, x, nullptr, nullptr, stage, y, 0.0f, nullptr, nullptr, 0.0f, nullptr);
            const uint64_t t1 = clock64();
            best = t1 - t0 < best ? t1 - t0 : best;
        }
        if (threadIdx.x == 0) cycles_out[order[i]] = best;
        __syncthreads();
    }
}

}  // namespace

int64_t batch_stage_limit() { return kStageFloats; }

size_t batch_smem_bytes(int64_t max_staged) {
    const size_t stage = sizeof(float) * static_cast<size_t>(max_staged < 0 ? 0 : max_staged);
    return kPersistBytes + (stage > kJacobiBytes ? stage : kJacobiBytes);
}

cudaError_t batch_configure(size_t max_smem_optin) {
    const size_t want = batch_smem_bytes(kStageFloats);
    if (want > max_smem_optin) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(batch_pca_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(want));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(batch_spmv_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(want));
    return e;
}

void launch_batch_pca(const BatchProblem* probs, const int32_t* order, int32_t count, const BatchParams& prm,
                      BatchResult* results, uint32_t* queue, int grid, size_t smem, cudaStream_t stream) {
    batch_pca_kernel<<<grid, kBT, smem, stream>>>(probs, order, count, prm, results, queue);
    count_launch();
}

void launch_batch_spmv_probe(const BatchProblem* probs, const int32_t* order, int32_t count, int32_t adjoint,
                             int32_t group, int32_t prefetch, int32_t reps, uint64_t* cycles_out, int grid,
                             size_t smem, cudaStream_t stream) {
    batch_spmv_probe_kernel<<<grid, kBT, smem, stream>>>(probs, order, count, adjoint, group, prefetch, reps,
                                                         cycles_out);
    count_launch();
}

}  // namespace irlba_gb300
