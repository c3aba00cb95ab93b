// Batched form: many PCAs of uneven size in one persistent launch.
//
// A team of C CTAs (a thread-block cluster; C = 1, 2, 4 or 8) takes one matrix at
// a time from a device queue (largest first) and runs its whole centred/scaled
// PCA: column statistics (pca.hpp:85-109), the IRLBA restart loop of
// compute.hpp:141-308 with Lanczos bidiagonalization (lanczos.hpp:54-143), full
// Gram-Schmidt reorthogonalization, the one-sided Jacobi SVD of B, the
// convergence test, update_k, the basis rotation and the output assembly
// (compute.hpp:298-305, pca.hpp:128-136).
//
// Work split inside a team: every length-m quantity (cells: W, the multiply's
// output) and every length-n quantity (genes: V, F, the adjoint's output, the
// column statistics) is cut into C contiguous row ranges, one per CTA. Each
// SpMV stages the whole gathered vector in every CTA's shared memory and
// computes the CTA's own output rows. Sums (reorthogonalization coefficients,
// norms, centring scalars) are reduced inside the CTA, exchanged through
// distributed shared memory and added in rank order, so every CTA holds the
// same values; the small SVD of B is then repeated identically by every CTA,
// which needs no communication. Cluster barriers (with a device-scope fence
// before them) separate the phases; no CTA waits on anything outside its own
// cluster.
//
// Arithmetic: the engine's FP32 form (FP32 matrix values, bases and matvecs;
// FP64 coefficient and norm accumulation, recurrence, small SVD and
// convergence test).
//
// A problem whose Lanczos vector falls into an invariant subspace (a norm below
// the invariant-subspace tolerance) stops with status 2; the host re-solves it
// with the single-problem engine, which refills from the host random engine as
// the reference does (lanczos.hpp:101-106,124-129).

#include <cooperative_groups.h>

#include "jacobi.cuh"
#include "kernels.cuh"
#include "segdot.cuh"

namespace irlba_gb300 {

namespace {

namespace cg = cooperative_groups;

#ifndef IRLBA_GB300_BATCH_THREADS
#define IRLBA_GB300_BATCH_THREADS 512
#endif
constexpr int kBT = IRLBA_GB300_BATCH_THREADS;   // threads per CTA
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
    double xred[2][kWM];     // this CTA's partials, read by the team (double-buffered)
    double bcast;
    float t32[kWM];
    float RV[kWM * kWM];     // restart rotations (FP32), V side and W side
    float RW[kWM * kWM];
    int order[kWM];
    int flags[8];
    int assign[8];
    int joint;
};
constexpr size_t kPersistBytes = (sizeof(Persist) + 127) / 128 * 128;
constexpr size_t kJacobiBytes = 4 * sizeof(double) * kWM * kWM;

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// One team: this CTA's rank, its row ranges and the reduction slot.
template <int C>
struct Team {
    int rank = 0;
    int slot = 0;
    __device__ int64_t lo(int64_t L) const { return L * rank / C; }
    __device__ int64_t hi(int64_t L) const { return L * (rank + 1) / C; }
    // Barrier over the team; writes to global memory before it are visible to
    // the team after it.
    __device__ void sync() const {
        if constexpr (C > 1) {
            __threadfence();
            cg::this_cluster().sync();
        } else {
            __syncthreads();
        }
    }
    template <typename T>
    __device__ T* peer(T* p, int r) const {
        if constexpr (C > 1) return cg::this_cluster().map_shared_rank(p, r);
        else return p;
    }
};

// Sum over the team in a fixed order; every thread gets the value.
template <int C>
__device__ double team_sum(double v, Team<C>& tm, Persist& ps) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) ps.red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
#pragma unroll
        for (int w = 0; w < kBW; ++w) s += ps.red[w];
        ps.xred[tm.slot][0] = s;
    }
    tm.sync();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int r = 0; r < C; ++r) s += tm.peer(ps.xred[tm.slot], r)[0];
        ps.bcast = s;
    }
    tm.slot ^= 1;
    __syncthreads();
    return ps.bcast;
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

// y[r] = epi(sum_s val[s] x[idx[s]]) over rows [r_lo, r_hi) of d, G lanes per row:
//   epi(v) = ((v - beta * (cvec ? cvec[r] : 1)) / (oscale ? oscale[r] : 1)) - alpha q[r]
template <bool STAGED, int G>
__device__ void spmv_rows(const BatchDir& d, int64_t r_lo, int64_t r_hi, const float* xs, const float* xg,
                          float* __restrict__ y, float beta, const float* cvec, const float* oscale, float alpha,
                          const float* q) {
    constexpr int kGroups = kBT / G;
    const int gid = threadIdx.x / G;
    const int gl = threadIdx.x % G;
    Gather<float, STAGED> g;
    g.xs = xs;
    g.x = xg;
    // Thread 0 keeps the L2 `prefetch` row batches ahead of the groups.
    const int pf = d.prefetch;
    if (pf > 0 && threadIdx.x == 0) prefetch_rows(d, r_lo, min(r_hi, r_lo + static_cast<int64_t>(pf + 1) * kGroups));
    int64_t r = r_lo + gid;
    int64_t b = 0, e = 0;
    if (r < r_hi) {
        b = d.ptr[r];
        e = d.ptr[r + 1];
    }
    for (int64_t r0 = r_lo; r0 < r_hi; r0 += kGroups) {
        if (pf > 0 && threadIdx.x == 0) {
            const int64_t ra = r0 + static_cast<int64_t>(pf + 1) * kGroups;
            if (ra < r_hi) prefetch_rows(d, ra, min(r_hi, ra + kGroups));
        }
        const int64_t rn = r + kGroups;
        int64_t nb = 0, ne = 0;
        if (rn < r_hi) {
            nb = d.ptr[rn];
            ne = d.ptr[rn + 1];
        }
        float acc = 0;
        if (r < r_hi) acc = segment_dot<float, float, STAGED, G>(d.val, d.idx, g, b, e, gl);
        acc = group_sum<G>(acc);
        if (gl == 0 && r < r_hi) {
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
__device__ void spmv_dispatch(const BatchDir& d, int64_t r_lo, int64_t r_hi, const float* xs, const float* xg,
                              float* y, float beta, const float* cvec, const float* oscale, float alpha,
                              const float* q) {
    switch (d.group) {
        case 4: spmv_rows<STAGED, 4>(d, r_lo, r_hi, xs, xg, y, beta, cvec, oscale, alpha, q); break;
        case 8: spmv_rows<STAGED, 8>(d, r_lo, r_hi, xs, xg, y, beta, cvec, oscale, alpha, q); break;
        case 16: spmv_rows<STAGED, 16>(d, r_lo, r_hi, xs, xg, y, beta, cvec, oscale, alpha, q); break;
        default: spmv_rows<STAGED, 32>(d, r_lo, r_hi, xs, xg, y, beta, cvec, oscale, alpha, q); break;
    }
}

// One direction over this CTA's output rows. The gathered vector x (written
// by the whole team) is staged in shared memory, or, when too long, scaled
// into the CTA's slice of a global scratch (then the team synchronizes before
// the gathers). Returns after a CTA barrier.
template <int C>
__device__ void batch_spmv(const BatchDir& d, const Team<C>& tm, const float* x, const float* xscale,
                           float* xscratch, float* stage, float* y, float beta, const float* cvec,
                           const float* oscale, float alpha, const float* q) {
    const int64_t r_lo = tm.lo(d.rows), r_hi = tm.hi(d.rows);
    if (d.staged) {
        for (int64_t c = threadIdx.x; c < d.cols; c += kBT) {
            float v = __ldcg(x + c);
            if (xscale) v /= __ldcg(xscale + c);
            stage[c] = v;
        }
        __syncthreads();
        spmv_dispatch<true>(d, r_lo, r_hi, stage, nullptr, y, beta, cvec, oscale, alpha, q);
    } else {
        const float* xg = x;
        if (xscale) {
            for (int64_t c = tm.lo(d.cols) + threadIdx.x; c < tm.hi(d.cols); c += kBT)
                xscratch[c] = __ldcg(x + c) / __ldcg(xscale + c);
            tm.sync();
            xg = xscratch;
        }
        spmv_dispatch<false>(d, r_lo, r_hi, nullptr, xg, y, beta, cvec, oscale, alpha, q);
    }
    __syncthreads();
}

// t[j] = sum_r Q[r, j] v[r] for j < c over the team's rows: FP32 products
// summed 8 rows at a time, then FP64 (the FP32 form's reorthogonalization
// coefficients). Columns go in blocks of 16 to bound the accumulator registers.
template <int C>
__device__ void team_dot(const float* __restrict__ Q, int64_t L, int64_t ldq, int c, const float* __restrict__ v,
                         Team<C>& tm, Persist& ps) {
    constexpr int kJB = 16;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t lo = tm.lo(L), hi = tm.hi(L);
    for (int j0 = 0; j0 < c; j0 += kJB) {
        const float* Qb = Q + j0 * ldq;
        const int cb = c - j0 < kJB ? c - j0 : kJB;
        double acc[kJB];
        float part[kJB];
#pragma unroll
        for (int j = 0; j < kJB; ++j) {
            acc[j] = 0;
            part[j] = 0;
        }
        int cnt = 0;
        for (int64_t r = lo + threadIdx.x; r < hi; r += kBT) {
            const float vr = v[r];
#pragma unroll
            for (int j = 0; j < kJB; ++j)
                if (j < cb) part[j] = fmaf(Qb[r + j * ldq], vr, part[j]);
            if (++cnt == 8) {
#pragma unroll
                for (int j = 0; j < kJB; ++j) {
                    acc[j] += static_cast<double>(part[j]);
                    part[j] = 0;
                }
                cnt = 0;
            }
        }
#pragma unroll
        for (int j = 0; j < kJB; ++j) acc[j] += static_cast<double>(part[j]);
#pragma unroll
        for (int j = 0; j < kJB; ++j) {
            if (j < cb) {
                const double s = warp_sum(acc[j]);
                if (lane == 0) ps.red[warp * kWM + j0 + j] = s;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < c) {
        double s = 0;
#pragma unroll
        for (int w = 0; w < kBW; ++w) s += ps.red[w * kWM + threadIdx.x];
        ps.xred[tm.slot][threadIdx.x] = s;
    }
    tm.sync();
    if (threadIdx.x < c) {
        double s = 0;
        for (int r = 0; r < C; ++r) s += tm.peer(ps.xred[tm.slot], r)[threadIdx.x];
        ps.t[threadIdx.x] = s;
        ps.t32[threadIdx.x] = static_cast<float>(s);
    }
    tm.slot ^= 1;
    __syncthreads();
}

// Reorthogonalize v against Q[:, :c] (classical Gram-Schmidt, one pass as in
// lanczos.hpp:27-44) on the team's rows and return ||v|| in FP64.
template <int C>
__device__ double team_cgs(const float* __restrict__ Q, int64_t L, int64_t ldq, int c, float* __restrict__ v,
                           Team<C>& tm, Persist& ps) {
    if (c > 0) team_dot(Q, L, ldq, c, v, tm, ps);
    double sq = 0;
    const int64_t hi = tm.hi(L);
    for (int64_t r = tm.lo(L) + threadIdx.x; r < hi; r += kBT) {
        float s = 0;
        for (int j = 0; j < c; ++j) s = fmaf(Q[r + j * ldq], ps.t32[j], s);
        const float nv = v[r] - s;
        v[r] = nv;
        sq += static_cast<double>(nv) * static_cast<double>(nv);
    }
    return sqrt(team_sum(sq, tm, ps));
}

// v /= norm; qcol = v on the team's rows. Returns sum_r v[r] (the centring
// scalar of the next adjoint). Always ends with a team barrier, after which the
// whole normalized vector is visible to the team.
template <int C>
__device__ double team_normalize(float* __restrict__ v, int64_t L, double norm, float* __restrict__ qcol,
                                 Team<C>& tm, Persist& ps) {
    const float inv = static_cast<float>(1.0 / norm);
    double acc = 0;
    const int64_t hi = tm.hi(L);
    for (int64_t r = tm.lo(L) + threadIdx.x; r < hi; r += kBT) {
        const float x = v[r] * inv;
        v[r] = x;
        qcol[r] = x;
        acc += static_cast<double>(x);
    }
    return team_sum(acc, tm, ps);
}

// R[j][i] = M[j + i * w] for j < w, i < k (FP64 column-major -> FP32).
__device__ void load_rotation(const double* M, int w, int k, float* R) {
    for (int e = threadIdx.x; e < kWM * kWM; e += kBT) {
        const int j = e / kWM, i = e % kWM;
        R[e] = (j < w && i < k) ? static_cast<float>(M[j + i * w]) : 0.0f;
    }
}

// Q[:, :k] = Q[:, :w] R (in place, one row per thread) on the team's rows;
// Q[:, k] = fcol * finv.
template <int C>
__device__ void team_rotate(float* Q, int64_t L, int64_t ldq, int w, int k, const float* fcol, float finv,
                            const float* R, const Team<C>& tm) {
    const int64_t hi = tm.hi(L);
    for (int64_t r = tm.lo(L) + threadIdx.x; r < hi; r += kBT) {
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
            for (int i = 0; i < kWM; ++i) acc[i] = fmaf(rj, R[j * kWM + i], acc[i]);
        }
#pragma unroll
        for (int i = 0; i < kWM; ++i)
            if (i < k) Q[r + i * ldq] = acc[i];
        if (fcol) Q[r + static_cast<int64_t>(k) * ldq] = fcol[r] * finv;
    }
    __syncthreads();
}

// Column means and standard deviations over the team's feature rows of the
// adjoint CSR (pca.hpp:85-109): implicit zeros enter the variance
// analytically, and a zero-variance column keeps a scale of 1. One warp per
// feature.
template <int C>
__device__ void column_stats(const BatchProblem& P, bool center, bool scale, const Team<C>& tm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t m = P.m;
    const int64_t hi = tm.hi(P.n);
    for (int64_t f = tm.lo(P.n) + warp; f < hi; f += kBW) {
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
    tm.sync();
}

template <int C>
__device__ void solve_problem(const BatchProblem& P, const BatchParams& prm, BatchResult* result, Team<C>& tm,
                              Persist& ps, unsigned char* uni) {
    const int64_t m = P.m, n = P.n;
    const int w = prm.work, req = prm.number;
    const bool center = prm.center != 0, scale = prm.scale != 0;
    float* stage = reinterpret_cast<float*>(uni);
    double* G = reinterpret_cast<double*>(uni);
    double* Vj = G + w * w;
    double* BU = Vj + w * w;
    double* BV = BU + w * w;

    if (center || scale) column_stats(P, center, scale, tm);
    const float* cvec = center ? P.center : nullptr;
    const float* svec = scale ? P.scale : nullptr;

    // Start vector (compute.hpp:179-190), normalized in FP64.
    {
        double s = 0;
        for (int64_t c = tm.lo(n) + threadIdx.x; c < tm.hi(n); c += kBT) s += P.init[c] * P.init[c];
        const double nrm = sqrt(team_sum(s, tm, ps));
        for (int64_t c = tm.lo(n) + threadIdx.x; c < tm.hi(n); c += kBT)
            P.V[c] = static_cast<float>(P.init[c] / nrm);
    }
    for (int e = threadIdx.x; e < kWM * kWM; e += kBT) ps.B[e] = 0.0;
    for (int e = threadIdx.x; e < kWM; e += kBT) ps.prevS[e] = 0.0;
    __syncthreads();

    // multiply: y = A (x / s) - (c . (x / s)) - alpha q   (centered.hpp, scaled.hpp)
    auto multiply = [&](const float* x, float* y, float alpha, const float* q) {
        double b = 0;
        if (cvec) {
            for (int64_t c = tm.lo(n) + threadIdx.x; c < tm.hi(n); c += kBT) {
                const float xv = svec ? x[c] / svec[c] : x[c];
                b += static_cast<double>(xv) * static_cast<double>(cvec[c]);
            }
        }
        // The team sum doubles as the barrier that publishes x.
        b = team_sum(b, tm, ps);
        batch_spmv(P.mul, tm, x, svec, P.xs, stage, y, static_cast<float>(b), nullptr, nullptr, alpha, q);
    };
    // adjoint: out = (A^T y - (sum y) c) / s - alpha q; y was published by team_normalize.
    auto adjoint = [&](const float* y, float* out, double ysum, float alpha, const float* q) {
        batch_spmv(P.adj, tm, y, nullptr, nullptr, stage, out, cvec ? static_cast<float>(ysum) : 0.0f, cvec, svec,
                   alpha, q);
    };

    const double eps = prm.eps;
    int iter = 0, k = 0, status = 0, sweeps = 0;
    bool converged = false;
    int64_t steps = 0;
    for (; iter < prm.max_iter; ++iter) {
        // Lanczos bidiagonalization from column k (lanczos.hpp:54-143).
        multiply(P.V + k * P.ldv, P.Wn, 0.0f, nullptr);
        double S = team_cgs(P.W, m, P.ldw, k, P.Wn, tm, ps);
        if (S < eps) {
            status = 2;
            break;
        }
        double ysum = team_normalize(P.Wn, m, S, P.W + k * P.ldw, tm, ps);
        double R_F = 0;
        for (int j = k; j < w; ++j) {
            adjoint(P.Wn, P.F, ysum, static_cast<float>(S), P.V + j * P.ldv);
            R_F = team_cgs(P.V, n, P.ldv, j + 1, P.F, tm, ps);
            if (j + 1 < w) {
                if (R_F < eps) {
                    status = 2;
                    break;
                }
                team_normalize(P.F, n, R_F, P.V + (j + 1) * P.ldv, tm, ps);
                if (threadIdx.x == 0) {
                    ps.B[j + j * w] = S;
                    ps.B[j + (j + 1) * w] = R_F;
                }
                multiply(P.V + (j + 1) * P.ldv, P.Wn, static_cast<float>(R_F), P.W + j * P.ldw);
                S = team_cgs(P.W, m, P.ldw, j + 1, P.Wn, tm, ps);
                if (S < eps) {
                    status = 2;
                    break;
                }
                ysum = team_normalize(P.Wn, m, S, P.W + (j + 1) * P.ldw, tm, ps);
            } else if (threadIdx.x == 0) {
                ps.B[j + j * w] = S;
            }
        }
        if (status) break;
        steps += w - k;
        __syncthreads();

        // Restart (compute.hpp:225-293), identical on every CTA of the team:
        // SVD of B, convergence test, update_k.
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
        load_rotation(BV, w, kn, ps.RV);
        load_rotation(BU, w, kn, ps.RW);
        __syncthreads();
        team_rotate(P.V, n, P.ldv, w, kn, P.F, static_cast<float>(1.0 / R_F), ps.RV, tm);
        team_rotate(P.W, m, P.ldw, w, kn, nullptr, 0.0f, ps.RW, tm);
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
        const int64_t m0 = tm.lo(m), mc = tm.hi(m) - m0;
        for (int64_t e = threadIdx.x; e < mc * req; e += kBT) {
            const int64_t r = m0 + e % mc;
            const int i = static_cast<int>(e / mc);
            double s = 0;
            for (int j = 0; j < w; ++j) s += static_cast<double>(P.W[r + j * P.ldw]) * BU[j + i * w];
            P.scores[r + i * m] = s * ps.BS[i];
        }
        const int64_t n0 = tm.lo(n), nc = tm.hi(n) - n0;
        for (int64_t e = threadIdx.x; e < nc * req; e += kBT) {
            const int64_t r = n0 + e % nc;
            const int i = static_cast<int>(e / nc);
            double s = 0;
            for (int j = 0; j < w; ++j) s += static_cast<double>(P.V[r + j * P.ldv]) * BV[j + i * w];
            P.rotation[r + i * n] = s;
        }
        if (tm.rank == 0)
            for (int i = threadIdx.x; i < req; i += kBT)
                P.variances[i] = n > 1 ? ps.BS[i] * ps.BS[i] / static_cast<double>(m - 1) : ps.BS[i];
    }
    if (tm.rank == 0 && threadIdx.x == 0) {
        result->status = status;
        result->converged = converged ? 1 : 0;
        result->iterations = converged ? iter + 1 : iter;
        result->svd_sweeps = sweeps;
        result->steps = steps;
    }
    // The team leaves the problem together (the workspace is reused next).
    tm.sync();
}

// The team's leader takes work from the queue: while the index is below
// n_joint (the largest matrices) the team solves one matrix together;
// afterwards it takes C matrices at a time and every CTA solves its own alone.
template <int C>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(kBT, 1)
    batch_pca_kernel(const BatchProblem* __restrict__ probs, const int32_t* __restrict__ order, int32_t count,
                     int32_t n_joint, BatchParams prm, BatchResult* results, uint32_t* queue) {
    extern __shared__ __align__(128) unsigned char smem[];
    Persist& ps = *reinterpret_cast<Persist*>(smem);
    unsigned char* uni = smem + kPersistBytes;
    Team<C> tm;
    if constexpr (C > 1) tm.rank = static_cast<int>(cg::this_cluster().block_rank());
    while (true) {
        if (tm.rank == 0 && threadIdx.x == 0) {
            const int i = static_cast<int>(atomicAdd(queue, 1u));
            ps.assign[0] = i;
            ps.joint = (C == 1 || i < n_joint) ? 1 : 0;
            if (!ps.joint) {
                const int j = i < count ? static_cast<int>(atomicAdd(queue, static_cast<unsigned>(C - 1))) : count;
                for (int r = 1; r < C; ++r) ps.assign[r] = j < count ? j + r - 1 : count;
            }
        }
        tm.sync();
        const int i0 = *tm.peer(&ps.assign[0], 0);
        const int joint = *tm.peer(&ps.joint, 0);
        const int mine = joint ? i0 : *tm.peer(&ps.assign[tm.rank], 0);
        tm.sync();
        if (i0 >= count) break;
        if (joint) {
            const int p = order[i0];
            const uint64_t t0 = global_ns();
            solve_problem<C>(probs[p], prm, results + p, tm, ps, uni);
            if (tm.rank == 0 && threadIdx.x == 0) {
                results[p].t_start = t0;
                results[p].t_end = global_ns();
            }
        } else if (mine < count) {
            const int p = order[mine];
            const uint64_t t0 = global_ns();
            Team<1> solo;
            solve_problem<1>(probs[p], prm, results + p, solo, ps, uni);
            if (threadIdx.x == 0) {
                results[p].t_start = t0;
                results[p].t_end = global_ns();
            }
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
    Team<1> tm;
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
            batch_spmv(d, tm, x, nullptr, nullptr, stage, y, 0.0f, nullptr, nullptr, 0.0f, nullptr);
            const uint64_t t1 = clock64();
            best = t1 - t0 < best ? t1 - t0 : best;
        }
        if (threadIdx.x == 0) cycles_out[order[i]] = best;
        __syncthreads();
    }
}

template <int C>
cudaError_t configure_one(size_t bytes) {
    return cudaFuncSetAttribute(batch_pca_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(bytes));
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
    cudaError_t e = configure_one<1>(want);
    if (e == cudaSuccess) e = configure_one<2>(want);
    if (e == cudaSuccess) e = configure_one<4>(want);
    if (e == cudaSuccess) e = configure_one<8>(want);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(batch_spmv_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(want));
    return e;
}

int batch_max_teams(int team, size_t smem) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(team), 1, 1);
    cfg.blockDim = dim3(kBT, 1, 1);
    cfg.dynamicSmemBytes = smem;
    int n = 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (team) {
        case 1: {
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_pca_kernel<1>, kBT, smem);
            int dev = 0, sms = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            n = per_sm * sms;
            break;
        }
        case 2: e = cudaOccupancyMaxActiveClusters(&n, batch_pca_kernel<2>, &cfg); break;
        case 4: e = cudaOccupancyMaxActiveClusters(&n, batch_pca_kernel<4>, &cfg); break;
        case 8: e = cudaOccupancyMaxActiveClusters(&n, batch_pca_kernel<8>, &cfg); break;
        default: break;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void launch_batch_pca(int team, const BatchProblem* probs, const int32_t* order, int32_t count, int32_t n_joint,
                      const BatchParams& prm, BatchResult* results, uint32_t* queue, int teams, size_t smem,
                      cudaStream_t stream) {
    const int grid = teams * team;
    switch (team) {
        case 2:
            batch_pca_kernel<2><<<grid, kBT, smem, stream>>>(probs, order, count, n_joint, prm, results, queue);
            break;
        case 4:
            batch_pca_kernel<4><<<grid, kBT, smem, stream>>>(probs, order, count, n_joint, prm, results, queue);
            break;
        case 8:
            batch_pca_kernel<8><<<grid, kBT, smem, stream>>>(probs, order, count, n_joint, prm, results, queue);
            break;
        default:
            batch_pca_kernel<1><<<grid, kBT, smem, stream>>>(probs, order, count, n_joint, prm, results, queue);
            break;
    }
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
