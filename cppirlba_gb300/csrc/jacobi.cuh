// One-sided Jacobi SVD building blocks shared by the restart kernels and the
// batched solver (device code, one CTA).
//
// Method: one-sided Jacobi (Hestenes 1958; Demmel & Veselic 1992) in FP64 with
// the parallel round-robin ("circle") pair ordering: one warp rotates one
// disjoint column pair per round. Rotations use Rutishauser's formulas; a pair
// is skipped when |g_p . g_q| <= m eps ||g_p|| ||g_q|| (m = rows, the rounding
// floor of the dot product, so sweeps terminate). Singular values are the final
// column norms sorted decreasingly (ties keep column order); U = G / sigma, and
// columns of U with a zero singular value are completed to an orthonormal basis
// by Gram-Schmidt against unit vectors. Signs are canonical: the
// largest-magnitude entry of each V column is positive.
#pragma once

#include "common.cuh"

namespace irlba_gb300 {
namespace jacobi {

constexpr int kMaxSweeps = 60;

static __device__ __forceinline__ int circle_partner_a(int round, int slot, int n2) {
    if (slot == 0) return round;
    return (round + slot) % (n2 - 1);
}
static __device__ __forceinline__ int circle_partner_b(int round, int slot, int n2) {
    if (slot == 0) return n2 - 1;
    return (round - slot + n2 - 1) % (n2 - 1);
}

// One-sided Jacobi on G (m x n, column-major, ld m) accumulating V (n x n, ld n).
// Whole CTA participates. Each round runs in three phases separated by CTA
// barriers: (1) one warp per column pair forms the dot product g_pq; (2) one
// thread per pair derives the rotation from g_pq and the column norms, so the
// long FP64 divide/square-root sequences run once per 32 pairs instead of
// once per warp; (3) one warp per pair rotates the two columns of G and V.
// pairs: >= 3 * ((n + 1) / 2) doubles of scratch (shared memory).
// Returns the number of sweeps in *sweeps.
static __device__ void jacobi_sweeps(double* G, int64_t m, int n, double* V, int* sweeps, int* not_converged,
                                     int* rotated_flag, double* nrm, double* pairs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n2 = n + (n & 1);
    const int half = n2 / 2;
    double* pg = pairs;
    double* pc = pairs + half;
    double* ps = pairs + 2 * half;
    const double eps = 2.220446049250313e-16;
    const double thresh = eps * static_cast<double>(m);
    int sweep = 0;
    for (; sweep < kMaxSweeps; ++sweep) {
        // Squared column norms, recomputed each sweep and updated per rotation
        // (Rutishauser: ||g_p'||^2 = a - t g, ||g_q'||^2 = b + t g).
        for (int j = warp; j < n; j += nw) {
            double a = 0;
            for (int64_t i = lane; i < m; i += 32) a += G[j * m + i] * G[j * m + i];
            a = warp_sum(a);
            if (lane == 0) nrm[j] = a;
        }
        if (threadIdx.x == 0) *rotated_flag = 0;
        __syncthreads();
        for (int round = 0; round < n2 - 1; ++round) {
            for (int slot = warp; slot < half; slot += nw) {
                int p = circle_partner_a(round, slot, n2);
                int q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                if (q >= n) continue;
                const double* gp = G + p * m;
                const double* gq = G + q * m;
                double g = 0;
                for (int64_t i = lane; i < m; i += 32) g += gp[i] * gq[i];
                g = warp_sum(g);
                if (lane == 0) pg[slot] = g;
            }
            __syncthreads();
            // Rotation parameters (c = 0 marks a pair left alone).
            for (int slot = threadIdx.x; slot < half; slot += blockDim.x) {
                int p = circle_partner_a(round, slot, n2);
                int q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                double c = 0, sn = 0;
                if (q < n) {
                    const double g = pg[slot];
                    const double a = nrm[p], b = nrm[q];
                    if (!(g == 0.0 || fabs(g) <= thresh * sqrt(a * b))) {
                        const double zeta = (b - a) / (2.0 * g);
                        const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                        c = 1.0 / sqrt(1.0 + t * t);
                        sn = c * t;
                        nrm[p] = a - t * g;
                        nrm[q] = b + t * g;
                        *rotated_flag = 1;
                    }
                }
                pc[slot] = c;
                ps[slot] = sn;
            }
            __syncthreads();
            for (int slot = warp; slot < half; slot += nw) {
                const double c = pc[slot];
                if (c == 0.0) continue;
                const double sn = ps[slot];
                int p = circle_partner_a(round, slot, n2);
                int q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                double* gp = G + p * m;
                double* gq = G + q * m;
                for (int64_t i = lane; i < m; i += 32) {
                    const double x = gp[i], y = gq[i];
                    gp[i] = c * x - sn * y;
                    gq[i] = sn * x + c * y;
                }
                double* vp = V + p * n;
                double* vq = V + q * n;
                for (int i = lane; i < n; i += 32) {
                    const double x = vp[i], y = vq[i];
                    vp[i] = c * x - sn * y;
                    vq[i] = sn * x + c * y;
                }
            }
            __syncthreads();
        }
        const int any = *rotated_flag;
        __syncthreads();
        if (!any) break;
    }
    if (threadIdx.x == 0) {
        *sweeps = sweep + 1;
        *not_converged = (sweep >= kMaxSweeps);
    }
    __syncthreads();
}

// From converged G, V: S sorted descending, U (m x n), Vout (n x n, ld ldv).
// norms: n doubles of scratch, order: n ints of scratch.
static __device__ void finish_svd(const double* G, int64_t m, int n, const double* V, double* S, double* U, int64_t ldu,
                           double* Vout, int64_t ldv, double* norms, int* order) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < n; j += nw) {
        double a = 0;
        for (int64_t i = lane; i < m; i += 32) a += G[j * m + i] * G[j * m + i];
        a = warp_sum(a);
        if (lane == 0) norms[j] = sqrt(a);
    }
    __syncthreads();
    // Rank of each column: number of columns with a larger norm (ties by index).
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double sj = norms[j];
        int rank = 0;
        for (int i = 0; i < n; ++i) {
            const double si = norms[i];
            if (si > sj || (si == sj && i < j)) ++rank;
        }
        order[rank] = j;
    }
    __syncthreads();
    double smax = 0;
    if (n > 0) smax = norms[order[0]];
    const double zero_tol = smax * 2.220446049250313e-16 * static_cast<double>(m > n ? m : n);
    for (int jj = warp; jj < n; jj += nw) {
        const int j = order[jj];
        const double sj = norms[j];
        if (lane == 0) S[jj] = sj;
        for (int i = lane; i < n; i += 32) Vout[jj * ldv + i] = V[j * n + i];
        if (sj > zero_tol) {
            const double inv = 1.0 / sj;
            for (int64_t i = lane; i < m; i += 32) U[jj * ldu + i] = G[j * m + i] * inv;
        } else {
            if (lane == 0) S[jj] = sj > 0 ? sj : 0.0;
            for (int64_t i = lane; i < m; i += 32) U[jj * ldu + i] = 0.0;
        }
    }
    __syncthreads();
    // Orthonormal completion for zero singular values (warp 0, sequential over
    // the missing columns).
    int nonzero = 0;
    for (int jj = 0; jj < n; ++jj)
        if (norms[order[jj]] > zero_tol) ++nonzero;
    if (warp == 0) {
        int64_t e = 0;
        for (int jj = nonzero; jj < n; ++jj) {
            double* u = U + jj * ldu;
            while (e < m) {
                for (int64_t i = lane; i < m; i += 32) u[i] = (i == e) ? 1.0 : 0.0;
                ++e;
                __syncwarp();
                for (int pass = 0; pass < 2; ++pass) {
                    for (int kk = 0; kk < jj; ++kk) {
                        const double* uk = U + kk * ldu;
                        double d = 0;
                        for (int64_t i = lane; i < m; i += 32) d += uk[i] * u[i];
                        d = warp_sum(d);
                        for (int64_t i = lane; i < m; i += 32) u[i] -= d * uk[i];
                        __syncwarp();
                    }
                }
                double nn = 0;
                for (int64_t i = lane; i < m; i += 32) nn += u[i] * u[i];
                nn = sqrt(warp_sum(nn));
                if (nn > 0.5) {
                    for (int64_t i = lane; i < m; i += 32) u[i] /= nn;
                    __syncwarp();
                    break;
                }
            }
        }
    }
    __syncthreads();
    // Canonical signs: the largest-magnitude entry of each V column (first one
    // on ties) is made positive and the U column follows, the convention the
    // oracle uses too.
    for (int jj = warp; jj < n; jj += nw) {
        double* v = Vout + jj * ldv;
        double best = -1.0;
        int arg = n;
        for (int i = lane; i < n; i += 32) {
            const double a = fabs(v[i]);
            if (a > best) {
                best = a;
                arg = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
            if (ob > best || (ob == best && oa < arg)) {
                best = ob;
                arg = oa;
            }
        }
        const bool flip = (arg < n) && v[arg] < 0;
        __syncwarp();
        if (flip) {
            for (int i = lane; i < n; i += 32) v[i] = -v[i];
            for (int64_t i = lane; i < m; i += 32) U[jj * ldu + i] = -U[jj * ldu + i];
        }
    }
    __syncthreads();
}

// update_k, compute.hpp:78-111.
static __device__ int update_k_dev(int k, int requested, int n_converged, int work) {
    if (work <= 3) return 1;
    const int limit = work - 3;
    auto less = [&](int val) { return val < requested || (val - requested) < n_converged; };
    if (less(k)) {
        if (less(limit)) return limit;
        const int out = requested + n_converged;
        return out > 1 ? out : 1;
    }
    const int out = k < limit ? k : limit;
    return out > 1 ? out : 1;
}


}  // namespace jacobi
}  // namespace irlba_gb300
