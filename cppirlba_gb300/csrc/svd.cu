// The restart step of the IRLBA loop on the device (CppIrlba compute.hpp:225-293)
// and the small dense SVD it needs.
//
// The SVD stands in for Eigen::JacobiSVD (compute.hpp:27-28): a one-sided
// Jacobi method (Hestenes 1958; Demmel & Veselic 1992) on the columns of B in
// FP64, with the parallel round-robin ("circle") pair ordering so that one
// warp rotates one disjoint column pair per round inside a single CTA.
// Rotations use Rutishauser's formulas; a pair is skipped when
// |g_p . g_q| <= m eps ||g_p|| ||g_q|| (m = rows; the rounding floor of the
// dot product, so sweeps terminate). Singular values are the final column
// norms, sorted decreasingly (ties keep column order); U = G / sigma, and
// columns of U with a zero singular value are completed to an orthonormal basis
// by Gram-Schmidt against unit vectors.

#include "kernels.cuh"

namespace irlba_gb300 {

namespace {

constexpr int kSvdThreads = 1024;
constexpr int kMaxSweeps = 60;

__device__ __forceinline__ int circle_partner_a(int round, int slot, int n2) {
    if (slot == 0) return round;
    return (round + slot) % (n2 - 1);
}
__device__ __forceinline__ int circle_partner_b(int round, int slot, int n2) {
    if (slot == 0) return n2 - 1;
    return (round - slot + n2 - 1) % (n2 - 1);
}

// One-sided Jacobi on G (m x n, column-major, ld m) accumulating V (n x n, ld n).
// Whole CTA participates. Returns the number of sweeps in *sweeps.
__device__ void jacobi_sweeps(double* G, int64_t m, int n, double* V, int* sweeps, int* not_converged,
                              int* rotated_flag) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n2 = n + (n & 1);
    const double eps = 2.220446049250313e-16;
    int sweep = 0;
    for (; sweep < kMaxSweeps; ++sweep) {
        if (threadIdx.x == 0) *rotated_flag = 0;
        __syncthreads();
        for (int round = 0; round < n2 - 1; ++round) {
            for (int slot = warp; slot < n2 / 2; slot += nw) {
                int p = circle_partner_a(round, slot, n2);
                int q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                if (q >= n) continue;
                double* gp = G + p * m;
                double* gq = G + q * m;
                double a = 0, b = 0, g = 0;
                for (int64_t i = lane; i < m; i += 32) {
                    const double x = gp[i], y = gq[i];
                    a += x * x;
                    b += y * y;
                    g += x * y;
                }
                a = warp_sum(a);
                b = warp_sum(b);
                g = warp_sum(g);
                if (g == 0.0 || fabs(g) <= eps * static_cast<double>(m) * sqrt(a * b)) continue;
                const double zeta = (b - a) / (2.0 * g);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t);
                const double s = c * t;
                for (int64_t i = lane; i < m; i += 32) {
                    const double x = gp[i], y = gq[i];
                    gp[i] = c * x - s * y;
                    gq[i] = s * x + c * y;
                }
                double* vp = V + p * n;
                double* vq = V + q * n;
                for (int i = lane; i < n; i += 32) {
                    const double x = vp[i], y = vq[i];
                    vp[i] = c * x - s * y;
                    vq[i] = s * x + c * y;
                }
                if (lane == 0) *rotated_flag = 1;
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
__device__ void finish_svd(const double* G, int64_t m, int n, const double* V, double* S, double* U, int64_t ldu,
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
__device__ int update_k_dev(int k, int requested, int n_converged, int work) {
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

__global__ void __launch_bounds__(kSvdThreads) restart_kernel(RestartArgs a, int use_smem) {
    extern __shared__ __align__(16) double sm[];
    __shared__ double norms[1024];
    __shared__ int order[1024];
    __shared__ int rotated;
    __shared__ int sweeps, notconv;
    Ctrl* ctrl = a.ctrl;
    if (ctrl->abort) return;
    const int n = a.work;
    double* G = use_smem ? sm : a.scratch;
    double* V = use_smem ? sm + n * n : a.scratch + n * n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        G[e] = a.B[e];
        V[e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
    }
    __syncthreads();
    jacobi_sweeps(G, n, n, V, &sweeps, &notconv, &rotated);
    finish_svd(G, n, n, V, a.BS, a.BU, n, a.BV, n, norms, order);

    // Convergence test, compute.hpp:231-264.
    if (threadIdx.x == 0) {
        ctrl->svd_sweeps = sweeps;
        ctrl->svd_not_converged = notconv;
        int converged = 0;
        int n_conv = 0;
        if (a.B[(n - 1) + static_cast<int64_t>(n - 1) * n] == 0.0) {
            converged = 1;
        } else {
            const double R_F = ctrl->norm_F;
            for (int j = 0; j < n; ++j) a.res[j] = R_F * a.BU[(n - 1) + static_cast<int64_t>(j) * n];
            if (a.iter > 0) {
                double smax = a.BS[0];
                for (int j = 1; j < n; ++j) smax = a.BS[j] > smax ? a.BS[j] : smax;
                const double threshold = smax * a.tol;
                for (int j = 0; j < n; ++j) {
                    if (fabs(a.res[j]) <= threshold) {
                        const double ratio = fabs(a.BS[j] - a.prevS[j]) / a.BS[j];
                        if (ratio <= a.svtol) ++n_conv;
                    }
                }
                if (n_conv >= a.requested) converged = 1;
            }
        }
        ctrl->converged = converged;
        ctrl->n_converged = n_conv;
        if (!converged) {
            for (int j = 0; j < n; ++j) a.prevS[j] = a.BS[j];
            ctrl->k_next = update_k_dev(a.k, a.requested, n_conv, n);
        } else {
            ctrl->k_next = a.k;
        }
    }
    __syncthreads();
    // B rebuilt for the next run, compute.hpp:282-293.
    if (!ctrl->converged) {
        const int kn = ctrl->k_next;
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) a.B[e] = 0.0;
        __syncthreads();
        for (int l = threadIdx.x; l < kn; l += blockDim.x) {
            a.B[l + static_cast<int64_t>(l) * n] = a.BS[l];
            a.B[l + static_cast<int64_t>(kn) * n] = a.res[l];
        }
    }
}

__global__ void __launch_bounds__(kSvdThreads) dense_svd_kernel(const double* A, int64_t m, int n, double* U, double* S,
                                                                 double* V, double* scratch, Ctrl* ctrl) {
    __shared__ double norms[1024];
    __shared__ int order[1024];
    __shared__ int rotated;
    __shared__ int sweeps, notconv;
    double* G = scratch;
    double* VV = scratch + m * n;
    for (int64_t e = threadIdx.x; e < m * n; e += blockDim.x) G[e] = A[e];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) VV[e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
    __syncthreads();
    jacobi_sweeps(G, m, n, VV, &sweeps, &notconv, &rotated);
    finish_svd(G, m, n, VV, S, U, m, V, n, norms, order);
    if (threadIdx.x == 0 && ctrl) {
        ctrl->svd_sweeps = sweeps;
        ctrl->svd_not_converged = notconv;
    }
}

}  // namespace

size_t restart_smem_bytes(int work) { return sizeof(double) * 2 * static_cast<size_t>(work) * work; }

cudaError_t restart_configure(size_t max_smem) {
    return cudaFuncSetAttribute(restart_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
}

void launch_restart(const RestartArgs& a, cudaStream_t stream, size_t max_smem) {
    const size_t need = restart_smem_bytes(a.work);
    const int use_smem = need <= max_smem ? 1 : 0;
    restart_kernel<<<1, kSvdThreads, use_smem ? need : 0, stream>>>(a, use_smem); count_launch();
}

void launch_dense_svd(const double* A, int64_t m, int64_t n, double* U, double* S, double* V, double* scratch,
                      Ctrl* ctrl, cudaStream_t stream) {
    dense_svd_kernel<<<1, kSvdThreads, 0, stream>>>(A, m, static_cast<int>(n), U, S, V, scratch, ctrl); count_launch();
}

}  // namespace irlba_gb300
