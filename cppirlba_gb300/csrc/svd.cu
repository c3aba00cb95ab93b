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

#include <cooperative_groups.h>

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
                              int* rotated_flag, double* nrm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n2 = n + (n & 1);
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
                double g = 0;
                for (int64_t i = lane; i < m; i += 32) g += gp[i] * gq[i];
                g = warp_sum(g);
                const double a = nrm[p], b = nrm[q];
                if (g == 0.0 || fabs(g) <= thresh * sqrt(a * b)) continue;
                // Rotation parameters once per pair (lane 0), then broadcast:
                // FP64 sqrt and division are long multi-instruction sequences.
                double c = 0, s = 0, t = 0;
                if (lane == 0) {
                    const double zeta = (b - a) / (2.0 * g);
                    t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                    c = 1.0 / sqrt(1.0 + t * t);
                    s = c * t;
                    nrm[p] = a - t * g;
                    nrm[q] = b + t * g;
                }
                c = __shfl_sync(0xffffffffu, c, 0);
                s = __shfl_sync(0xffffffffu, s, 0);
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

// Convergence test (compute.hpp:231-264), update_k (compute.hpp:267) and the
// rebuild of B (compute.hpp:282-293), by one CTA after the SVD of B is in
// a.BS, a.BU, a.BV.
__device__ void restart_tail(const RestartArgs& a, int sweeps, int notconv) {
    Ctrl* ctrl = a.ctrl;
    const int n = a.work;
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

// Restart step on one CTA (used when the cluster form does not apply).
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
    jacobi_sweeps(G, n, n, V, &sweeps, &notconv, &rotated, norms);
    finish_svd(G, n, n, V, a.BS, a.BU, n, a.BV, n, norms, order);
    restart_tail(a, sweeps, notconv);
}

// ---------------------------------------------------------------------------
// Restart step on a thread-block cluster. GB300 retires about two FP64 lane
// operations per clock per SM, so one SM runs a 57 x 57 Jacobi sweep in about
// half a millisecond. The cluster keeps G and V in CTA 0's shared memory and
// gives each of its warps one column pair per round through distributed shared
// memory; rounds are separated by cluster barriers. The arithmetic is the same
// as the single-CTA form (same ordering, same formulas).
// ---------------------------------------------------------------------------
constexpr int kClusterCTAs = 8;
constexpr int kClusterThreads = 128;
constexpr int kClusterMaxRows = 128;  // per-lane register cache: 4 rows

__global__ void __cluster_dims__(kClusterCTAs, 1, 1) __launch_bounds__(kClusterThreads)
    restart_cluster_kernel(RestartArgs a) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) double sm[];
    __shared__ double norms_local[kClusterMaxRows];
    __shared__ int order[kClusterMaxRows];
    __shared__ int rotated_local;
    const unsigned rank = cl.block_rank();
    const int n = a.work;
    const int nn = n * n;
    // The abort flag does not change while the kernel runs: every CTA takes the
    // same branch, so no CTA waits at a barrier the others skip.
    if (a.ctrl->abort) return;
    double* G = cl.map_shared_rank(sm, 0);
    double* V = G + nn;
    double* nrm = cl.map_shared_rank(norms_local, 0);
    int* rotated = cl.map_shared_rank(&rotated_local, 0);
    if (rank == 0) {
        for (int e = threadIdx.x; e < nn; e += blockDim.x) {
            sm[e] = a.B[e];
            sm[nn + e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
        }
    }
    cl.sync();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int gw = static_cast<int>(rank) * nw + warp;
    const int gnw = static_cast<int>(cl.num_blocks()) * nw;
    const int n2 = n + (n & 1);
    const double thresh = 2.220446049250313e-16 * static_cast<double>(n);
    int sweep = 0;
    for (; sweep < kMaxSweeps; ++sweep) {
        for (int j = gw; j < n; j += gnw) {
            double s = 0;
            for (int i = lane; i < n; i += 32) {
                const double x = G[j * n + i];
                s += x * x;
            }
            s = warp_sum(s);
            if (lane == 0) nrm[j] = s;
        }
        if (rank == 0 && threadIdx.x == 0) *rotated = 0;
        cl.sync();
        for (int round = 0; round < n2 - 1; ++round) {
            for (int slot = gw; slot < n2 / 2; slot += gnw) {
                int p = circle_partner_a(round, slot, n2);
                int q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                if (q >= n) continue;
                double* gp = G + p * n;
                double* gq = G + q * n;
                double xp[kClusterMaxRows / 32], xq[kClusterMaxRows / 32];
                double g = 0;
#pragma unroll
                for (int u = 0; u < kClusterMaxRows / 32; ++u) {
                    const int i = lane + 32 * u;
                    xp[u] = i < n ? gp[i] : 0.0;
                    xq[u] = i < n ? gq[i] : 0.0;
                    g += xp[u] * xq[u];
                }
                g = warp_sum(g);
                const double av = nrm[p], bv = nrm[q];
                if (g == 0.0 || fabs(g) <= thresh * sqrt(av * bv)) continue;
                double c = 0, s = 0;
                if (lane == 0) {
                    const double zeta = (bv - av) / (2.0 * g);
                    const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                    c = 1.0 / sqrt(1.0 + t * t);
                    s = c * t;
                    nrm[p] = av - t * g;
                    nrm[q] = bv + t * g;
                    *rotated = 1;
                }
                c = __shfl_sync(0xffffffffu, c, 0);
                s = __shfl_sync(0xffffffffu, s, 0);
                double* vp = V + p * n;
                double* vq = V + q * n;
#pragma unroll
                for (int u = 0; u < kClusterMaxRows / 32; ++u) {
                    const int i = lane + 32 * u;
                    if (i < n) {
                        gp[i] = c * xp[u] - s * xq[u];
                        gq[i] = s * xp[u] + c * xq[u];
                        const double y = vp[i], z = vq[i];
                        vp[i] = c * y - s * z;
                        vq[i] = s * y + c * z;
                    }
                }
            }
            cl.sync();
        }
        const int any = *rotated;
        cl.sync();
        if (!any) break;
    }
    // CTA 0 finishes; the others stop touching its shared memory after the
    // last barrier above and may exit.
    if (rank != 0) return;
    finish_svd(sm, n, n, sm + nn, a.BS, a.BU, n, a.BV, n, norms_local, order);
    restart_tail(a, sweep + 1, sweep >= kMaxSweeps ? 1 : 0);
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
    jacobi_sweeps(G, m, n, VV, &sweeps, &notconv, &rotated, norms);
    finish_svd(G, m, n, VV, S, U, m, V, n, norms, order);
    if (threadIdx.x == 0 && ctrl) {
        ctrl->svd_sweeps = sweeps;
        ctrl->svd_not_converged = notconv;
    }
}

}  // namespace

size_t restart_smem_bytes(int work) { return 2 * sizeof(double) * static_cast<size_t>(work) * work; }

// Dynamic shared memory available to the restart kernel: the per-block opt-in
// limit minus the kernel's own static shared memory.
static size_t g_restart_max_dynamic = 0;

static size_t g_restart_cluster_max_dynamic = 0;

template <typename K>
static cudaError_t allow_dynamic_smem(K kernel, size_t smem_optin, size_t* avail_out) {
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, kernel);
    if (e != cudaSuccess) return e;
    const size_t avail = smem_optin > attr.sharedSizeBytes ? smem_optin - attr.sharedSizeBytes : 0;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(avail));
    if (e == cudaSuccess) *avail_out = avail;
    return e;
}

cudaError_t restart_configure(size_t smem_optin) {
    cudaError_t e = allow_dynamic_smem(restart_kernel, smem_optin, &g_restart_max_dynamic);
    if (e == cudaSuccess) e = allow_dynamic_smem(restart_cluster_kernel, smem_optin, &g_restart_cluster_max_dynamic);
    return e;
}

void launch_restart(const RestartArgs& a, cudaStream_t stream, size_t /*max_smem*/) {
    const size_t need = restart_smem_bytes(a.work);
    if (a.work <= kClusterMaxRows && need <= g_restart_cluster_max_dynamic) {
        restart_cluster_kernel<<<kClusterCTAs, kClusterThreads, need, stream>>>(a);
        count_launch();
        return;
    }
    const int use_smem = need <= g_restart_max_dynamic ? 1 : 0;
    restart_kernel<<<1, kSvdThreads, use_smem ? need : 0, stream>>>(a, use_smem); count_launch();
}

void launch_dense_svd(const double* A, int64_t m, int64_t n, double* U, double* S, double* V, double* scratch,
                      Ctrl* ctrl, cudaStream_t stream) {
    dense_svd_kernel<<<1, kSvdThreads, 0, stream>>>(A, m, static_cast<int>(n), U, S, V, scratch, ctrl); count_launch();
}

}  // namespace irlba_gb300
