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

#include "jacobi.cuh"
#include "kernels.cuh"

namespace irlba_gb300 {

namespace {

constexpr int kSvdThreads = 1024;
constexpr int kMaxSweeps = jacobi::kMaxSweeps;
using jacobi::circle_partner_a;
using jacobi::circle_partner_b;
using jacobi::jacobi_sweeps;
using jacobi::finish_svd;
using jacobi::update_k_dev;

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
    __shared__ double pairs[3 * 64];
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
    jacobi_sweeps(G, n, n, V, &sweeps, &notconv, &rotated, norms, pairs);
    finish_svd(G, n, n, V, a.BS, a.BU, n, a.BV, n, norms, order);
    restart_tail(a, sweeps, notconv);
}

// ---------------------------------------------------------------------------
// Restart step on a thread-block cluster. GB300 retires about two FP64 lane
// operations per clock per SM, so one SM runs a 57 x 57 Jacobi sweep in about
// half a millisecond. The cluster keeps G and V in CTA 0's shared memory and
// gives each of its warps one column pair per round through distributed shared
// memory; rounds are separated by cluster barriers. Within a CTA the rotation
// parameters of its warps' pairs are derived by one thread each, in parallel
// lanes. The arithmetic is the same as the single-CTA form (same ordering,
// same formulas).
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
    __shared__ double pair_g[kClusterThreads / 32], pair_c[kClusterThreads / 32], pair_s[kClusterThreads / 32];
    __shared__ int pair_p[kClusterThreads / 32], pair_q[kClusterThreads / 32];
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
            // Slots are taken gnw at a time so every thread runs the same
            // number of phases. Phase 1: each warp caches its two columns and
            // forms g; phase 2: one thread per local warp derives the rotation
            // (the FP64 divides and square roots run in parallel lanes of one
            // warp, not once per warp); phase 3: the warps rotate.
            for (int base = 0; base < n2 / 2; base += gnw) {
                const int slot = base + gw;
                int p = 0, q = n;
                if (slot < n2 / 2) {
                    p = circle_partner_a(round, slot, n2);
                    q = circle_partner_b(round, slot, n2);
                    if (p > q) {
                        const int tmp = p;
                        p = q;
                        q = tmp;
                    }
                }
                const bool live = q < n;
                double* gp = G + p * n;
                double* gq = G + q * n;
                double xp[kClusterMaxRows / 32], xq[kClusterMaxRows / 32];
                if (live) {
                    double g = 0;
#pragma unroll
                    for (int u = 0; u < kClusterMaxRows / 32; ++u) {
                        const int i = lane + 32 * u;
                        xp[u] = i < n ? gp[i] : 0.0;
                        xq[u] = i < n ? gq[i] : 0.0;
                        g += xp[u] * xq[u];
                    }
                    g = warp_sum(g);
                    if (lane == 0) {
                        pair_g[warp] = g;
                        pair_p[warp] = p;
                        pair_q[warp] = q;
                    }
                } else if (lane == 0) {
                    pair_q[warp] = n;
                }
                __syncthreads();
                if (threadIdx.x < nw) {
                    const int t = threadIdx.x;
                    double c = 0, sn = 0;
                    if (pair_q[t] < n) {
                        const int pp = pair_p[t], qq = pair_q[t];
                        const double g = pair_g[t];
                        const double av = nrm[pp], bv = nrm[qq];
                        if (!(g == 0.0 || fabs(g) <= thresh * sqrt(av * bv))) {
                            const double zeta = (bv - av) / (2.0 * g);
                            const double tt = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                            c = 1.0 / sqrt(1.0 + tt * tt);
                            sn = c * tt;
                            nrm[pp] = av - tt * g;
                            nrm[qq] = bv + tt * g;
                            *rotated = 1;
                        }
                    }
                    pair_c[t] = c;
                    pair_s[t] = sn;
                }
                __syncthreads();
                const double c = pair_c[warp], sn = pair_s[warp];
                if (live && c != 0.0) {
                    double* vp = V + p * n;
                    double* vq = V + q * n;
#pragma unroll
                    for (int u = 0; u < kClusterMaxRows / 32; ++u) {
                        const int i = lane + 32 * u;
                        if (i < n) {
                            gp[i] = c * xp[u] - sn * xq[u];
                            gq[i] = sn * xp[u] + c * xq[u];
                            const double y = vp[i], z = vq[i];
                            vp[i] = c * y - sn * z;
                            vq[i] = sn * y + c * z;
                        }
                    }
                }
                __syncthreads();
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
    __shared__ double pairs[3 * 512];
    __shared__ int rotated;
    __shared__ int sweeps, notconv;
    double* G = scratch;
    double* VV = scratch + m * n;
    for (int64_t e = threadIdx.x; e < m * n; e += blockDim.x) G[e] = A[e];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) VV[e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
    __syncthreads();
    jacobi_sweeps(G, m, n, VV, &sweeps, &notconv, &rotated, norms, pairs);
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
