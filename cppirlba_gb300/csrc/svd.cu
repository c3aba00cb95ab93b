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
// Restart step on a thread-block cluster, G and V distributed by rows. One-sided
// Jacobi rotates column pairs; each CTA keeps a contiguous slice of the rows of
// G and V in its own shared memory, forms the partial dot products of its rows
// for every pair of the round, and publishes them; after one cluster barrier
// every CTA adds the eight partials in rank order (so all CTAs hold identical
// sums), derives the same rotations and applies them to its own rows. Column
// norms follow Rutishauser's updates, identical in every CTA, and are
// recomputed from partials once per sweep. Per round this is one cluster
// barrier, eight distributed-shared-memory loads per pair and no remote
// stores; the work per CTA is a few rows. At the end the slices are gathered
// into CTA 0, which finishes the SVD and the restart tail.
// Rotation: t = sign(zeta) |2g| / (|b - a| + sqrt((b - a)^2 + 4 g^2)) with
// zeta = (b - a) / (2g) (Rutishauser's t without the zeta division),
// c = 1 / sqrt(1 + t^2), s = c t.
// ---------------------------------------------------------------------------
constexpr int kClusterCTAs = 8;
constexpr int kClusterThreads = 128;
constexpr int kClusterMaxN = 128;                               // work <= 128
constexpr int kClusterRows = kClusterMaxN / kClusterCTAs;       // local rows per CTA

__global__ void __cluster_dims__(kClusterCTAs, 1, 1) __launch_bounds__(kClusterThreads)
    restart_cluster_kernel(RestartArgs a) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) double sm[];   // CTA 0: gathered G and V (2 n^2 doubles)
    __shared__ double Gl[kClusterRows][kClusterMaxN];
    __shared__ double Vl[kClusterRows][kClusterMaxN];
    __shared__ double part[2][kClusterMaxN];
    __shared__ double nrm[kClusterMaxN];
    __shared__ double pc[kClusterMaxN / 2], ps[kClusterMaxN / 2];
    __shared__ double norms_local[kClusterMaxN];
    __shared__ int order[kClusterMaxN];
    __shared__ int rotated;
    // The abort flag does not change while the kernel runs: every CTA takes the
    // same branch, so no CTA waits at a barrier the others skip.
    if (a.ctrl->abort) return;
    const int rank = static_cast<int>(cl.block_rank());
    const int n = a.work;
    const int r0 = n * rank / kClusterCTAs, r1 = n * (rank + 1) / kClusterCTAs, nr = r1 - r0;
    const int tid = threadIdx.x;
    for (int e = tid; e < nr * n; e += blockDim.x) {
        const int i = e / n, j = e % n;
        Gl[i][j] = a.B[(r0 + i) + static_cast<int64_t>(j) * n];
        Vl[i][j] = (r0 + i == j) ? 1.0 : 0.0;
    }
    __syncthreads();

    const int n2 = n + (n & 1), half = n2 / 2;
    const double thresh = 2.220446049250313e-16 * static_cast<double>(n);
    // The skip test |g| <= thresh sqrt(a b), squared: one FP64 square root less
    // on each round's dependent chain (a, b >= 0).
    const double thresh2 = thresh * thresh;
    int buf = 0;
    int sweep = 0;
    for (; sweep < kMaxSweeps; ++sweep) {
        for (int j = tid; j < n; j += blockDim.x) {
            double s = 0;
            for (int i = 0; i < nr; ++i) s += Gl[i][j] * Gl[i][j];
            part[buf][j] = s;
        }
        cl.sync();
        for (int j = tid; j < n; j += blockDim.x) {
            double s = 0;
            for (int r = 0; r < kClusterCTAs; ++r) s += cl.map_shared_rank(part[buf], r)[j];
            nrm[j] = s;
        }
        buf ^= 1;
        if (tid == 0) rotated = 0;
        __syncthreads();
        for (int round = 0; round < n2 - 1; ++round) {
            for (int slot = tid; slot < half; slot += blockDim.x) {
                int p = circle_partner_a(round, slot, n2);
                int q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                double g = 0;
                if (q < n)
                    for (int i = 0; i < nr; ++i) g += Gl[i][p] * Gl[i][q];
                part[buf][slot] = g;
            }
            cl.sync();
            for (int slot = tid; slot < half; slot += blockDim.x) {
                int p = circle_partner_a(round, slot, n2);
                int q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                double c = 0, sn = 0;
                if (q < n) {
                    double g = 0;
                    for (int r = 0; r < kClusterCTAs; ++r) g += cl.map_shared_rank(part[buf], r)[slot];
                    const double av = nrm[p], bv = nrm[q];
                    if (!(g == 0.0 || g * g <= thresh2 * (av * bv))) {
                        const double d = bv - av;
                        const double t = (d >= 0 ? 1.0 : -1.0) * (g >= 0 ? 1.0 : -1.0) * fabs(2.0 * g) /
                                         (fabs(d) + sqrt(d * d + 4.0 * g * g));
                        c = rsqrt(1.0 + t * t);
                        sn = c * t;
                        nrm[p] = av - t * g;
                        nrm[q] = bv + t * g;
                        rotated = 1;
                    }
                }
                pc[slot] = c;
                ps[slot] = sn;
            }
            buf ^= 1;
            __syncthreads();
            for (int e = tid; e < half * nr; e += blockDim.x) {
                const int slot = e / nr, i = e % nr;
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
                const double x = Gl[i][p], y = Gl[i][q];
                Gl[i][p] = c * x - sn * y;
                Gl[i][q] = sn * x + c * y;
                const double u = Vl[i][p], v = Vl[i][q];
                Vl[i][p] = c * u - sn * v;
                Vl[i][q] = sn * u + c * v;
            }
            __syncthreads();
        }
        // Every CTA made the same decisions, so `rotated` agrees across the cluster.
        const int any = rotated;
        __syncthreads();
        if (!any) break;
    }
    // Gather the row slices into CTA 0 (column-major G, then V), then CTA 0
    // finishes; the others are done with distributed shared memory after the
    // barrier and may exit.
    double* G0 = cl.map_shared_rank(sm, 0);
    for (int e = tid; e < nr * n; e += blockDim.x) {
        const int i = e / n, j = e % n;
        G0[(r0 + i) + j * n] = Gl[i][j];
        G0[n * n + (r0 + i) + j * n] = Vl[i][j];
    }
    cl.sync();
    if (rank != 0) return;
    finish_svd(sm, n, n, sm + n * n, a.BS, a.BU, n, a.BV, n, norms_local, order);
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

// update_k of the restart kernel evaluated for `count` argument quadruples
// (k, requested, n_converged, work), so that the device arithmetic can be
// checked against the reference's known answers.
static __global__ void update_k_kernel(const int32_t* args, int64_t count, int32_t* out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = jacobi::update_k_dev(args[4 * i], args[4 * i + 1], args[4 * i + 2], args[4 * i + 3]);
}

void launch_update_k(const int32_t* args, int64_t count, int32_t* out, cudaStream_t stream) {
    if (count <= 0) return;
    const int64_t blocks = std::min<int64_t>((count + 255) / 256, 1024);
    update_k_kernel<<<static_cast<int>(blocks), 256, 0, stream>>>(args, count, out);
    count_launch();
}

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
    if (a.work <= kClusterMaxN && need <= g_restart_cluster_max_dynamic) {
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
