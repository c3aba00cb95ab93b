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
// a.BS, a.BU, a.BV. Warp 0 forms the residuals and the largest singular value
// and counts the converged values in parallel (a maximum and an integer count:
// the same result as the serial loops of the reference); lane 0 decides.
__device__ void restart_tail(const RestartArgs& a, int sweeps, int notconv) {
    Ctrl* ctrl = a.ctrl;
    const int n = a.work;
    const int64_t last = n - 1;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int converged = 0;
        int n_conv = 0;
        if (a.B[last + last * n] == 0.0) {
            converged = 1;
        } else {
            const double R_F = ctrl->norm_F;
            double smax = 0.0;
            for (int j = lane; j < n; j += 32) {
                a.res[j] = R_F * a.BU[last + static_cast<int64_t>(j) * n];
                smax = fmax(smax, a.BS[j]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
            if (a.iter > 0) {
                const double threshold = smax * a.tol;
                int cnt = 0;
                for (int j = lane; j < n; j += 32) {
                    const double r = R_F * a.BU[last + static_cast<int64_t>(j) * n];
                    if (fabs(r) <= threshold) {
                        const double ratio = fabs(a.BS[j] - a.prevS[j]) / a.BS[j];
                        if (ratio <= a.svtol) ++cnt;
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
                n_conv = cnt;
                if (n_conv >= a.requested) converged = 1;
            }
        }
        if (!converged)
            for (int j = lane; j < n; j += 32) a.prevS[j] = a.BS[j];
        if (lane == 0) {
            ctrl->svd_sweeps = sweeps;
            ctrl->svd_not_converged = notconv;
            ctrl->converged = converged;
            ctrl->n_converged = n_conv;
            ctrl->k_next = converged ? a.k : update_k_dev(a.k, a.requested, n_conv, n);
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
    __shared__ double pairs[3 * 512];
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

// ---------------------------------------------------------------------------
// Restart SVD for work <= 64: FP32 Jacobi preconditioning, FP64 refinement.
//
// GB300 issues FP64 at about 1/64 of its FP32 rate (two FP64 FMAs per SM and
// clock), so the Jacobi forms above spend most of their time in the FP64
// rotations of 5 to 7 sweeps of n - 1 rounds each, one round after the other.
// This form needs a few FP64 matrix products instead:
//  1. One-sided Jacobi in FP32 on B (scaled to max |B| = 1), rotating pairs
//     whose columns have |cos| > 1e-6, gives approximate right singular
//     vectors X0 (columns orthonormal and B X0 orthogonal to about 1e-6).
//  2. Refinement in FP64 (a simultaneous Jacobi step with the polar
//     orthonormalization folded in): with G = B X, C = G^T G, N = X^T X,
//     E = N - I and the skew matrix K of the Jacobi angles of C
//     (tan 2 theta_pq = 2 C_pq / (C_qq - C_pp), K_pq = theta_pq, K_qp =
//     -theta_pq), X <- X (I + D) with
//       D = -E/2 + K + 3/8 E^2 + 1/2 K^2 - 1/2 E K,
//     the second-order expansion of (I - E/2 + 3/8 E^2)(I + K + 1/2 K^2).
//     C and N are formed in FP64; D and the product X D only need FP32
//     (their rounding is below what the next step removes), so each step's
//     error falls by a factor of about 1e-7 or quadratically in the
//     off-diagonal size, whichever is smaller. Pairs with |theta| > 1e-4
//     (singular values too close for the FP32 stage to separate) are left out
//     of K and rotated exactly instead: c = cos theta, s = sin theta in FP64,
//     applied one after the other after the matrix update. It stops when
//     every pair has |C_pq| <= 8 eps sqrt(C_pp C_qq) and |N_pq - delta_pq| <=
//     8 eps, or, once both are below n eps (the skip threshold of the
//     one-sided Jacobi above), when a step no longer shrinks the coupling 4x
//     (the rounding floor of the Gram sums); columns of a null G are exempt
//     from the first test. This is a mixed-precision Jacobi method in the
//     sense of Higham, Tisseur, Webb and Zhou (refinement of a low-precision
//     Jacobi SVD in higher precision), here with the refinement written as
//     matrix products instead of sweeps.
//  3. If the refinement has not converged after kRefMaxSteps steps, CTA 0
//     runs the FP64 one-sided Jacobi above on B itself.
// The cluster's CTAs all run step 1 on the same data (identical results, no
// broadcast); in step 2 CTA r forms the Gram entries (p <= q) of the columns
// q = r, r + R, ... and the new columns X[:, q], and every CTA copies its
// results into the others' shared memory before a cluster barrier.
// Singular values are then the norms of G = B X, as in the Jacobi form
// (finish_svd: sort, U = G / sigma, completion for zero singular values,
// canonical signs).
// ---------------------------------------------------------------------------
constexpr int kRefCTAs = 8;
constexpr int kRefThreads = 512;
constexpr int kRefMaxN = 64;
constexpr int kRefLd = 65;          // column stride of the shared-memory matrices (odd: fewer bank conflicts)
constexpr int kRefMaxSteps = 8;
constexpr int kRefMaxSweeps32 = 30;
constexpr float kRefTol32 = 1e-6f;
constexpr float kRefBigAngle = 1e-4f;   // |theta| above this: an exact FP64 rotation
constexpr int kRefMaxBig = 256;         // exact rotations per step (the rest wait a step)
constexpr int kRefOwn = (kRefMaxN + kRefCTAs - 1) / kRefCTAs;   // columns owned per CTA

struct RefSmem {
    double B[kRefMaxN * kRefLd];
    double X[kRefMaxN * kRefLd];
    double G[kRefMaxN * kRefLd];
    double E[kRefMaxN * kRefLd];     // N - I, upper triangle (q >= p at [q * ld + p])
    union {
        struct {                     // step 1
            float G32[kRefMaxN * kRefLd];
            float V32[kRefMaxN * kRefLd];
        } s1;
        struct {                     // step 2
            float K32[kRefMaxN * kRefLd];   // theta_pq, upper triangle
            float E32[kRefMaxN * kRefLd];   // E, both triangles
            float D32[kRefOwn * kRefLd];    // D[:, own columns]
            float X32[kRefMaxN * kRefLd];
        } s2;
    } u;
    double lam[kRefMaxN];            // diag(C)
    double rsq[kRefMaxN];            // 1 / sqrt(C_pp), 0 for null columns
    double maxima[2 * kRefCTAs];     // per CTA: max relative off-diagonal of C, max |E|
    double big_c[kRefMaxBig], big_s[kRefMaxBig];
    unsigned char big_p[kRefMaxBig], big_q[kRefMaxBig];
    int nbig;
    int nzc[kRefMaxN][4];            // nonzero columns of each row of B (count in nzn)
    int nzn[kRefMaxN];
    double norms[kRefMaxN];
    int order[kRefMaxN];
    double pairs[3 * kRefMaxN];
    double red[32];
    int rotated, sweeps, notconv;
};

// One-sided Jacobi in FP32 on G (n x n, column stride kRefLd) accumulating V,
// rotating a pair when |g_p . g_q| > tol |g_p| |g_q|. Eight lanes per pair
// (four pairs per warp), lane l of a pair holding rows l, l + 8, ..., so a
// round costs three shuffle levels per sum; rotation parameters by every lane
// of the pair (Rutishauser's formulas). n <= 64. Returns the sweeps made.
constexpr int kJ32Lanes = 8;
constexpr int kJ32Rows = kRefMaxN / kJ32Lanes;
__device__ int jacobi32_sweeps(float* G, float* V, int n, float tol) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = static_cast<int>(blockDim.x >> 5);
    const int sub = lane / kJ32Lanes, gl = lane % kJ32Lanes;
    const int n2 = n + (n & 1), half = n2 / 2;
    int sweep = 0;
    for (; sweep < kRefMaxSweeps32; ++sweep) {
        int rotated = 0;
        for (int round = 0; round < n2 - 1; ++round) {
            for (int slot = warp * (32 / kJ32Lanes) + sub; slot - sub < half; slot += nw * (32 / kJ32Lanes)) {
                int p = 0, q = n;
                if (slot < half) {
                    p = circle_partner_a(round, slot, n2);
                    q = circle_partner_b(round, slot, n2);
                    if (p > q) {
                        const int tmp = p;
                        p = q;
                        q = tmp;
                    }
                }
                const bool live = q < n;
                float* gp = G + p * kRefLd;
                float* gq = G + q * kRefLd;
                float x[kJ32Rows], y[kJ32Rows];
                float a = 0.f, b = 0.f, g = 0.f;
#pragma unroll
                for (int t = 0; t < kJ32Rows; ++t) {
                    const int i = gl + t * kJ32Lanes;
                    x[t] = (live && i < n) ? gp[i] : 0.f;
                    y[t] = (live && i < n) ? gq[i] : 0.f;
                    a = fmaf(x[t], x[t], a);
                    b = fmaf(y[t], y[t], b);
                    g = fmaf(x[t], y[t], g);
                }
#pragma unroll
                for (int o = kJ32Lanes / 2; o > 0; o >>= 1) {
                    a += __shfl_xor_sync(0xffffffffu, a, o);
                    b += __shfl_xor_sync(0xffffffffu, b, o);
                    g += __shfl_xor_sync(0xffffffffu, g, o);
                }
                if (live && fabsf(g) > tol * sqrtf(a) * sqrtf(b)) {
                    const float zeta = (b - a) / (2.f * g);
                    const float tt = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
                    const float c = rsqrtf(1.f + tt * tt), sn = c * tt;
                    float* vp = V + p * kRefLd;
                    float* vq = V + q * kRefLd;
#pragma unroll
                    for (int t = 0; t < kJ32Rows; ++t) {
                        const int i = gl + t * kJ32Lanes;
                        if (i < n) {
                            gp[i] = c * x[t] - sn * y[t];
                            gq[i] = sn * x[t] + c * y[t];
                            const float u = vp[i], v = vq[i];
                            vp[i] = c * u - sn * v;
                            vq[i] = sn * u + c * v;
                        }
                    }
                    rotated = 1;
                }
            }
            __syncthreads();
        }
        if (!__syncthreads_or(rotated)) break;
    }
    return sweep + 1;
}

// G = B X with B's rows given as lists of nonzero columns (rows with more than
// four nonzeros are marked with nzn = -1 and summed densely).
__device__ void ref_bx(RefSmem& S, int n) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int j = e / n, i = e % n;
        const double* x = S.X + j * kRefLd;
        double acc = 0;
        const int cnt = S.nzn[i];
        if (cnt >= 0) {
            for (int t = 0; t < cnt; ++t) {
                const int l = S.nzc[i][t];
                acc += S.B[l * kRefLd + i] * x[l];
            }
        } else {
            for (int l = i; l < n; ++l) acc += S.B[l * kRefLd + i] * x[l];
        }
        S.G[j * kRefLd + i] = acc;
    }
}

// Maximum of v over the CTA (fixed order), valid in every thread.
__device__ double ref_block_max(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double m = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    __syncthreads();
    return m;
}

__global__ void __cluster_dims__(kRefCTAs, 1, 1) __launch_bounds__(kRefThreads)
    restart_refine_kernel(RestartArgs a) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char ref_raw[];
    RefSmem& S = *reinterpret_cast<RefSmem*>(ref_raw);
    // The abort flag does not change while the kernel runs: every CTA returns
    // together, so none waits at a barrier the others skip.
    if (a.ctrl->abort) return;
    const int rank = static_cast<int>(cl.block_rank());
    const int n = a.work;
    const int tid = threadIdx.x;

    // B into shared memory, its row structure, and the FP32 copy scaled by max |B|.
    double bmax = 0;
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int j = e / n, i = e % n;
        const double v = a.B[static_cast<int64_t>(j) * n + i];
        S.B[j * kRefLd + i] = v;
        bmax = fmax(bmax, fabs(v));
    }
    bmax = ref_block_max(bmax, S.red);
    const float inv = bmax > 0 ? static_cast<float>(1.0 / bmax) : 1.f;
    for (int i = tid; i < n; i += blockDim.x) {
        int cnt = 0;
        for (int l = 0; l < n; ++l) {
            if (S.B[l * kRefLd + i] != 0.0) {
                if (cnt < 4) S.nzc[i][cnt] = l;
                ++cnt;
            }
        }
        S.nzn[i] = cnt <= 4 ? cnt : -1;
    }
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int j = e / n, i = e % n;
        S.u.s1.G32[j * kRefLd + i] = static_cast<float>(S.B[j * kRefLd + i]) * inv;
        S.u.s1.V32[j * kRefLd + i] = (i == j) ? 1.f : 0.f;
    }
    __syncthreads();

    // Step 1: FP32 Jacobi (every CTA, identical results).
    jacobi32_sweeps(S.u.s1.G32, S.u.s1.V32, n, kRefTol32);
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int j = e / n, i = e % n;
        S.X[j * kRefLd + i] = static_cast<double>(S.u.s1.V32[j * kRefLd + i]);
    }
    // The FP32 arrays share storage with what the other CTAs write next.
    cl.sync();

    // Own columns of this CTA and the offsets of their Gram items (p <= q).
    int own_q[kRefOwn];
    int own_off[kRefOwn + 1];
    int nown = 0;
    own_off[0] = 0;
    for (int q = rank; q < n; q += kRefCTAs) {
        own_q[nown] = q;
        own_off[nown + 1] = own_off[nown] + q + 1;
        ++nown;
    }
    const int nitems = own_off[nown];
    const double eps = 2.220446049250313e-16;

    int steps = 0;
    bool converged = false;
    double prev_off = 1.0;
    for (; steps <= kRefMaxSteps; ++steps) {
        // X is stable until this step's update phase (the other CTAs write
        // their new columns only after the barrier below).
        ref_bx(S, n);
        for (int e = tid; e < n * n; e += blockDim.x) {
            const int j = e / n, i = e % n;
            S.u.s2.X32[j * kRefLd + i] = static_cast<float>(S.X[j * kRefLd + i]);
        }
        __syncthreads();
        // diag(C) and 1 / sqrt(C_pp) (0 for columns of a null G).
        double lmax = 0;
        for (int j = tid; j < n; j += blockDim.x) {
            const double* g = S.G + j * kRefLd;
            double s = 0;
            for (int i = 0; i < n; ++i) s += g[i] * g[i];
            S.lam[j] = s;
            lmax = fmax(lmax, s);
        }
        lmax = ref_block_max(lmax, S.red);
        const double null_floor = lmax * (eps * n) * (eps * n);
        for (int j = tid; j < n; j += blockDim.x) S.rsq[j] = S.lam[j] > null_floor ? rsqrt(S.lam[j]) : 0.0;
        __syncthreads();

        // Gram items of the own columns: C_pq, N_pq; E_pq and theta_pq to every
        // CTA. Four lanes per item (rows i = l, l + 4, ...), so the FP64 work
        // spreads over all warps of the CTA.
        double offmax = 0, emax = 0;
        const int q4 = tid & 3;
        for (int it0 = 0; it0 < nitems; it0 += static_cast<int>(blockDim.x >> 2)) {
            const int it = it0 + (tid >> 2);
            const bool has = it < nitems;
            int o = 0;
            if (has)
                while (own_off[o + 1] <= it) ++o;
            const int q = has ? own_q[o] : 0, p = has ? it - own_off[o] : 0;
            const double* gp = S.G + p * kRefLd;
            const double* gq = S.G + q * kRefLd;
            const double* xp = S.X + p * kRefLd;
            const double* xq = S.X + q * kRefLd;
            double c = 0, nn = 0;
            if (has)
                for (int i = q4; i < n; i += 4) {
                    c += gp[i] * gq[i];
                    nn += xp[i] * xq[i];
                }
            c += __shfl_xor_sync(0xffffffffu, c, 1);
            nn += __shfl_xor_sync(0xffffffffu, nn, 1);
            c += __shfl_xor_sync(0xffffffffu, c, 2);
            nn += __shfl_xor_sync(0xffffffffu, nn, 2);
            if (!has || q4 != 0) continue;
            const double e = nn - (p == q ? 1.0 : 0.0);
            emax = fmax(emax, fabs(e));
            float th = 0.f;
            if (p != q && c != 0.0) {
                // tan 2 theta = 2 C_pq / (C_qq - C_pp), |theta| <= pi / 4, from
                // the scaled C_pq sqrt(1 / (C_pp C_qq)) and difference (no FP64
                // division on the common path).
                const double rp = S.rsq[p], rq = S.rsq[q];
                float num, den;
                if (rp > 0 && rq > 0) {
                    const double r = rp * rq;
                    const double cr = c * r;
                    offmax = fmax(offmax, fabs(cr));
                    num = static_cast<float>(cr);
                    den = static_cast<float>((S.lam[q] - S.lam[p]) * r);
                } else if (rp > 0 || rq > 0) {
                    // One column of a null G: a small rotation against the other.
                    const double big = rp > 0 ? S.lam[p] : S.lam[q];
                    num = static_cast<float>(c / big);
                    den = rp > 0 ? -1.f : 1.f;
                } else {
                    num = 0.f;
                    den = 1.f;
                }
                if (num != 0.f) th = den == 0.f ? copysignf(0.78539816f, num) : 0.5f * atanf(2.f * num / den);
            }
            for (int r = 0; r < kRefCTAs; ++r) {
                double* Er = cl.map_shared_rank(S.E, r);
                float* Kr = cl.map_shared_rank(S.u.s2.K32, r);
                Er[q * kRefLd + p] = e;
                Kr[q * kRefLd + p] = th;
            }
        }
        offmax = ref_block_max(offmax, S.red);
        emax = ref_block_max(emax, S.red);
        if (tid == 0)
            for (int r = 0; r < kRefCTAs; ++r) {
                double* mr = cl.map_shared_rank(S.maxima, r);
                mr[2 * rank] = offmax;
                mr[2 * rank + 1] = emax;
            }
        cl.sync();
        double goff = 0, gem = 0;
        for (int r = 0; r < kRefCTAs; ++r) {
            goff = fmax(goff, S.maxima[2 * r]);
            gem = fmax(gem, S.maxima[2 * r + 1]);
        }
        // Converged at 8 eps; or, once below the one-sided Jacobi's skip
        // threshold n eps, as soon as a step no longer shrinks the coupling by
        // 4x (the Gram sums' rounding floor).
        if ((goff <= 8 * eps && gem <= 8 * eps) ||
            (goff <= n * eps && gem <= n * eps && goff > 0.25 * prev_off)) {
            converged = true;
            break;
        }
        prev_off = goff;
        if (steps == kRefMaxSteps) break;

        // D[:, own] = -E/2 + K + 3/8 E^2 + 1/2 K^2 - 1/2 E K (second order in FP32).
        for (int e = tid; e < n * n; e += blockDim.x) {
            const int q = e / n, p = e % n;
            S.u.s2.E32[q * kRefLd + p] = static_cast<float>(p <= q ? S.E[q * kRefLd + p] : S.E[p * kRefLd + q]);
        }
        __syncthreads();
        auto Eat = [&](int p, int q) -> float { return S.u.s2.E32[q * kRefLd + p]; };
        auto Kat = [&](int p, int q) -> float {
            const float t = p == q ? 0.f : (p < q ? S.u.s2.K32[q * kRefLd + p] : -S.u.s2.K32[p * kRefLd + q]);
            return fabsf(t) > kRefBigAngle ? 0.f : t;
        };
        // The large angles, in a fixed order (column q, then row p), with
        // their FP64 cosines and sines.
        if (tid < 32) {
            int count = 0;
            for (int q = 1; q < n; ++q) {
                for (int p0 = 0; p0 < q; p0 += 32) {
                    const int p = p0 + tid;
                    const bool big = p < q && fabsf(S.u.s2.K32[q * kRefLd + p]) > kRefBigAngle;
                    const unsigned m = __ballot_sync(0xffffffffu, big);
                    const int slot = count + __popc(m & ((1u << tid) - 1u));
                    if (big && slot < kRefMaxBig) {
                        S.big_p[slot] = static_cast<unsigned char>(p);
                        S.big_q[slot] = static_cast<unsigned char>(q);
                    }
                    count += __popc(m);
                }
            }
            if (tid == 0) S.nbig = count < kRefMaxBig ? count : kRefMaxBig;
        }
        __syncthreads();
        for (int b = tid; b < S.nbig; b += blockDim.x) {
            const double t = static_cast<double>(S.u.s2.K32[S.big_q[b] * kRefLd + S.big_p[b]]);
            sincos(t, &S.big_s[b], &S.big_c[b]);
        }
        for (int e = tid; e < nown * n; e += blockDim.x) {
            const int o = e / n, p = e % n, q = own_q[o];
            float ee = 0, kk = 0, ek = 0;
            for (int r = 0; r < n; ++r) {
                const float epr = Eat(p, r), kpr = Kat(p, r);
                const float erq = Eat(r, q), krq = Kat(r, q);
                ee += epr * erq;
                kk += kpr * krq;
                ek += epr * krq;
            }
            const double first = -0.5 * (p <= q ? S.E[q * kRefLd + p] : S.E[p * kRefLd + q]) +
                                 static_cast<double>(Kat(p, q));
            S.u.s2.D32[o * kRefLd + p] = static_cast<float>(first) + (0.375f * ee + 0.5f * kk - 0.5f * ek);
        }
        __syncthreads();
        // X[:, q] += X D[:, q] for the own columns, into every CTA.
        for (int e = tid; e < nown * n; e += blockDim.x) {
            const int o = e / n, i = e % n, q = own_q[o];
            float acc = 0;
            const float* d = S.u.s2.D32 + o * kRefLd;
            for (int p = 0; p < n; ++p) acc += S.u.s2.X32[p * kRefLd + i] * d[p];
            const double xn = S.X[q * kRefLd + i] + static_cast<double>(acc);
            for (int r = 0; r < kRefCTAs; ++r) cl.map_shared_rank(S.X, r)[q * kRefLd + i] = xn;
        }
        cl.sync();
        // The exact rotations, on every CTA's copy of X (same order, same result):
        // x_p <- c x_p - s x_q, x_q <- s x_p + c x_q.
        for (int b = 0; b < S.nbig; ++b) {
            const int p = S.big_p[b], q = S.big_q[b];
            const double c = S.big_c[b], sn = S.big_s[b];
            for (int i = tid; i < n; i += blockDim.x) {
                const double xv = S.X[p * kRefLd + i], yv = S.X[q * kRefLd + i];
                S.X[p * kRefLd + i] = c * xv - sn * yv;
                S.X[q * kRefLd + i] = sn * xv + c * yv;
            }
            __syncthreads();
        }
    }
    // No CTA touches another's shared memory after this barrier.
    cl.sync();
    if (rank != 0) return;

    // G and X into contiguous n x n arrays (reusing E and the FP32 area); if
    // the refinement did not converge, B and the identity instead, for the
    // FP64 one-sided Jacobi.
    double* Gc = S.E;
    double* Xc = reinterpret_cast<double*>(&S.u);
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int j = e / n, i = e % n;
        Gc[j * n + i] = converged ? S.G[j * kRefLd + i] : S.B[j * kRefLd + i];
        Xc[j * n + i] = converged ? S.X[j * kRefLd + i] : (i == j ? 1.0 : 0.0);
    }
    __syncthreads();
    int sweeps = steps, notconv = 0;
    if (!converged) {
        jacobi_sweeps(Gc, n, n, Xc, &S.sweeps, &S.notconv, &S.rotated, S.norms, S.pairs);
        sweeps = steps + 100 * S.sweeps;
        notconv = S.notconv;
    }
    finish_svd(Gc, n, n, Xc, a.BS, a.BU, n, a.BV, n, S.norms, S.order);
    restart_tail(a, sweeps, notconv);
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

// The restart tail alone (convergence test, update_k, B rebuilt) after the
// SVD of B was formed elsewhere (cuSOLVER for working subspaces above 1024).
static __global__ void __launch_bounds__(256) restart_tail_kernel(RestartArgs a) {
    if (a.ctrl->abort) return;
    restart_tail(a, 0, 0);
}

void launch_restart_tail(const RestartArgs& a, cudaStream_t stream) {
    restart_tail_kernel<<<1, 256, 0, stream>>>(a);
    count_launch();
}

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

static bool g_restart_refine_ok = false;

cudaError_t restart_configure(size_t smem_optin) {
    cudaError_t e = allow_dynamic_smem(restart_kernel, smem_optin, &g_restart_max_dynamic);
    if (e == cudaSuccess) e = allow_dynamic_smem(restart_cluster_kernel, smem_optin, &g_restart_cluster_max_dynamic);
    if (e == cudaSuccess) {
        size_t avail = 0;
        e = allow_dynamic_smem(restart_refine_kernel, smem_optin, &avail);
        g_restart_refine_ok = e == cudaSuccess && avail >= sizeof(RefSmem);
    }
    return e;
}

void launch_restart(const RestartArgs& a, cudaStream_t stream, size_t /*max_smem*/) {
    if (a.work <= kRefMaxN && g_restart_refine_ok) {
        restart_refine_kernel<<<kRefCTAs, kRefThreads, sizeof(RefSmem), stream>>>(a);
        count_launch();
        return;
    }
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
