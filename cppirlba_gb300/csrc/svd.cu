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
//     C and N are formed in FP64; D, the angles and the product X D only need
//     FP32 (their rounding is below what the next step removes), so each
//     step's error falls by a factor of about 1e-7 or quadratically in the
//     off-diagonal size, whichever is smaller. Pairs with |theta| > 1e-4
//     (singular values too close for the FP32 stage to separate) are left out
//     of K and rotated exactly instead, after the matrix update, in a fixed
//     order (column q, then row p); their cosines and sines are FP32 values
//     scaled to c^2 + s^2 = 1 in FP64, so the rotations are orthogonal to FP64
//     precision. It stops when every pair has |C_pq| <= 8 eps sqrt(C_pp C_qq)
//     and |N_pq - delta_pq| <= 8 eps, or, once both are below n eps (the skip
//     threshold of the one-sided Jacobi above), when a step no longer shrinks
//     the coupling 4x (the rounding floor of the Gram sums); columns of a null
//     G are exempt from the first test. This is a mixed-precision Jacobi method
//     in the sense of Higham, Tisseur, Webb and Zhou (refinement of a
//     low-precision Jacobi SVD in higher precision), here with the refinement
//     written as matrix products instead of sweeps.
//  3. If the refinement has not converged after kRefMaxSteps steps, CTA 0
//     runs the FP64 one-sided Jacobi above on B itself.
// Work split: the cluster's CTAs all run step 1 on the same data (identical
// results, no broadcast). In step 2 CTA r owns the columns q = r, r + R, ...:
// it forms G[:, q] = B X[:, q], C_qq and the FP32 copy of X[:, q], then the
// Gram entries (p <= q) and the new X[:, q], and copies each result into
// every CTA's shared memory before the cluster barrier that publishes it
// (three per step). Every CTA applies the exact rotations to its own full
// copy of X, in the same order (thread i rotates row i, so no barrier
// separates them). Singular values are then the norms of G = B X, as in the
// Jacobi form; each CTA writes the singular values and the U = G / sigma and
// V = X columns of its own columns in sorted order with canonical signs (the
// finish_svd conventions), and CTA 0 runs the restart tail. If a singular
// value is zero (U has to be completed) CTA 0 finishes alone with finish_svd.
// ---------------------------------------------------------------------------
constexpr int kRefCTAs = 8;
constexpr int kRefThreads = 512;
constexpr int kRefMaxN = 64;
constexpr int kRefLd = 65;          // column stride of the FP64 matrices (odd: fewer bank conflicts)
constexpr int kJ32Ld = 64;          // column stride of the FP32 Jacobi matrices (rows n..63 zero)
constexpr int kRefMaxSteps = 8;
constexpr int kRefMaxSweeps32 = 30;
constexpr float kRefTol32 = 1e-6f;
constexpr float kRefStop32 = 1e-4f;     // a sweep whose rotations all had |cos| below this is the last
constexpr float kRefBigAngle = 1e-4f;   // |theta| above this: an exact rotation (first two steps)
constexpr float kRefBigAngleLate = 1e-6f;   // the same from the third step on
constexpr int kRefMaxBig = 256;         // exact rotations per step (the rest wait a step)
constexpr int kRefOwn = (kRefMaxN + kRefCTAs - 1) / kRefCTAs;   // columns owned per CTA

struct RefSmem {
    double B[kRefMaxN * kRefLd];
    double X[kRefMaxN * kRefLd];
    double G[kRefMaxN * kRefLd];
    double E[kRefMaxN * kRefLd];     // N - I, upper triangle (q >= p at [q * ld + p])
    union {
        struct {                     // step 1
            float4 G32[kRefMaxN * kJ32Ld / 4];
            float4 V32[kRefMaxN * kJ32Ld / 4];
            unsigned short ptab[kRefMaxN * 32];   // round r, slot s: p | q << 8 (p < q), 0xffff: no pair
        } s1;
        struct {                     // step 2
            float2 EK[kRefMaxN * kRefLd];   // (E_pq, theta_pq) at [q * ld + p]: upper triangle, then full
            float D32[kRefOwn * kRefLd];    // D[:, own columns]
            float X32[kRefMaxN * kRefLd];
        } s2;
    } u;
    double lam[kRefMaxN];            // C_jj = |G[:, j]|^2
    float lamf[kRefMaxN];            // C_jj / max C
    float rsqf[kRefMaxN];            // (C_jj / max C)^(-1/2), 0 for null columns
    double inv_lmax;
    float maxima[3 * kRefCTAs];      // per CTA: max relative off-diagonal of C, max |E|, max |theta|
    float redf[96];
    double big_c[kRefMaxBig], big_s[kRefMaxBig];
    unsigned char big_p[kRefMaxBig], big_q[kRefMaxBig];
    int big_cnt[kRefMaxN];           // large angles in column q, then their offsets
    int nbig;
    int nzc[kRefMaxN][4];            // nonzero columns of each row of B (count in nzn)
    int nzn[kRefMaxN];
    double norms[kRefMaxN];
    int order[kRefMaxN];
    int rankof[kRefMaxN];
    double invsg[kRefMaxN];          // canonical sign / singular value of column j (from its owner)
    double prevS[kRefMaxN];          // the previous restart's singular values
    double tail_res[kRefMaxN];
    double R_F;
    int tail_conv, tail_kn;
    double pairs[3 * kRefMaxN];
    double red[32];
    unsigned long long redu[32];
    int rotated, sweeps, notconv;
    unsigned int j32max;
};

// One-sided Jacobi in FP32 on G (n x n) accumulating V, both stored as n
// columns of kJ32Ld floats (rows n..63 zero), rotating a pair when
// (g_p . g_q)^2 > tol^2 |g_p|^2 |g_q|^2. Sixteen lanes per pair (two pairs per
// warp, so 16 warps cover the 32 slots of n <= 64), lane l holding rows
// 4l .. 4l + 3 of both columns of G and V in one 16-byte load each, so a
// round is four loads, a four-level shuffle tree, the rotation and one CTA
// barrier. The pairs of each round come from ptab (the circle ordering,
// prepared once); the rotation is Rutishauser's, written as
// t = sign(d) 2 g / (|d| + sqrt(d^2 + 4 g^2)), d = |g_q|^2 - |g_p|^2, with the
// hardware reciprocal and reciprocal square root: this stage only has to
// bring the angles below what the FP64 refinement resolves. The sweeps stop
// when a sweep rotates nothing, or when the largest |cos| it rotated was
// below `stop` (the next sweep would take them to about stop^2: no further
// sweep is needed for the refinement). jmax: one shared word, zero on entry.
// The rounds are limited by shared-memory and shuffle throughput (every
// column is read each round), so V is read only for pairs that rotate.
// Returns the sweeps made.
__device__ int jacobi32_sweeps(float4* G, float4* V, const unsigned short* ptab, int n, float tol, float stop,
                               unsigned int* jmax) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane >> 4, gl = lane & 15;
    const int n2 = n + (n & 1), half = n2 / 2;
    const int nrounds = n2 - 1;
    const int slot = 2 * warp + sub;
    const bool busy = 2 * warp < half;     // warp-uniform
    const float tol2 = tol * tol, stop2 = stop * stop;
    constexpr int kC = kJ32Ld / 4;         // float4 per column
    int sweep = 0;
    for (; sweep < kRefMaxSweeps32; ++sweep) {
        int rotated = 0;
        float cmax2 = 0.f;
        unsigned int pq_next = (busy && slot < half) ? ptab[slot] : 0xffffu;
        for (int round = 0; round < nrounds; ++round) {
            const unsigned int pq = pq_next;
            if (busy && slot < half && round + 1 < nrounds) pq_next = ptab[(round + 1) * 32 + slot];
            if (busy) {
                const bool live = pq != 0xffffu;
                const int p = static_cast<int>(pq & 0xffu), q = static_cast<int>(pq >> 8);
                float4 x = make_float4(0.f, 0.f, 0.f, 0.f), y = x;
                if (live) {
                    x = G[p * kC + gl];
                    y = G[q * kC + gl];
                }
                float a = x.x * x.x, b = y.x * y.x, g = x.x * y.x;
                a = fmaf(x.y, x.y, a);
                b = fmaf(y.y, y.y, b);
                g = fmaf(x.y, y.y, g);
                a = fmaf(x.z, x.z, a);
                b = fmaf(y.z, y.z, b);
                g = fmaf(x.z, y.z, g);
                a = fmaf(x.w, x.w, a);
                b = fmaf(y.w, y.w, b);
                g = fmaf(x.w, y.w, g);
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) {
                    a += __shfl_xor_sync(0xffffffffu, a, o);
                    b += __shfl_xor_sync(0xffffffffu, b, o);
                    g += __shfl_xor_sync(0xffffffffu, g, o);
                }
                if (live && g * g > tol2 * a * b) {
                    const float4 u = V[p * kC + gl], v = V[q * kC + gl];
                    cmax2 = fmaxf(cmax2, __fdividef(g * g, a * b));
                    const float d = b - a;
                    const float h = fmaf(d, d, 4.f * g * g);
                    const float den = fabsf(d) + h * rsqrtf(h);
                    const float t = __fdividef((d >= 0.f ? 2.f : -2.f) * g, den);
                    const float c = rsqrtf(fmaf(t, t, 1.f)), s = c * t;
                    G[p * kC + gl] = make_float4(c * x.x - s * y.x, c * x.y - s * y.y, c * x.z - s * y.z,
                                                 c * x.w - s * y.w);
                    G[q * kC + gl] = make_float4(s * x.x + c * y.x, s * x.y + c * y.y, s * x.z + c * y.z,
                                                 s * x.w + c * y.w);
                    V[p * kC + gl] = make_float4(c * u.x - s * v.x, c * u.y - s * v.y, c * u.z - s * v.z,
                                                 c * u.w - s * v.w);
                    V[q * kC + gl] = make_float4(s * u.x + c * v.x, s * u.y + c * v.y, s * u.z + c * v.z,
                                                 s * u.w + c * v.w);
                    rotated = 1;
                }
            }
            __syncthreads();
        }
        const unsigned int wm = __reduce_max_sync(0xffffffffu, __float_as_uint(cmax2));
        if ((threadIdx.x & 31) == 0 && wm != 0u) atomicMax(jmax, wm);
        __syncthreads();
        const float m2 = __uint_as_float(*jmax);
        const int go_on = __syncthreads_or(rotated) && !(m2 < stop2);
        if (threadIdx.x == 0) *jmax = 0u;
        if (!go_on) break;
    }
    return sweep + 1;
}

// Maxima of three non-negative values over the CTA, valid in every thread.
// red: 96 floats not otherwise in use until the CTA's next barrier after this
// call.
__device__ void ref_block_max3f(float& x, float& y, float& z, float* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
        y = fmaxf(y, __shfl_xor_sync(0xffffffffu, y, o));
        z = fmaxf(z, __shfl_xor_sync(0xffffffffu, z, o));
    }
    if (lane == 0) {
        red[warp] = x;
        red[32 + warp] = y;
        red[64 + warp] = z;
    }
    __syncthreads();
    x = 0.f;
    y = 0.f;
    z = 0.f;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
        x = fmaxf(x, red[w]);
        y = fmaxf(y, red[32 + w]);
        z = fmaxf(z, red[64 + w]);
    }
}

// Maximum of v over the CTA, valid in every thread (integer: the order of
// non-negative doubles is the order of their bit patterns).
__device__ unsigned long long ref_block_maxu(unsigned long long v, unsigned long long* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    if (lane == 0) red[warp] = v;
    __syncthreads();
    unsigned long long m = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) m = red[w] > m ? red[w] : m;
    return m;
}

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7fffffffffffffffull;
}

// The restart tail of restart_tail (the convergence test, update_k and the
// rebuild of B, with the same predicates and values) on CTA 0 of the refine
// kernel, from shared memory: the singular values and their order, B, and the
// sign / singular value factors the owners of the columns used, so that
// U[last, jj] = G[last, j] * invsg[j] is the value the owner wrote.
__device__ void refine_tail(const RestartArgs& a, RefSmem& S, int sweeps) {
    Ctrl* ctrl = a.ctrl;
    const int n = a.work;
    const int last = n - 1;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int converged = 0;
        int n_conv = 0;
        if (S.B[last * kRefLd + last] == 0.0) {
            converged = 1;
        } else {
            const double R_F = S.R_F;
            for (int jj = lane; jj < n; jj += 32) {
                const int j = S.order[jj];
                const double r = R_F * (S.G[j * kRefLd + last] * S.invsg[j]);
                S.tail_res[jj] = r;
                a.res[jj] = r;
            }
        }
        if (!converged && a.iter > 0) {
            const double threshold = S.norms[S.order[0]] * a.tol;
            int cnt = 0;
            for (int jj = lane; jj < n; jj += 32) {
                if (fabs(S.tail_res[jj]) <= threshold) {
                    const double bs = S.norms[S.order[jj]];
                    const double ratio = fabs(bs - S.prevS[jj]) / bs;
                    if (ratio <= a.svtol) ++cnt;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            n_conv = cnt;
            if (n_conv >= a.requested) converged = 1;
        }
        if (!converged)
            for (int jj = lane; jj < n; jj += 32) a.prevS[jj] = S.norms[S.order[jj]];
        if (lane == 0) {
            const int kn = converged ? a.k : update_k_dev(a.k, a.requested, n_conv, n);
            ctrl->svd_sweeps = sweeps;
            ctrl->svd_not_converged = 0;
            ctrl->converged = converged;
            ctrl->n_converged = n_conv;
            ctrl->k_next = kn;
            S.tail_conv = converged;
            S.tail_kn = kn;
        }
    }
    __syncthreads();
    if (!S.tail_conv) {
        const int kn = S.tail_kn;
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            const int j = e / n, i = e % n;
            double v = 0.0;
            if (i < kn && j == i) v = S.norms[S.order[i]];
            else if (i < kn && j == kn) v = S.tail_res[i];
            a.B[e] = v;
        }
    }
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
    const int lane = tid & 31, warp = tid >> 5;
    const int nw = static_cast<int>(blockDim.x >> 5);

    // B into shared memory, its row structure, and the FP32 copy scaled by max
    // |B| (the comparisons on integer bit patterns: FP64 compares use the
    // narrow FP64 pipe); the pair table of the FP32 Jacobi; the previous
    // singular values and ||F|| for the tail.
    unsigned long long bmaxu = 0;
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int j = e / n, i = e % n;
        const double v = a.B[static_cast<int64_t>(j) * n + i];
        S.B[j * kRefLd + i] = v;
        const unsigned long long av = abs_bits(v);
        bmaxu = av > bmaxu ? av : bmaxu;
    }
    if (rank == 0) {
        for (int j = tid; j < n; j += blockDim.x) S.prevS[j] = a.prevS[j];
        if (tid == 0) S.R_F = a.ctrl->norm_F;
    }
    if (tid == 0) S.j32max = 0u;
    {
        const int n2 = n + (n & 1), half = n2 / 2;
        for (int e = tid; e < (n2 - 1) * 32; e += blockDim.x) {
            const int round = e / 32, slot = e % 32;
            unsigned short v = 0xffffu;
            if (slot < half) {
                int p = circle_partner_a(round, slot, n2), q = circle_partner_b(round, slot, n2);
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                if (q < n) v = static_cast<unsigned short>(p | (q << 8));
            }
            S.u.s1.ptab[e] = v;
        }
    }
    const double bmax = __longlong_as_double(static_cast<long long>(ref_block_maxu(bmaxu, S.redu)));
    const float inv = bmax > 0 ? static_cast<float>(1.0 / bmax) : 1.f;
    for (int i = tid; i < n; i += blockDim.x) {
        int cnt = 0;
        for (int l = 0; l < n; ++l) {
            if (abs_bits(S.B[l * kRefLd + i]) != 0ull) {
                if (cnt < 4) S.nzc[i][cnt] = l;
                ++cnt;
            }
        }
        S.nzn[i] = cnt <= 4 ? cnt : -1;
    }
    float* G32 = reinterpret_cast<float*>(S.u.s1.G32);
    float* V32 = reinterpret_cast<float*>(S.u.s1.V32);
    for (int e = tid; e < n * kJ32Ld; e += blockDim.x) {
        const int j = e / kJ32Ld, i = e % kJ32Ld;
        G32[e] = i < n ? static_cast<float>(S.B[j * kRefLd + i]) * inv : 0.f;
        V32[e] = i == j ? 1.f : 0.f;
    }
    __syncthreads();

    // Step 1: FP32 Jacobi (every CTA, identical results).
    jacobi32_sweeps(S.u.s1.G32, S.u.s1.V32, S.u.s1.ptab, n, kRefTol32, kRefStop32, &S.j32max);
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int j = e / n, i = e % n;
        S.X[j * kRefLd + i] = static_cast<double>(V32[j * kJ32Ld + i]);
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
    const float feps = 2.220446049250313e-16f;
    float2* EK = S.u.s2.EK;

    int steps = 0;
    bool converged = false;
    float prev_off = 1.f;
    for (; steps <= kRefMaxSteps; ++steps) {
        // (a) G[:, q] = B X[:, q], C_qq and the FP32 copy of X[:, q] for the own
        // columns (one warp per column), into every CTA.
        if (warp < nown) {
            const int q = own_q[warp];
            const double* x = S.X + q * kRefLd;
            double ss = 0;
            for (int i = lane; i < n; i += 32) {
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
                ss += acc * acc;
                const float x32 = static_cast<float>(x[i]);
                for (int r = 0; r < kRefCTAs; ++r) {
                    cl.map_shared_rank(S.G, r)[q * kRefLd + i] = acc;
                    cl.map_shared_rank(S.u.s2.X32, r)[q * kRefLd + i] = x32;
                }
            }
            ss = warp_sum(ss);
            if (lane < kRefCTAs) cl.map_shared_rank(S.lam, lane)[q] = ss;
        }
        cl.sync();
        // C_jj / max C in FP32 for the angles and the coupling measure.
        if (warp == 0) {
            const double l0 = lane < n ? S.lam[lane] : 0.0, l1 = lane + 32 < n ? S.lam[lane + 32] : 0.0;
            double lm = fmax(l0, l1);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
            const double il = lm > 0 ? 1.0 / lm : 0.0;
            if (lane == 0) S.inv_lmax = il;
            const float nfl = static_cast<float>(n) * feps;
            for (int j = lane; j < n; j += 32) {
                const float lf = static_cast<float>(S.lam[j] * il);
                S.lamf[j] = lf;
                S.rsqf[j] = lf > nfl * nfl ? rsqrtf(lf) : 0.f;
            }
        }
        __syncthreads();

        // (b) Gram entries of the own columns: C_pq, N_pq in FP64, four lanes
        // per entry (rows i = l, l + 4, ...), so the FP64 work spreads over all
        // warps; E_pq and theta_pq to every CTA (each lane of the four writes two).
        float offmax = 0.f, emax = 0.f, thmax = 0.f;
        const int q4 = tid & 3;
        const double il = S.inv_lmax;
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
            const double e = nn - (p == q ? 1.0 : 0.0);
            float th = 0.f;
            if (has && q4 == 0) {
                emax = fmaxf(emax, fabsf(static_cast<float>(e)));
                if (p != q && c != 0.0) {
                    // tan 2 theta = 2 C_pq / (C_qq - C_pp), |theta| <= pi / 4, from
                    // C scaled by its largest diagonal entry.
                    const float rp = S.rsqf[p], rq = S.rsqf[q];
                    const float cn = static_cast<float>(c * il);
                    float num, den;
                    if (rp > 0.f && rq > 0.f) {
                        const float r = rp * rq;
                        num = cn * r;
                        offmax = fmaxf(offmax, fabsf(num));
                        den = static_cast<float>((S.lam[q] - S.lam[p]) * il) * r;
                    } else if (rp > 0.f || rq > 0.f) {
                        // One column of a null G: a small rotation against the other.
                        num = cn / (rp > 0.f ? S.lamf[p] : S.lamf[q]);
                        den = rp > 0.f ? -1.f : 1.f;
                    } else {
                        num = 0.f;
                        den = 1.f;
                    }
                    if (num != 0.f) th = den == 0.f ? copysignf(0.78539816f, num) : 0.5f * atanf(2.f * num / den);
                    thmax = fmaxf(thmax, fabsf(th));
                }
            }
            th = __shfl_sync(0xffffffffu, th, lane & ~3);
            if (has) {
                const float2 ek = make_float2(static_cast<float>(e), th);
                for (int r = q4; r < kRefCTAs; r += 4) {
                    cl.map_shared_rank(S.E, r)[q * kRefLd + p] = e;
                    cl.map_shared_rank(EK, r)[q * kRefLd + p] = ek;
                }
            }
        }
        ref_block_max3f(offmax, emax, thmax, S.redf);
        if (tid < kRefCTAs) {
            float* mr = cl.map_shared_rank(S.maxima, tid);
            mr[3 * rank] = offmax;
            mr[3 * rank + 1] = emax;
            mr[3 * rank + 2] = thmax;
        }
        cl.sync();
        float goff = 0.f, gem = 0.f, gth = 0.f;
        for (int r = 0; r < kRefCTAs; ++r) {
            goff = fmaxf(goff, S.maxima[3 * r]);
            gem = fmaxf(gem, S.maxima[3 * r + 1]);
            gth = fmaxf(gth, S.maxima[3 * r + 2]);
        }
        // Converged at 8 eps; or, once below the one-sided Jacobi's skip
        // threshold n eps, as soon as a step no longer shrinks the coupling by
        // 4x (the Gram sums' rounding floor).
        const float nf = static_cast<float>(n);
        if ((goff <= 8.f * feps && gem <= 8.f * feps) ||
            (goff <= nf * feps && gem <= nf * feps && goff > 0.25f * prev_off)) {
            converged = true;
            break;
        }
        prev_off = goff;
        if (steps == kRefMaxSteps) break;

        // (c) The large angles (above 1e-4 in the first two steps, where the
        // FP32 stage leaves them, 1e-6 later, where exact rotations settle the
        // last clusters of close singular values) in a fixed order (column q,
        // then row p): counts per column, their offsets, then the entries (one
        // warp per column). Skipped when no angle is that large.
        const float big = steps < 2 ? kRefBigAngle : kRefBigAngleLate;
        int nbig = 0;
        if (gth > big) {
            for (int q = warp; q < n; q += nw) {
                int cnt = 0;
                for (int p0 = 0; p0 < q; p0 += 32) {
                    const int p = p0 + lane;
                    cnt += __popc(__ballot_sync(0xffffffffu, p < q && fabsf(EK[q * kRefLd + p].y) > big));
                }
                if (lane == 0) S.big_cnt[q] = cnt;
            }
            __syncthreads();
            if (warp == 0) {
                const int c0 = lane < n ? S.big_cnt[lane] : 0;
                const int c1 = lane + 32 < n ? S.big_cnt[lane + 32] : 0;
                int s0 = c0, s1 = c1;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t0 = __shfl_up_sync(0xffffffffu, s0, o), t1 = __shfl_up_sync(0xffffffffu, s1, o);
                    if (lane >= o) {
                        s0 += t0;
                        s1 += t1;
                    }
                }
                const int tot0 = __shfl_sync(0xffffffffu, s0, 31), tot1 = __shfl_sync(0xffffffffu, s1, 31);
                __syncwarp();
                if (lane < n) S.big_cnt[lane] = s0 - c0;
                if (lane + 32 < n) S.big_cnt[lane + 32] = tot0 + s1 - c1;
                if (lane == 0) S.nbig = tot0 + tot1 < kRefMaxBig ? tot0 + tot1 : kRefMaxBig;
            }
            __syncthreads();
            for (int q = warp; q < n; q += nw) {
                int base = S.big_cnt[q];
                for (int p0 = 0; p0 < q; p0 += 32) {
                    const int p = p0 + lane;
                    const bool isbig = p < q && fabsf(EK[q * kRefLd + p].y) > big;
                    const unsigned m = __ballot_sync(0xffffffffu, isbig);
                    const int slot = base + __popc(m & ((1u << lane) - 1u));
                    if (isbig && slot < kRefMaxBig) {
                        S.big_p[slot] = static_cast<unsigned char>(p);
                        S.big_q[slot] = static_cast<unsigned char>(q);
                    }
                    base += __popc(m);
                }
            }
            __syncthreads();
            nbig = S.nbig;
            // Cosines and sines of the large angles: FP32 sincos, then scaled to
            // c^2 + s^2 = 1 in FP64 ((1 + d)^(-1/2) to second order in d ~ 1e-7).
            for (int b = tid; b < nbig; b += blockDim.x) {
                float s32, c32;
                sincosf(EK[S.big_q[b] * kRefLd + S.big_p[b]].y, &s32, &c32);
                const double c = c32, s = s32;
                const double d = fma(c, c, fma(s, s, -1.0));
                const double f = fma(0.375 * d, d, fma(-0.5, d, 1.0));
                S.big_c[b] = c * f;
                S.big_s[b] = s * f;
            }
            __syncthreads();
        }
        // The full E (symmetric) and K (skew, large angles removed) in FP32:
        // each thread completes one pair (p < q) or a diagonal entry.
        for (int e = tid; e < n * (n + 1) / 2; e += blockDim.x) {
            // e -> (p, q) with p <= q, column by column.
            int q = static_cast<int>((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
            while (q * (q + 1) / 2 > e) --q;
            while ((q + 1) * (q + 2) / 2 <= e) ++q;
            const int p = e - q * (q + 1) / 2;
            float2 v = EK[q * kRefLd + p];
            if (p == q || fabsf(v.y) > big) v.y = 0.f;
            EK[q * kRefLd + p] = v;
            if (p != q) EK[p * kRefLd + q] = make_float2(v.x, -v.y);
        }
        __syncthreads();

        // (d) D[:, own] = -E/2 + K + 3/8 E^2 + 1/2 K^2 - 1/2 E K (second order in
        // FP32), then X[:, q] += X D[:, q] for the own columns, into every CTA.
        for (int e = tid; e < nown * n; e += blockDim.x) {
            const int o = e / n, p = e % n, q = own_q[o];
            float ee = 0, kk = 0, ek = 0;
            for (int r = 0; r < n; ++r) {
                const float2 pr = EK[r * kRefLd + p], rq = EK[q * kRefLd + r];
                ee = fmaf(pr.x, rq.x, ee);
                kk = fmaf(pr.y, rq.y, kk);
                ek = fmaf(pr.x, rq.y, ek);
            }
            const double first = -0.5 * (p <= q ? S.E[q * kRefLd + p] : S.E[p * kRefLd + q]) +
                                 static_cast<double>(EK[q * kRefLd + p].y);
            S.u.s2.D32[o * kRefLd + p] = static_cast<float>(first) + (0.375f * ee + 0.5f * kk - 0.5f * ek);
        }
        __syncthreads();
        for (int e = tid; e < nown * n; e += blockDim.x) {
            const int o = e / n, i = e % n, q = own_q[o];
            float acc = 0;
            const float* d = S.u.s2.D32 + o * kRefLd;
            for (int p = 0; p < n; ++p) acc = fmaf(S.u.s2.X32[p * kRefLd + i], d[p], acc);
            const double xn = S.X[q * kRefLd + i] + static_cast<double>(acc);
            for (int r = 0; r < kRefCTAs; ++r) cl.map_shared_rank(S.X, r)[q * kRefLd + i] = xn;
        }
        cl.sync();
        // (e) The exact rotations on this CTA's full copy of X: thread i rotates
        // row i through the whole list (x_p <- c x_p - s x_q, x_q <- s x_p + c x_q).
        if (tid < n) {
            for (int b = 0; b < nbig; ++b) {
                const int p = S.big_p[b], q = S.big_q[b];
                const double c = S.big_c[b], sn = S.big_s[b];
                const double xv = S.X[p * kRefLd + tid], yv = S.X[q * kRefLd + tid];
                S.X[p * kRefLd + tid] = c * xv - sn * yv;
                S.X[q * kRefLd + tid] = sn * xv + c * yv;
            }
        }
        __syncthreads();
    }

    if (converged) {
        // Singular values |G[:, j]| = sqrt(C_jj), their reciprocals and their
        // order (every CTA; the order compares bit patterns, ties by index).
        for (int j = tid; j < n; j += blockDim.x) {
            const double sj = sqrt(S.lam[j]);
            S.norms[j] = sj;
            S.pairs[j] = 1.0 / sj;
        }
        __syncthreads();
        for (int j = tid; j < n; j += blockDim.x) {
            const long long sj = __double_as_longlong(S.norms[j]);
            int r = 0;
            for (int i = 0; i < n; ++i) {
                const long long si = __double_as_longlong(S.norms[i]);
                if (si > sj || (si == sj && i < j)) ++r;
            }
            S.order[r] = j;
            S.rankof[j] = r;
        }
        __syncthreads();
        const double zero_tol = S.norms[S.order[0]] * 2.220446049250313e-16 * static_cast<double>(n);
        if (S.norms[S.order[n - 1]] > zero_tol) {
            // The own columns: V = X, U = G / sigma, the largest-magnitude entry
            // of each V column (first on ties) made positive.
            if (warp < nown) {
                const int j = own_q[warp], jj = S.rankof[j];
                const double* x = S.X + j * kRefLd;
                unsigned long long best = 0;
                int arg = n;
                for (int i = lane; i < n; i += 32) {
                    const unsigned long long av = abs_bits(x[i]);
                    if (arg == n || av > best) {
                        best = av;
                        arg = i;
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
                    if (oa < n && (arg == n || ob > best || (ob == best && oa < arg))) {
                        best = ob;
                        arg = oa;
                    }
                }
                const bool neg = arg < n && x[arg] < 0.0;
                const double sj = S.norms[j];
                const double invs = neg ? -S.pairs[j] : S.pairs[j];
                if (lane == 0) {
                    a.BS[jj] = sj;
                    cl.map_shared_rank(S.invsg, 0)[j] = invs;
                }
                for (int i = lane; i < n; i += 32) {
                    a.BV[static_cast<int64_t>(jj) * n + i] = neg ? -x[i] : x[i];
                    a.BU[static_cast<int64_t>(jj) * n + i] = S.G[j * kRefLd + i] * invs;
                }
            }
            // Every CTA's columns are in global memory, and their factors in
            // CTA 0, before CTA 0's tail.
            cl.sync();
            if (rank != 0) return;
            refine_tail(a, S, steps);
            return;
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
