// Shared device-side definitions of the GB300 IRLBA engine.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>

namespace irlba_gb300 {

// Host-side count of kernel launches issued by this library.
extern std::atomic<int64_t> g_launch_count;
inline void count_launch(int64_t n = 1) { g_launch_count.fetch_add(n, std::memory_order_relaxed); }

// Device control block: scalars of the Lanczos recurrence, flags read by the
// host once per restart, and the tickets of the last-block reductions.
struct Ctrl {
    double S;            // alpha: norm of the latest W column before normalization
    double R_F;          // beta: norm of the latest residual F
    double norm_F;       // ||F|| after the last reorthogonalization of a run
    double beta_mul;     // centring scalar of the next multiply  (x' . c)
    double beta_adj;     // centring scalar of the next adjoint   (sum y')
    double eps;          // invariant-subspace tolerance
    double tmp[4];
    int32_t abort;       // nonzero: skip all remaining work of this restart
    int32_t invariant;   // a norm fell below eps (fast mode) -> host re-runs carefully
    int32_t null_start;  // starting vector near the null space
    int32_t converged;   // set by the restart kernel
    int32_t n_converged;
    int32_t k_next;
    int32_t svd_sweeps;
    int32_t svd_not_converged;
    uint32_t ticket[16]; // last-block reduction counters (reset by the last block)
};

enum TicketSlot {
    kTicketDot = 0,
    kTicketUpdate = 1,
    kTicketNormalize = 2,
    kTicketBeta = 3,
    kTicketStats = 4,
    kTicketMisc = 5,
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum in a fixed order (deterministic). `red` holds >= 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0;
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = (lane < nw) ? red[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;  // valid in warp 0
}

// Last-block election: every block calls this after writing its partials; the
// one block that returns true sees all partials (after the fence) and must reset
// the ticket when done.
__device__ __forceinline__ bool last_block(uint32_t* ticket, bool* flag_smem) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t t = atomicAdd(ticket, 1u);
        *flag_smem = (t == gridDim.x * gridDim.y * gridDim.z - 1);
    }
    __syncthreads();
    if (*flag_smem) __threadfence();
    return *flag_smem;
}

template <typename T>
__device__ __forceinline__ T ld_stream(const T* p) {
    return __ldcs(p);
}

}  // namespace irlba_gb300
