// Sparse matrix-vector products of the IRLBA loop (the multiply / adjoint
// multiply of CppIrlba's ParallelSparseMatrix, Matrix/sparse.hpp:185-267, with
// the deferred centring and scaling of Matrix/centered.hpp:46-52,83-87 and
// Matrix/scaled.hpp:52-69,106-123 fused into the prologue and epilogue).
//
// Both directions are gathers over a "panel CSR" (see DirPlanDev): each CTA owns
// a contiguous, nnz-balanced range of segments; warps take whole segments from a
// shared counter and reduce them with lane-strided, 4-way unrolled streaming
// loads and a warp-shuffle tree, so every output is computed in a fixed order
// (bit-reproducible run to run). The x panel is staged in shared memory.

#include "kernels.cuh"

namespace irlba_gb300 {

namespace {

template <typename T>
struct EpiVals {
    T beta;
    T alpha;
};

template <typename T>
__device__ __forceinline__ T apply_epilogue(T v, int64_t r, const Epilogue<T>& e, const EpiVals<T>& ev) {
    if (e.beta && !e.center_after) v -= ev.beta * (e.cvec ? e.cvec[r] : T(1));
    if (e.oscale) v = e.odivide ? v / e.oscale[r] : v * e.oscale[r];
    if (e.beta && e.center_after) v -= ev.beta * (e.cvec ? e.cvec[r] : T(1));
    if (e.alpha) v -= ev.alpha * e.q[r];
    return v;
}

template <typename VT, typename T, bool STAGED>
__global__ void __launch_bounds__(kSpmvThreads) spmv_kernel(const DirPlanDev p, const T* __restrict__ x,
                                                            T* __restrict__ y, T* __restrict__ partial,
                                                            const Epilogue<T> e, const int32_t* abort) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);
    __shared__ unsigned int seg_counter;
    if (*abort) return;

    EpiVals<T> ev;
    ev.beta = e.beta ? static_cast<T>(*e.beta) : T(0);
    ev.alpha = e.alpha ? static_cast<T>(*e.alpha) : T(0);

    const VT* __restrict__ val = static_cast<const VT*>(p.val);
    const int64_t sb = p.block_seg[blockIdx.x];
    const int64_t se = p.block_seg[blockIdx.x + 1];
    const int lane = threadIdx.x & 31;

    int64_t s = sb;
    while (s < se) {
        const int64_t panel = s / p.nrows;
        const int64_t pe = min(se, (panel + 1) * p.nrows);
        __syncthreads();
        if (STAGED) {
            const int64_t c0 = panel * p.panel_width;
            const int64_t w = min(p.panel_width, p.ncols - c0);
            for (int64_t i = threadIdx.x; i < w; i += blockDim.x) {
                T xv = x[c0 + i];
                if (e.iscale) xv = e.idivide ? xv / e.iscale[c0 + i] : xv * e.iscale[c0 + i];
                xs[i] = xv;
            }
        }
        if (threadIdx.x == 0) seg_counter = 0;
        __syncthreads();

        const unsigned int nhere = static_cast<unsigned int>(pe - s);
        while (true) {
            unsigned int mine = 0;
            if (lane == 0) mine = atomicAdd(&seg_counter, 1u);
            mine = __shfl_sync(0xffffffffu, mine, 0);
            if (mine >= nhere) break;
            const int64_t seg = s + mine;
            const int64_t row = seg - panel * p.nrows;
            const int64_t b = p.segptr[seg];
            const int64_t en = p.segptr[seg + 1];
            T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
            int64_t i = b + lane;
            if (STAGED) {
                const uint16_t* __restrict__ idx = p.idx16;
                for (; i + 96 < en; i += 128) {
                    const VT v0 = ld_stream(val + i), v1 = ld_stream(val + i + 32);
                    const VT v2 = ld_stream(val + i + 64), v3 = ld_stream(val + i + 96);
                    const uint16_t j0 = ld_stream(idx + i), j1 = ld_stream(idx + i + 32);
                    const uint16_t j2 = ld_stream(idx + i + 64), j3 = ld_stream(idx + i + 96);
                    a0 += static_cast<T>(v0) * xs[j0];
                    a1 += static_cast<T>(v1) * xs[j1];
                    a2 += static_cast<T>(v2) * xs[j2];
                    a3 += static_cast<T>(v3) * xs[j3];
                }
                for (; i < en; i += 32) a0 += static_cast<T>(ld_stream(val + i)) * xs[ld_stream(idx + i)];
            } else {
                const int32_t* __restrict__ idx = p.idx32;
                for (; i + 96 < en; i += 128) {
                    const VT v0 = ld_stream(val + i), v1 = ld_stream(val + i + 32);
                    const VT v2 = ld_stream(val + i + 64), v3 = ld_stream(val + i + 96);
                    const int32_t j0 = ld_stream(idx + i), j1 = ld_stream(idx + i + 32);
                    const int32_t j2 = ld_stream(idx + i + 64), j3 = ld_stream(idx + i + 96);
                    a0 += static_cast<T>(v0) * __ldg(x + j0);
                    a1 += static_cast<T>(v1) * __ldg(x + j1);
                    a2 += static_cast<T>(v2) * __ldg(x + j2);
                    a3 += static_cast<T>(v3) * __ldg(x + j3);
                }
                for (; i < en; i += 32) a0 += static_cast<T>(ld_stream(val + i)) * __ldg(x + ld_stream(idx + i));
            }
            T acc = (a0 + a1) + (a2 + a3);
            acc = warp_sum(acc);
            if (lane == 0) {
                if (p.npanels == 1) y[row] = apply_epilogue(acc, row, e, ev);
                else partial[panel * p.nrows + row] = acc;
            }
        }
        s = pe;
    }
}

template <typename T>
__global__ void panel_reduce_kernel(const T* __restrict__ partial, int32_t npanels, int64_t nrows, T* __restrict__ y,
                                    const Epilogue<T> e, const int32_t* abort) {
    if (*abort) return;
    EpiVals<T> ev;
    ev.beta = e.beta ? static_cast<T>(*e.beta) : T(0);
    ev.alpha = e.alpha ? static_cast<T>(*e.alpha) : T(0);
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < nrows;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        T acc = 0;
        for (int32_t pnl = 0; pnl < npanels; ++pnl) acc += partial[pnl * nrows + r];
        y[r] = apply_epilogue(acc, r, e, ev);
    }
}

template <typename T>
__global__ void scale_vector_kernel(const T* __restrict__ x, const T* __restrict__ s, int32_t divide, int64_t n,
                                    T* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = divide ? x[i] / s[i] : x[i] * s[i];
}

int grid_for(int64_t n, int threads, int cap) {
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return static_cast<int>(g);
}

}  // namespace

template <typename T>
void launch_spmv(const DirPlanDev& p, const T* x, T* y, T* partial, const Epilogue<T>& e, const int32_t* abort,
                 cudaStream_t stream) {
    if (p.nrows == 0) return;
    const bool vf64 = p.val_f64 != 0;
    if (p.nblocks > 0) {
        if (p.staged) {
            if (vf64) {
                spmv_kernel<double, T, true><<<p.nblocks, kSpmvThreads, p.smem_bytes, stream>>>(p, x, y, partial, e, abort); count_launch();
            } else {
                spmv_kernel<float, T, true><<<p.nblocks, kSpmvThreads, p.smem_bytes, stream>>>(p, x, y, partial, e, abort); count_launch();
            }
        } else {
            if (vf64) {
                spmv_kernel<double, T, false><<<p.nblocks, kSpmvThreads, 0, stream>>>(p, x, y, partial, e, abort); count_launch();
            } else {
                spmv_kernel<float, T, false><<<p.nblocks, kSpmvThreads, 0, stream>>>(p, x, y, partial, e, abort); count_launch();
            }
        }
    }
    if (p.npanels > 1) {
        panel_reduce_kernel<T><<<grid_for(p.nrows, 256, 152 * 16), 256, 0, stream>>>(partial, p.npanels, p.nrows, y, e,
                                                                                   abort); count_launch();
    }
}

template <typename T>
void launch_scale_vector(const T* x, const T* s, int32_t divide, int64_t n, T* out, cudaStream_t stream) {
    if (n == 0) return;
    scale_vector_kernel<T><<<grid_for(n, 256, 152 * 16), 256, 0, stream>>>(x, s, divide, n, out); count_launch();
}

// Raise the dynamic shared-memory limit of the staged kernels (once per device).
template <typename K>
static cudaError_t set_smem(K kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

cudaError_t spmv_configure(size_t max_smem) {
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = set_smem(spmv_kernel<float, float, true>, max_smem);
    if (e == cudaSuccess) e = set_smem(spmv_kernel<double, double, true>, max_smem);
    if (e == cudaSuccess) e = set_smem(spmv_kernel<float, double, true>, max_smem);
    if (e == cudaSuccess) e = set_smem(spmv_kernel<double, float, true>, max_smem);
    return e;
}

int spmv_blocks_per_sm(bool staged, bool vf64, bool tf64, size_t smem) {
    int nb = 0;
    if (staged) {
        if (tf64) {
            if (vf64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<double, double, true>, kSpmvThreads, smem);
            else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<float, double, true>, kSpmvThreads, smem);
        } else {
            if (vf64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<double, float, true>, kSpmvThreads, smem);
            else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<float, float, true>, kSpmvThreads, smem);
        }
    } else {
        if (tf64) {
            if (vf64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<double, double, false>, kSpmvThreads, 0);
            else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<float, double, false>, kSpmvThreads, 0);
        } else {
            if (vf64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<double, float, false>, kSpmvThreads, 0);
            else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spmv_kernel<float, float, false>, kSpmvThreads, 0);
        }
    }
    return nb < 1 ? 1 : nb;
}

template void launch_spmv<float>(const DirPlanDev&, const float*, float*, float*, const Epilogue<float>&,
                                 const int32_t*, cudaStream_t);
template void launch_spmv<double>(const DirPlanDev&, const double*, double*, double*, const Epilogue<double>&,
                                  const int32_t*, cudaStream_t);
template void launch_scale_vector<float>(const float*, const float*, int32_t, int64_t, float*, cudaStream_t);
template void launch_scale_vector<double>(const double*, const double*, int32_t, int64_t, double*, cudaStream_t);

}  // namespace irlba_gb300
