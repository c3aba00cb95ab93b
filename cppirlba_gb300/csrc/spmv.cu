// Sparse matrix-vector products of the IRLBA loop (the multiply / adjoint
// multiply of CppIrlba's ParallelSparseMatrix, Matrix/sparse.hpp:185-267, with
// the deferred centring and scaling of Matrix/centered.hpp:46-52,83-87 and
// Matrix/scaled.hpp:52-69,106-123 fused into the prologue and epilogue).
//
// Both directions are gathers over a "panel CSR" (see DirPlanDev): each CTA owns
// a contiguous, nnz-balanced range of segments; groups of G lanes (G = 4..32 by
// the plan's average segment length) take whole segments from a shared counter
// and reduce them with 16-byte vector loads of values and packed panel offsets
// and a shuffle tree, so every output is computed in a fixed order
// (bit-reproducible run to run). The x panel is staged in shared memory.

#include "kernels.cuh"
#include "segdot.cuh"

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

// G lanes per segment (32 / G segments per warp), chosen per plan from the
// average segment length so that short rows share the per-segment bookkeeping.
template <typename VT, typename T, bool STAGED, int G, int TH = kSpmvThreads, int MINB = 1>
__global__ void __launch_bounds__(TH, MINB) spmv_kernel(const DirPlanDev p, const T* __restrict__ x,
                                                            T* __restrict__ y, T* __restrict__ partial,
                                                            const Epilogue<T> e, const int32_t* abort) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);
    __shared__ unsigned int seg_counter;
    if (*abort) return;
    constexpr int kGroups = 32 / G;

    EpiVals<T> ev;
    ev.beta = e.beta ? static_cast<T>(*e.beta) : T(0);
    ev.alpha = e.alpha ? static_cast<T>(*e.alpha) : T(0);

    const VT* __restrict__ val = static_cast<const VT*>(p.val);
    const void* idxp = STAGED ? static_cast<const void*>(p.idx16) : static_cast<const void*>(p.idx32);
    Gather<T, STAGED> g;
    g.xs = xs;
    g.x = x;
    const int64_t sb = p.block_seg[blockIdx.x];
    const int64_t se = p.block_seg[blockIdx.x + 1];
    const int lane = threadIdx.x & 31;
    const int group = lane / G, glane = lane % G;

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

        // Warps take kGroups whole segments at a time from the counter; the
        // next batch's bounds are fetched before the current one streams.
        const unsigned int nhere = static_cast<unsigned int>(pe - s);
        unsigned int base = 0;
        if (lane == 0) base = atomicAdd(&seg_counter, static_cast<unsigned int>(kGroups));
        base = __shfl_sync(0xffffffffu, base, 0);
        int64_t b = 0, en = 0;
        if (base + group < nhere) {
            b = p.segptr[s + base + group];
            en = p.segptr[s + base + group + 1];
        }
        while (base < nhere) {
            unsigned int next = 0;
            if (lane == 0) next = atomicAdd(&seg_counter, static_cast<unsigned int>(kGroups));
            next = __shfl_sync(0xffffffffu, next, 0);
            int64_t nb = 0, nen = 0;
            if (next + group < nhere) {
                nb = p.segptr[s + next + group];
                nen = p.segptr[s + next + group + 1];
            }
            const unsigned int mine = base + group;
            T acc = 0;
            if (mine < nhere) acc = segment_dot<VT, T, STAGED, G>(val, idxp, g, b, en, glane);
            acc = group_sum<G>(acc);
            if (glane == 0 && mine < nhere) {
                const int64_t row = s + mine - panel * p.nrows;
                if (p.npanels == 1) y[row] = apply_epilogue(acc, row, e, ev);
                else partial[panel * p.nrows + row] = acc;
            }
            base = next;
            b = nb;
            en = nen;
        }
        s = pe;
    }
}

// The FP32 staged gather over dictionary-coded values (DirPlanDev::code):
// the dictionary is staged in shared memory behind the x panel once per CTA,
// then the same segment walk as spmv_kernel with 8-entry vectors.
template <int G, int TH, int MINB, int U>
__global__ void __launch_bounds__(TH, MINB) spmv_coded_kernel(const DirPlanDev p, const float* __restrict__ x,
                                                                float* __restrict__ y, float* __restrict__ partial,
                                                                const Epilogue<float> e, const int32_t* abort) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* xs = reinterpret_cast<float*>(smem_raw);
    float* ds = xs + p.dict_offset;
    __shared__ unsigned int seg_counter;
    if (*abort) return;
    constexpr int kGroups = 32 / G;

    EpiVals<float> ev;
    ev.beta = e.beta ? static_cast<float>(*e.beta) : 0.0f;
    ev.alpha = e.alpha ? static_cast<float>(*e.alpha) : 0.0f;
    for (int i = threadIdx.x; i < p.ndict; i += blockDim.x) ds[i] = p.dict[i];

    const int64_t sb = p.block_seg[blockIdx.x];
    const int64_t se = p.block_seg[blockIdx.x + 1];
    const int lane = threadIdx.x & 31;
    const int group = lane / G, glane = lane % G;

    int64_t s = sb;
    while (s < se) {
        const int64_t panel = s / p.nrows;
        const int64_t pe = min(se, (panel + 1) * p.nrows);
        __syncthreads();
        {
            const int64_t c0 = panel * p.panel_width;
            const int64_t w = min(p.panel_width, p.ncols - c0);
            for (int64_t i = threadIdx.x; i < w; i += blockDim.x) {
                float xv = x[c0 + i];
                if (e.iscale) xv = e.idivide ? xv / e.iscale[c0 + i] : xv * e.iscale[c0 + i];
                xs[i] = xv;
            }
        }
        if (threadIdx.x == 0) seg_counter = 0;
        __syncthreads();

        const unsigned int nhere = static_cast<unsigned int>(pe - s);
        unsigned int base = 0;
        if (lane == 0) base = atomicAdd(&seg_counter, static_cast<unsigned int>(kGroups));
        base = __shfl_sync(0xffffffffu, base, 0);
        int64_t b = 0, en = 0;
        if (base + group < nhere) {
            b = p.segptr[s + base + group];
            en = p.segptr[s + base + group + 1];
        }
        while (base < nhere) {
            unsigned int next = 0;
            if (lane == 0) next = atomicAdd(&seg_counter, static_cast<unsigned int>(kGroups));
            next = __shfl_sync(0xffffffffu, next, 0);
            int64_t nb = 0, nen = 0;
            if (next + group < nhere) {
                nb = p.segptr[s + next + group];
                nen = p.segptr[s + next + group + 1];
            }
            const unsigned int mine = base + group;
            float acc = 0;
            if (mine < nhere) acc = segment_dot_coded<G, U>(p.code, p.idx16, ds, xs, b, en, glane);
            acc = group_sum<G>(acc);
            if (glane == 0 && mine < nhere) {
                const int64_t row = s + mine - panel * p.nrows;
                if (p.npanels == 1) y[row] = apply_epilogue(acc, row, e, ev);
                else partial[panel * p.nrows + row] = acc;
            }
            base = next;
            b = nb;
            en = nen;
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

// The epilogue alone, in place, over the raw product of a user-defined operator.
template <typename T>
__global__ void epilogue_kernel(T* y, int64_t nrows, const Epilogue<T> e, const int32_t* abort) {
    if (*abort) return;
    EpiVals<T> ev;
    ev.beta = e.beta ? static_cast<T>(*e.beta) : T(0);
    ev.alpha = e.alpha ? static_cast<T>(*e.alpha) : T(0);
    for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r < nrows;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        y[r] = apply_epilogue(y[r], r, e, ev);
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

// Calls f with the kernel instantiation for (value type, vector type, staged,
// group lanes, launch shape). Launch shapes (FP32 staged plans with FP32
// vectors; the others use shape 0): 0 = 256 threads; 1 = 256 threads,
// registers capped for six CTAs per SM; 2 = 512 threads, registers capped for
// three CTAs per SM.
template <typename T, typename F>
static void with_spmv_kernel(bool vf64, bool staged, int group, F f, int shape = 0) {
#define IRLBA_SPMV_G(VT, ST, TH, MB)                                    \
    switch (group) {                                                    \
        case 4: f(spmv_kernel<VT, T, ST, 4, TH, MB>); break;            \
        case 8: f(spmv_kernel<VT, T, ST, 8, TH, MB>); break;            \
        case 16: f(spmv_kernel<VT, T, ST, 16, TH, MB>); break;          \
        default: f(spmv_kernel<VT, T, ST, 32, TH, MB>); break;          \
    }
    if (vf64) {
        if (staged) { IRLBA_SPMV_G(double, true, 256, 1) } else { IRLBA_SPMV_G(double, false, 256, 1) }
    } else if (!staged || !std::is_same<T, float>::value || shape == 0) {
        if (staged) { IRLBA_SPMV_G(float, true, 256, 1) } else { IRLBA_SPMV_G(float, false, 256, 1) }
    } else if (shape == 1) {
        IRLBA_SPMV_G(float, true, 256, 6)
    } else {
        IRLBA_SPMV_G(float, true, 512, 3)
    }
#undef IRLBA_SPMV_G
}

// Calls f with the coded-value kernel for (group lanes, launch shape).
template <typename F>
static void with_coded_kernel(int group, F f, int shape) {
#define IRLBA_SPMV_C(TH, MB, U)                                  \
    switch (group) {                                             \
        case 4: f(spmv_coded_kernel<4, TH, MB, U>); break;       \
        case 8: f(spmv_coded_kernel<8, TH, MB, U>); break;       \
        case 16: f(spmv_coded_kernel<16, TH, MB, U>); break;     \
        default: f(spmv_coded_kernel<32, TH, MB, U>); break;     \
    }
    // The coded loop holds eight entries per vector: two vectors in flight per
    // lane keep the three-per-SM shapes within their 40 registers.
    if (shape == 1) {
        IRLBA_SPMV_C(256, 6, 2)
    } else if (shape == 2) {
        IRLBA_SPMV_C(512, 3, 2)
    } else {
        IRLBA_SPMV_C(256, 1, 4)
    }
#undef IRLBA_SPMV_C
}

int spmv_shape_threads(int shape) { return shape == 2 ? 512 : 256; }

template <typename T>
void launch_spmv(const DirPlanDev& p, const T* x, T* y, T* partial, const Epilogue<T>& e, const int32_t* abort,
                 cudaStream_t stream) {
    if (p.nrows == 0) return;
    if (p.nblocks > 0) {
        const size_t smem = p.staged ? p.smem_bytes : 0;
        const int th = spmv_shape_threads(p.shape);
        bool coded = false;
        if constexpr (std::is_same<T, float>::value) {
            if (p.code) {
                with_coded_kernel(p.group_lanes, [&](auto kernel) {
                    kernel<<<p.nblocks, th, smem, stream>>>(p, x, y, partial, e, abort);
                }, p.shape);
                coded = true;
            }
        }
        if (!coded)
            with_spmv_kernel<T>(p.val_f64 != 0, p.staged != 0, p.group_lanes, [&](auto kernel) {
                kernel<<<p.nblocks, th, smem, stream>>>(p, x, y, partial, e, abort);
            }, p.shape);
        count_launch();
    }
    if (p.npanels > 1) {
        panel_reduce_kernel<T><<<grid_for(p.nrows, 256, 152 * 16), 256, 0, stream>>>(partial, p.npanels, p.nrows, y, e,
                                                                                   abort);
        count_launch();
    }
}

template <typename T>
void launch_epilogue(T* y, int64_t nrows, const Epilogue<T>& e, const int32_t* abort, cudaStream_t stream) {
    if (nrows == 0) return;
    if (!e.beta && !e.oscale && !e.alpha) return;
    epilogue_kernel<T><<<grid_for(nrows, 256, 152 * 16), 256, 0, stream>>>(y, nrows, e, abort);
    count_launch();
}

template <typename T>
void launch_scale_vector(const T* x, const T* s, int32_t divide, int64_t n, T* out, cudaStream_t stream) {
    if (n == 0) return;
    scale_vector_kernel<T><<<grid_for(n, 256, 152 * 16), 256, 0, stream>>>(x, s, divide, n, out);
    count_launch();
}

// Raise the dynamic shared-memory limit of the staged kernels (once per device).
cudaError_t spmv_configure(size_t max_smem) {
    cudaError_t err = cudaSuccess;
    auto set = [&](auto kernel) {
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(max_smem));
    };
    auto set_coded = [&](auto kernel) {
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(max_smem + sizeof(float) * (kMaxDict + 4)));
    };
    for (int g = 4; g <= 32; g *= 2) {
        for (int shape = 0; shape <= 2; ++shape) with_coded_kernel(g, set_coded, shape);
        with_spmv_kernel<float>(false, true, g, set);
        with_spmv_kernel<float>(false, true, g, set, 1);
        with_spmv_kernel<float>(false, true, g, set, 2);
        with_spmv_kernel<float>(true, true, g, set);
        with_spmv_kernel<double>(false, true, g, set);
        with_spmv_kernel<double>(true, true, g, set);
    }
    return err;
}

int spmv_blocks_per_sm(bool staged, bool vf64, bool tf64, size_t smem, int group, int shape, bool coded) {
    int nb = 0;
    const int th = spmv_shape_threads(shape);
    auto occ = [&](auto kernel) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, th, staged ? smem : 0);
    };
    if (coded) {
        with_coded_kernel(group, occ, shape);
        return nb < 1 ? 1 : nb;
    }
    if (tf64) with_spmv_kernel<double>(vf64, staged, group, occ, shape);
    else with_spmv_kernel<float>(vf64, staged, group, occ, shape);
    return nb < 1 ? 1 : nb;
}

template void launch_spmv<float>(const DirPlanDev&, const float*, float*, float*, const Epilogue<float>&,
                                 const int32_t*, cudaStream_t);
template void launch_spmv<double>(const DirPlanDev&, const double*, double*, double*, const Epilogue<double>&,
                                  const int32_t*, cudaStream_t);
template void launch_epilogue<float>(float*, int64_t, const Epilogue<float>&, const int32_t*, cudaStream_t);
template void launch_epilogue<double>(double*, int64_t, const Epilogue<double>&, const int32_t*, cudaStream_t);
template void launch_scale_vector<float>(const float*, const float*, int32_t, int64_t, float*, cudaStream_t);
template void launch_scale_vector<double>(const double*, const double*, int32_t, int64_t, double*, cudaStream_t);

}  // namespace irlba_gb300
