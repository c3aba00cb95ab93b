// Segment dot products of the sparse gathers, shared by the SpMV kernels and the
// batched solver: groups of G lanes reduce one compressed row (a "segment")
// with 16-byte vector loads of values and indices (packed u16 offsets into a
// staged x, or int32 columns of a global x) and a fixed-order shuffle tree.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace irlba_gb300 {

// Vector widths of one 16-byte value load: 4 FP32 or 2 FP64 values, with the
// matching packed u16 panel offsets (8 or 4 bytes) or int32 columns.
template <typename VT>
struct VecTraits;
template <>
struct VecTraits<float> {
    static constexpr int N = 4;
    typedef float4 V;
    typedef uint2 I16;
    typedef int4 I32;
};
template <>
struct VecTraits<double> {
    static constexpr int N = 2;
    typedef double2 V;
    typedef unsigned int I16;
    typedef int2 I32;
};

template <typename T, bool STAGED>
struct Gather {
    const T* xs;              // staged panel (shared memory)
    const T* __restrict__ x;  // global vector when not staged
    __device__ __forceinline__ T operator()(int64_t j) const { return STAGED ? xs[j] : __ldg(x + j); }
};

// acc += sum_v val[v] * x[idx[v]] over one vector of entries, one FMA per
// entry (a separate product sum would cost an extra add per pair on GB300's
// narrow FP64 pipe).
template <typename T, bool STAGED>
__device__ __forceinline__ void vec_acc(T& acc, const float4& v, const uint2& i, const Gather<T, STAGED>& g) {
    acc += static_cast<T>(v.x) * g(i.x & 0xffffu);
    acc += static_cast<T>(v.y) * g(i.x >> 16);
    acc += static_cast<T>(v.z) * g(i.y & 0xffffu);
    acc += static_cast<T>(v.w) * g(i.y >> 16);
}
template <typename T, bool STAGED>
__device__ __forceinline__ void vec_acc(T& acc, const float4& v, const int4& i, const Gather<T, STAGED>& g) {
    acc += static_cast<T>(v.x) * g(i.x);
    acc += static_cast<T>(v.y) * g(i.y);
    acc += static_cast<T>(v.z) * g(i.z);
    acc += static_cast<T>(v.w) * g(i.w);
}
template <typename T, bool STAGED>
__device__ __forceinline__ void vec_acc(T& acc, const double2& v, const unsigned int& i, const Gather<T, STAGED>& g) {
    acc += static_cast<T>(v.x) * g(i & 0xffffu);
    acc += static_cast<T>(v.y) * g(i >> 16);
}
template <typename T, bool STAGED>
__device__ __forceinline__ void vec_acc(T& acc, const double2& v, const int2& i, const Gather<T, STAGED>& g) {
    acc += static_cast<T>(v.x) * g(i.x);
    acc += static_cast<T>(v.y) * g(i.y);
}

// One lane's share of the segment [b, en) for a group of G lanes (glane =
// lane within the group): a scalar head up to the first 16-byte boundary of
// the value array, a body of vector loads (up to four per lane, all issued
// before use), and a scalar tail. The order of the partial sums is fixed.
template <typename VT, typename T, bool STAGED, int G>
__device__ __forceinline__ T segment_dot(const VT* __restrict__ val, const void* idxp, const Gather<T, STAGED>& g,
                                         int64_t b, int64_t en, int glane) {
    typedef VecTraits<VT> VTr;
    constexpr int N = VTr::N;
    typedef typename VTr::V V;
    typedef typename std::conditional<STAGED, typename VTr::I16, typename VTr::I32>::type IV;
    typedef typename std::conditional<STAGED, uint16_t, int32_t>::type IS;
    const IS* __restrict__ idx = static_cast<const IS*>(idxp);
    T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    const int64_t head = min(en, (b + (N - 1)) & ~static_cast<int64_t>(N - 1));
    if (glane < head - b) {
        const int64_t i = b + glane;
        a0 += static_cast<T>(ld_stream(val + i)) * g(ld_stream(idx + i));
    }
    const int64_t q1 = en / N;
    int64_t q = head / N + glane;
    const V* __restrict__ v4 = reinterpret_cast<const V*>(val);
    const IV* __restrict__ i4 = reinterpret_cast<const IV*>(idx);
    for (; q < q1; q += 4 * G) {
        V va = {}, vb = {}, vc = {}, vd = {};
        IV ia = {}, ib = {}, ic = {}, id = {};
        const bool hb = q + G < q1, hc = q + 2 * G < q1, hd = q + 3 * G < q1;
        va = ld_stream(v4 + q);
        ia = ld_stream(i4 + q);
        if (hb) {
            vb = ld_stream(v4 + q + G);
            ib = ld_stream(i4 + q + G);
        }
        if (hc) {
            vc = ld_stream(v4 + q + 2 * G);
            ic = ld_stream(i4 + q + 2 * G);
        }
        if (hd) {
            vd = ld_stream(v4 + q + 3 * G);
            id = ld_stream(i4 + q + 3 * G);
        }
        // FP64 accumulation (GB300's narrow FP64 pipe): two accumulators, so
        // combining them costs one add; FP32: four independent chains.
        constexpr bool kTwo = std::is_same<T, double>::value;
        vec_acc<T, STAGED>(a0, va, ia, g);
        if (hb) vec_acc<T, STAGED>(a1, vb, ib, g);
        if (hc) vec_acc<T, STAGED>(kTwo ? a0 : a2, vc, ic, g);
        if (hd) vec_acc<T, STAGED>(kTwo ? a1 : a3, vd, id, g);
    }
    const int64_t t0 = max(head, q1 * N);
    if (glane < en - t0) {
        const int64_t i = t0 + glane;
        (std::is_same<T, double>::value ? a1 : a2) += static_cast<T>(ld_stream(val + i)) * g(ld_stream(idx + i));
    }
    if constexpr (std::is_same<T, double>::value) return a0 + a1;
    else return (a0 + a1) + (a2 + a3);
}

// The same for dictionary-coded values: entry i's value is dict[code[i]]
// (exact: the dictionary holds the stored FP32 values), with u16 codes and u16
// panel offsets, so one 16-byte vector carries eight entries (4 bytes per
// entry instead of 6). dict and xs are in shared memory.
__device__ __forceinline__ void coded_acc(float& acc, const uint4& c, const uint4& i, const float* dict,
                                          const float* xs) {
    acc += dict[c.x & 0xffffu] * xs[i.x & 0xffffu];
    acc += dict[c.x >> 16] * xs[i.x >> 16];
    acc += dict[c.y & 0xffffu] * xs[i.y & 0xffffu];
    acc += dict[c.y >> 16] * xs[i.y >> 16];
    acc += dict[c.z & 0xffffu] * xs[i.z & 0xffffu];
    acc += dict[c.z >> 16] * xs[i.z >> 16];
    acc += dict[c.w & 0xffffu] * xs[i.w & 0xffffu];
    acc += dict[c.w >> 16] * xs[i.w >> 16];
}

// U vectors per lane in flight per iteration (2 or 4).
template <int G, int U>
__device__ __forceinline__ float segment_dot_coded(const uint16_t* __restrict__ code, const uint16_t* __restrict__ idx,
                                                   const float* dict, const float* xs, int64_t b, int64_t en,
                                                   int glane) {
    constexpr int N = 8;
    float a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) a[u] = 0.0f;
    const int64_t head = min(en, (b + (N - 1)) & ~static_cast<int64_t>(N - 1));
    for (int64_t i = b + glane; i < head; i += G) a[0] += dict[ld_stream(code + i)] * xs[ld_stream(idx + i)];
    const int64_t q1 = en / N;
    int64_t q = head / N + glane;
    const uint4* __restrict__ c4 = reinterpret_cast<const uint4*>(code);
    const uint4* __restrict__ i4 = reinterpret_cast<const uint4*>(idx);
    for (; q < q1; q += U * G) {
        uint4 c[U], ix[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            c[u] = make_uint4(0, 0, 0, 0);
            ix[u] = make_uint4(0, 0, 0, 0);
            if (u == 0 || q + u * G < q1) {
                c[u] = ld_stream(c4 + q + u * G);
                ix[u] = ld_stream(i4 + q + u * G);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (u == 0 || q + u * G < q1) coded_acc(a[u], c[u], ix[u], dict, xs);
    }
    const int64_t t0 = max(head, q1 * N);
    for (int64_t i = t0 + glane; i < en; i += G) a[U - 1] += dict[ld_stream(code + i)] * xs[ld_stream(idx + i)];
    float r = 0.0f;
#pragma unroll
    for (int u = 0; u < U; ++u) r += a[u];
    return r;
}

template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace irlba_gb300
