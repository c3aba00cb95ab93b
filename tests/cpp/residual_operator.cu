// A user-defined residual matrix R = A - X B^T for the device-operator path of
// the engine (irlba_gb300_matrix_create_device_operator): the kind of matrix a
// caller never stores, e.g. log-expression values with fitted covariate
// effects regressed out. A is an engine sparse matrix whose products come from
// irlba_gb300_spmv_device; X (m x r) and B (n x r) are column-major device
// arrays; the low-rank correction runs in this file's own kernels:
//   R x   = A x   - X (B^T x)
//   R^T y = A^T y - B (X^T y)
// Built by tests/test_gpu_operator.py with nvcc and loaded through ctypes.
#include <cstdint>

#include <cuda_runtime.h>

#include "irlba_gb300.h"

struct Residual {
    const irlba_gb300_matrix* A;
    int64_t m, n, r;
    const void* X;  // m x r
    const void* B;  // n x r
    void* t;        // r entries of scratch
    int32_t f32;    // vectors and factors are float (FP32 form) instead of double
};

// t[j] = sum_i P[i, j] x[i]: one block per column j.
template <typename T>
__global__ void contract_kernel(const T* P, int64_t L, const T* x, T* t) {
    __shared__ double red[256];
    const int64_t j = blockIdx.x;
    double acc = 0;
    for (int64_t i = threadIdx.x; i < L; i += blockDim.x) acc += static_cast<double>(P[j * L + i]) * x[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w /= 2) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) t[j] = static_cast<T>(red[0]);
}

// y[i] -= sum_j Q[i, j] t[j].
template <typename T>
__global__ void expand_kernel(const T* Q, int64_t L, int64_t r, const T* t, T* y) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < L;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        T acc = 0;
        for (int64_t j = 0; j < r; ++j) acc += Q[j * L + i] * t[j];
        y[i] -= acc;
    }
}

template <typename T>
static int32_t residual_run(const Residual& R, bool adjoint, const void* x, void* y, cudaStream_t s) {
    const T* P = static_cast<const T*>(adjoint ? R.X : R.B);  // contracted with the input
    const T* Q = static_cast<const T*>(adjoint ? R.B : R.X);  // expanded into the output
    const int64_t lin = adjoint ? R.m : R.n, lout = adjoint ? R.n : R.m;
    T* t = static_cast<T*>(R.t);
    if (R.r > 0) {
        contract_kernel<T><<<static_cast<unsigned>(R.r), 256, 0, s>>>(P, lin, static_cast<const T*>(x), t);
        const int64_t grid = (lout + 255) / 256;
        expand_kernel<T><<<static_cast<unsigned>(grid < 1024 ? (grid > 0 ? grid : 1) : 1024), 256, 0, s>>>(
            Q, lout, R.r, t, static_cast<T*>(y));
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

extern "C" int32_t residual_product(void* user, int32_t adjoint, const void* x, void* y, void* stream) {
    const Residual& R = *static_cast<const Residual*>(user);
    // A x (or A^T y) first: the correction is subtracted from it in place.
    if (irlba_gb300_spmv_device(R.A, adjoint, x, y, stream) != IRLBA_GB300_OK) return 2;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return R.f32 ? residual_run<float>(R, adjoint != 0, x, y, s) : residual_run<double>(R, adjoint != 0, x, y, s);
}
