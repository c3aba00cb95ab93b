// Host-side helpers shared by the single-problem engine and the batched form:
// error reporting of the C ABI, counted host<->device copies, device buffers,
// per-device configuration, host thread pools and the host random normals.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/irlba_gb300.h"
#include "kernels.cuh"

namespace irlba_gb300 {

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
extern thread_local std::string g_last_error;

struct Error : public std::runtime_error {
    irlba_gb300_status status;
    Error(irlba_gb300_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define CUDA_TRY(expr)                                                                                  \
    do {                                                                                                \
        cudaError_t err__ = (expr);                                                                     \
        if (err__ != cudaSuccess)                                                                       \
            throw irlba_gb300::Error(IRLBA_GB300_ERROR_CUDA,                                            \
                                     std::string(#expr) + ": " + cudaGetErrorString(err__));            \
    } while (0)

[[noreturn]] inline void invalid(const std::string& m) { throw Error(IRLBA_GB300_ERROR_INVALID_ARGUMENT, m); }

// Runs f, mapping exceptions to a status code and the thread's last error.
template <typename F>
inline irlba_gb300_status guarded(F f) {
    try {
        f();
        return IRLBA_GB300_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return IRLBA_GB300_ERROR_CUDA;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return IRLBA_GB300_ERROR_INVALID_ARGUMENT;
    }
}

// ---------------------------------------------------------------------------
// Host<->device traffic issued by this library (bytes), for end-to-end accounting.
// ---------------------------------------------------------------------------
extern std::atomic<int64_t> g_h2d_bytes;
extern std::atomic<int64_t> g_d2h_bytes;

// Copies between host memory and the device (staging.cu): large copies of
// pageable host memory go through pinned staging buffers filled by several
// host threads; everything else is a plain cudaMemcpyAsync on `s`.
cudaError_t copy_staged(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s);

inline cudaError_t h2d_async(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    g_h2d_bytes.fetch_add(static_cast<int64_t>(bytes));
    return copy_staged(dst, src, bytes, cudaMemcpyHostToDevice, s);
}
inline cudaError_t d2h_async(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    g_d2h_bytes.fetch_add(static_cast<int64_t>(bytes));
    return copy_staged(dst, src, bytes, cudaMemcpyDeviceToHost, s);
}
// Synchronous forms, ordered on the default stream like cudaMemcpy.
inline cudaError_t h2d_sync(void* dst, const void* src, size_t bytes) {
    g_h2d_bytes.fetch_add(static_cast<int64_t>(bytes));
    const cudaError_t e = copy_staged(dst, src, bytes, cudaMemcpyHostToDevice, 0);
    return e != cudaSuccess ? e : cudaStreamSynchronize(0);
}
inline cudaError_t d2h_sync(void* dst, const void* src, size_t bytes) {
    g_d2h_bytes.fetch_add(static_cast<int64_t>(bytes));
    const cudaError_t e = copy_staged(dst, src, bytes, cudaMemcpyDeviceToHost, 0);
    return e != cudaSuccess ? e : cudaStreamSynchronize(0);
}

// ---------------------------------------------------------------------------
// Device memory
// ---------------------------------------------------------------------------
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() {}
    explicit DevBuf(size_t b) { alloc(b); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), bytes(o.bytes) { o.ptr = nullptr; o.bytes = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        release();
        ptr = o.ptr;
        bytes = o.bytes;
        o.ptr = nullptr;
        o.bytes = 0;
        return *this;
    }
    void alloc(size_t b) {
        release();
        bytes = b;
        if (b) CUDA_TRY(cudaMalloc(&ptr, b));
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    ~DevBuf() { release(); }
    template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

template <typename T>
inline DevBuf upload(const T* host, size_t n) {
    DevBuf b(sizeof(T) * n);
    if (n) CUDA_TRY(h2d_sync(b.ptr, host, sizeof(T) * n));
    return b;
}

inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// Device properties, configured once per device and host thread
// ---------------------------------------------------------------------------
struct DeviceInfo {
    int device = -1;
    int sms = 0;
    size_t max_smem_optin = 0;
};
DeviceInfo& device_info();

// IRLBA_GB300_TRACE=1 prints the set-up and ingestion steps to stderr.
inline bool trace_on() {
    static const bool on = [] {
        const char* e = std::getenv("IRLBA_GB300_TRACE");
        return e && e[0] == '1';
    }();
    return on;
}
#define TRACE(...)                                              \
    do {                                                        \
        if (irlba_gb300::trace_on()) {                          \
            std::fprintf(stderr, "[irlba_gb300] " __VA_ARGS__); \
            std::fprintf(stderr, "\n");                         \
            std::fflush(stderr);                                \
        }                                                       \
    } while (0)

// ---------------------------------------------------------------------------
// Host thread pools
// ---------------------------------------------------------------------------
inline int host_threads() {
    unsigned n = std::thread::hardware_concurrency();
    return n == 0 ? 1 : static_cast<int>(std::min(n, 64u));
}

template <typename F>
inline void parallel_chunks(int64_t n, F f) {
    const int nt = static_cast<int>(std::min<int64_t>(host_threads(), std::max<int64_t>(1, n / 4096)));
    if (nt <= 1) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) {
        const int64_t b = n * t / nt, e = n * (t + 1) / nt;
        pool.emplace_back([=, &f]() { f(b, e, t); });
    }
    for (auto& th : pool) th.join();
}

// Rows [0, R) split into one contiguous range per host thread, balanced by the
// number of nonzeros (ptr has R + 1 entries).
template <typename F>
inline void parallel_rows(const int64_t* ptr, int64_t R, F f) {
    const int64_t nnz = ptr[R];
    const int nt = static_cast<int>(std::min<int64_t>(host_threads(), std::max<int64_t>(1, (nnz + R) / 65536)));
    if (nt <= 1 || R < 2) {
        f(0, R, 0);
        return;
    }
    std::vector<int64_t> bounds(nt + 1, 0);
    bounds[nt] = R;
    int64_t r = 0;
    for (int t = 1; t < nt; ++t) {
        const int64_t target = (nnz + R) * t / nt;
        while (r < R && ptr[r] + r < target) ++r;
        bounds[t] = r;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back([=, &f]() { f(bounds[t], bounds[t + 1], t); });
    for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------
// Host random normals: std::mt19937_64 with Box-Muller pairs on 53-bit uniforms
// (stands in for aarand::standard_normal; fill order as utils.hpp:16-37).
// ---------------------------------------------------------------------------
inline double uniform01(std::mt19937_64& eng) {
    return (static_cast<double>(eng() >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

inline void fill_normals(std::vector<double>& v, std::mt19937_64& eng) {
    const int64_t n = static_cast<int64_t>(v.size());
    int64_t total = n;
    const bool odd = total % 2;
    if (odd) --total;
    auto pair = [&](double& a, double& b) {
        const double u1 = uniform01(eng), u2 = uniform01(eng);
        const double r = std::sqrt(-2.0 * std::log(u1));
        const double th = 6.283185307179586476925286766559 * u2;
        a = r * std::cos(th);
        b = r * std::sin(th);
    };
    for (int64_t i = 0; i < total; i += 2) pair(v[i], v[i + 1]);
    if (odd) {
        double a, b;
        pair(a, b);
        v[total] = a;
    }
}

}  // namespace irlba_gb300
