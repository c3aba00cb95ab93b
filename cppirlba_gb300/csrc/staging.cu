// Large copies between pageable host memory and the device through a pool of
// pinned staging buffers.
//
// cudaMemcpy from or to pageable memory runs at 5-25 GB/s on a Grace host:
// the driver stages it through its own small pinned buffer one piece at a
// time. Here up to eight host threads each own two pinned slices; a thread
// copies its share of the host range slice by slice (host memcpy, in parallel
// across threads) and moves each slice with cudaMemcpyAsync on the caller's
// stream, double-buffered on per-slice events. The DMA engine runs at ~200 GB/s
// from pinned memory, so the copy is bound by the host threads' memcpy.
//
// Semantics match the plain calls they replace: host->device returns once the
// source range has been read (the DMAs stay queued on the stream, behind its
// earlier work); device->host returns with the data in the destination. Copies
// smaller than the threshold, and copies whose host side is already pinned or
// device-accessible, go straight to cudaMemcpyAsync.
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

#include "host.hpp"

namespace irlba_gb300 {

namespace {

constexpr int kMaxStagingWorkers = 8;

struct StagingLane {
    void* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

struct StagingPool {
    std::mutex mu;
    size_t slice = 0;  // bytes per staging buffer of the allocated lanes
    std::vector<StagingLane> lanes;

    void release() {
        for (auto& l : lanes)
            for (int b = 0; b < 2; ++b) {
                if (l.ev[b]) {
                    cudaEventSynchronize(l.ev[b]);  // no DMA still reads or writes the buffer
                    cudaEventDestroy(l.ev[b]);
                }
                if (l.buf[b]) cudaFreeHost(l.buf[b]);
            }
        lanes.clear();
        slice = 0;
    }
    // Lanes of `bytes` per buffer on the current device (called with mu held).
    cudaError_t ensure(int workers, size_t bytes) {
        if (slice != bytes) release();
        while (static_cast<int>(lanes.size()) < workers) {
            StagingLane l;
            for (int b = 0; b < 2; ++b) {
                cudaError_t e = cudaHostAlloc(&l.buf[b], bytes, cudaHostAllocPortable);
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.ev[b], cudaEventDisableTiming);
                if (e != cudaSuccess) {
                    for (int c = 0; c <= b; ++c) {
                        if (l.ev[c]) cudaEventDestroy(l.ev[c]);
                        if (l.buf[c]) cudaFreeHost(l.buf[c]);
                    }
                    return e;
                }
            }
            lanes.push_back(l);
        }
        slice = bytes;
        return cudaSuccess;
    }
};

std::atomic<int64_t> g_staged_min{16ll << 20};   // below this: plain cudaMemcpyAsync; < 0: never staged
std::atomic<int64_t> g_staged_slice{8ll << 20};  // bytes per staging buffer

StagingPool& pool_of(int device) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<StagingPool>> pools;
    std::lock_guard<std::mutex> g(mu);
    auto& p = pools[device];
    if (!p) p.reset(new StagingPool());
    return *p;
}

bool host_side_is_pageable(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

}  // namespace

cudaError_t copy_staged(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    const int64_t min_bytes = g_staged_min.load();
    const bool h2d = kind == cudaMemcpyHostToDevice;
    if (bytes == 0) return cudaSuccess;
    if (min_bytes < 0 || static_cast<int64_t>(bytes) < min_bytes || (!h2d && kind != cudaMemcpyDeviceToHost) ||
        !host_side_is_pageable(h2d ? src : dst))
        return cudaMemcpyAsync(dst, src, bytes, kind, s);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const size_t slice = static_cast<size_t>(std::max<int64_t>(g_staged_slice.load(), 4096));
    const size_t nslices = (bytes + slice - 1) / slice;
    const int workers = static_cast<int>(std::min<size_t>(
        std::min(host_threads(), kMaxStagingWorkers), nslices));
    StagingPool& pool = pool_of(dev);
    std::lock_guard<std::mutex> g(pool.mu);
    e = pool.ensure(workers, slice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cudaMemcpyAsync(dst, src, bytes, kind, s);  // no pinned memory to spare: the plain copy
    }
    std::atomic<int> failed{0};
    std::vector<cudaError_t> errs(workers, cudaSuccess);
    auto run = [&](int t) {
        cudaError_t err = cudaSetDevice(dev);
        StagingLane& L = pool.lanes[t];
        auto range = [&](size_t i, size_t& off, size_t& len) {
            off = i * slice;
            len = std::min(slice, bytes - off);
        };
        size_t off = 0, len = 0;
        if (h2d) {
            int b = 0;
            for (size_t i = t; i < nslices && err == cudaSuccess && !failed.load(); i += workers) {
                range(i, off, len);
                err = cudaEventSynchronize(L.ev[b]);  // the buffer's previous DMA has finished
                if (err != cudaSuccess) break;
                std::memcpy(L.buf[b], static_cast<const char*>(src) + off, len);
                err = cudaMemcpyAsync(static_cast<char*>(dst) + off, L.buf[b], len, kind, s);
                if (err == cudaSuccess) err = cudaEventRecord(L.ev[b], s);
                b ^= 1;
            }
        } else {
            auto issue = [&](size_t i, int b) {
                size_t o, n;
                range(i, o, n);
                cudaError_t r = cudaMemcpyAsync(L.buf[b], static_cast<const char*>(src) + o, n, kind, s);
                if (r == cudaSuccess) r = cudaEventRecord(L.ev[b], s);
                return r;
            };
            size_t i = t;
            int b = 0;
            if (i < nslices && err == cudaSuccess) err = issue(i, b);
            while (i < nslices && err == cudaSuccess && !failed.load()) {
                const size_t next = i + workers;
                if (next < nslices) err = issue(next, b ^ 1);  // the other buffer was drained last pass
                if (err == cudaSuccess) err = cudaEventSynchronize(L.ev[b]);
                if (err != cudaSuccess) break;
                range(i, off, len);
                std::memcpy(static_cast<char*>(dst) + off, L.buf[b], len);
                i = next;
                b ^= 1;
            }
            // Leave no DMA in flight into a buffer the next copy may reuse.
            for (int c = 0; c < 2; ++c) cudaEventSynchronize(L.ev[c]);
        }
        if (err != cudaSuccess) {
            errs[t] = err;
            failed.store(1);
        }
    };
    if (workers <= 1) {
        run(0);
    } else {
        std::vector<std::thread> threads;
        for (int t = 0; t < workers; ++t) threads.emplace_back(run, t);
        for (auto& th : threads) th.join();
    }
    for (cudaError_t r : errs)
        if (r != cudaSuccess) return r;
    return cudaSuccess;
}

}  // namespace irlba_gb300

extern "C" void irlba_gb300_set_staging(int64_t min_bytes, int64_t slice_bytes) {
    irlba_gb300::g_staged_min.store(min_bytes);
    if (slice_bytes > 0) irlba_gb300::g_staged_slice.store(slice_bytes);
}
