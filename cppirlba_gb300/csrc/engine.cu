// Host driver and C ABI of the GB300 IRLBA engine.
//
// The restart loop of CppIrlba's irlba::compute (compute.hpp:141-308) runs here
// with every vector and matrix resident on the device; the host issues the
// kernels of one restart, then reads a 100-byte control block once per restart
// (k for the next run, the convergence flag, error flags). Lanczos
// bidiagonalization (lanczos.hpp:54-143) is issued step by step on one stream.
// Invariant subspaces (lanczos.hpp:101-106,124-129) are handled by re-running a
// restart in a careful mode that synchronizes after each norm and draws the
// random refill from the host engine, in the reference's order.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include <dlfcn.h>
#include <cusolverDn.h>

#include "host.hpp"
#include "matrix.hpp"

namespace irlba_gb300 {

std::atomic<int64_t> g_launch_count{0};
thread_local std::string g_last_error;
std::atomic<int64_t> g_h2d_bytes{0};
std::atomic<int64_t> g_d2h_bytes{0};

// ---------------------------------------------------------------------------
// Device properties, configured once per device
// ---------------------------------------------------------------------------
// Shared-memory budget for a staged x panel.
constexpr size_t kPanelBytes = 64 * 1024;

DeviceInfo& device_info() {
    static thread_local DeviceInfo info;
    int dev = 0;
    TRACE("device_info: cudaGetDevice");
    CUDA_TRY(cudaGetDevice(&dev));
    if (info.device != dev) {
        cudaDeviceProp prop;
        TRACE("device_info: properties");
        CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
        info.device = dev;
        info.sms = prop.multiProcessorCount;
        info.max_smem_optin = prop.sharedMemPerBlockOptin;
        TRACE("device_info: %d SMs, smem opt-in %zu; spmv attributes", info.sms, info.max_smem_optin);
        CUDA_TRY(spmv_configure(kPanelBytes));
        TRACE("device_info: rotate attributes");
        CUDA_TRY(rotate_configure(sizeof(double) * 128 * 128));
        CUDA_TRY(rotate_tc_configure(info.max_smem_optin));
        TRACE("device_info: restart attributes");
        CUDA_TRY(restart_configure(info.max_smem_optin));
        TRACE("device_info: batch attributes");
        CUDA_TRY(batch_configure(info.max_smem_optin));
        CUDA_TRY(cudaGetLastError());
        TRACE("device_info: done");
    }
    return info;
}

// ---------------------------------------------------------------------------
// Host-side ingestion: compressed matrix -> panel CSR gather plans
// ---------------------------------------------------------------------------
// A compressed gather view on the host: rows x cols, ptr (rows+1), idx, val.
struct HostCompressed {
    int64_t rows = 0, cols = 0;
    const int64_t* ptr = nullptr;
    const int32_t* idx = nullptr;
    const void* val = nullptr;
    bool f64 = false;
    // Owned storage when produced by a transpose or a dense conversion.
    std::vector<int64_t> own_ptr;
    std::vector<int32_t> own_idx;
    std::vector<float> own_f32;
    std::vector<double> own_f64;
};

static double value_at(const HostCompressed& h, int64_t s) {
    return h.f64 ? static_cast<const double*>(h.val)[s] : static_cast<double>(static_cast<const float*>(h.val)[s]);
}

// Transpose (counting sort by column, stable in row order), multithreaded.
static void transpose_host(const HostCompressed& in, HostCompressed& out) {
    const int64_t R = in.rows, C = in.cols;
    const int64_t nnz = in.ptr[R];
    out.rows = C;
    out.cols = R;
    out.f64 = in.f64;
    out.own_ptr.assign(C + 1, 0);
    out.own_idx.resize(nnz);
    if (in.f64) out.own_f64.resize(nnz); else out.own_f32.resize(nnz);
    const int nt = static_cast<int>(std::min<int64_t>(host_threads(), std::max<int64_t>(1, nnz / 65536)));
    std::vector<std::vector<int64_t>> hist(nt, std::vector<int64_t>(C, 0));
    auto row_range = [&](int t, int64_t& b, int64_t& e) {
        b = R * t / nt;
        e = R * (t + 1) / nt;
    };
    {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&, t]() {
                int64_t b, e;
                row_range(t, b, e);
                auto& h = hist[t];
                for (int64_t s = in.ptr[b]; s < in.ptr[e]; ++s) ++h[in.idx[s]];
            });
        for (auto& th : pool) th.join();
    }
    // Column-major exclusive offsets: column c, thread t.
    int64_t run = 0;
    for (int64_t c = 0; c < C; ++c) {
        out.own_ptr[c] = run;
        for (int t = 0; t < nt; ++t) {
            const int64_t v = hist[t][c];
            hist[t][c] = run;
            run += v;
        }
    }
    out.own_ptr[C] = run;
    {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&, t]() {
                int64_t b, e;
                row_range(t, b, e);
                auto& h = hist[t];
                for (int64_t r = b; r < e; ++r)
                    for (int64_t s = in.ptr[r]; s < in.ptr[r + 1]; ++s) {
                        const int64_t dst = h[in.idx[s]]++;
                        out.own_idx[dst] = static_cast<int32_t>(r);
                        if (in.f64) out.own_f64[dst] = static_cast<const double*>(in.val)[s];
                        else out.own_f32[dst] = static_cast<const float*>(in.val)[s];
                    }
            });
        for (auto& th : pool) th.join();
    }
    out.ptr = out.own_ptr.data();
    out.idx = out.own_idx.data();
    out.val = in.f64 ? static_cast<const void*>(out.own_f64.data()) : static_cast<const void*>(out.own_f32.data());
}

// A device gather plan with the buffers it owns.

// Relative cost of a segment against one nonzero when balancing CTAs.
constexpr int64_t kSegCost = 8;

// Launch shape of the SpMV kernel for FP32 staged plans of matrices created
// from now on (see spmv_shape_threads): 2, 512-thread CTAs three per SM, is
// the default (the fastest measured on the 2,000 x 1.3M FP32 workload: more
// resident warps, more loads in flight); FP64 and unstaged plans use shape 0.
static int g_spmv_shape = 2;
static int plan_shape(bool staged, bool store_f64, bool x_f64) {
    return (staged && !store_f64 && !x_f64) ? g_spmv_shape : 0;
}

// Lanes per segment of the gather from the average segment length in 16-byte
// vectors. With FP64 vectors (FP64 accumulation) the per-segment FP64 work
// (combining a lane's partial sums, the shuffle tree, the epilogue) costs as
// much as the products on GB300's narrow FP64 pipe unless several segments
// share each warp instruction, so those groups stay at 4 lanes, or 8 for
// segments of 256 vectors and more (measured: 100-vector cell rows 4 lanes
// 13 % faster than 8, 800-vector gene panel segments 8 lanes 11 % faster
// than 4). FP32 groups take 32 lanes only for long segments (several
// hundred vectors); below that, 8 lanes and four segments per warp keep more
// loads in flight between the per-segment reductions (measured on the
// 2,000-gene single-cell matrices: 50 vectors per cell row, 8 lanes 10 %
// faster than 16; about 400 per gene panel segment, 32 lanes fastest).
static int plan_group_lanes(int64_t nnz, int64_t nseg, bool store_f64, bool x_f64) {
    const double avg = nseg > 0 ? static_cast<double>(nnz) / static_cast<double>(nseg) : 0.0;
    const double vecs = avg / (store_f64 ? 2.0 : 4.0);
    if (x_f64) return vecs >= 256 ? 8 : 4;
    return vecs >= 128 ? 32 : vecs >= 6 ? 8 : 4;
}

static void build_plan(const HostCompressed& h, bool store_f64, bool x_f64, DirPlan& plan) {
    TRACE("build_plan: %lld x %lld, nnz %lld", (long long)h.rows, (long long)h.cols, (long long)h.ptr[h.rows]);
    const DeviceInfo& di = device_info();
    DirPlanDev& d = plan.dev;
    d.nrows = h.rows;
    d.ncols = h.cols;
    d.nnz = h.ptr[h.rows];
    d.val_f64 = store_f64 ? 1 : 0;
    const size_t xbytes = x_f64 ? 8 : 4;
    const int64_t pw_max = static_cast<int64_t>(kPanelBytes / xbytes);
    int64_t npanels = 1;
    bool staged = true;
    int64_t pw = std::max<int64_t>(1, std::min<int64_t>(h.cols, pw_max));
    if (h.cols > pw_max) {
        npanels = (h.cols + pw_max - 1) / pw_max;
        const double avg = static_cast<double>(d.nnz) / (static_cast<double>(h.rows) * static_cast<double>(npanels));
        if (avg < 4.0 || npanels > (1 << 20)) {
            staged = false;
            npanels = 1;
        }
    }
    d.staged = staged ? 1 : 0;
    d.npanels = static_cast<int32_t>(npanels);
    d.panel_width = staged ? pw : h.cols;
    d.nseg = npanels * h.rows;

    const int64_t R = h.rows, nnz = d.nnz, nseg = d.nseg;
    std::vector<int64_t> segptr(nseg + 1, 0);
    std::vector<uint16_t> idx16;
    std::vector<int32_t> idx32;
    std::vector<float> v32;
    std::vector<double> v64;
    if (store_f64) v64.resize(nnz); else v32.resize(nnz);

    auto put_value = [&](int64_t dst, int64_t src) {
        if (store_f64) v64[dst] = value_at(h, src);
        else v32[dst] = h.f64 ? static_cast<float>(static_cast<const double*>(h.val)[src])
                              : static_cast<const float*>(h.val)[src];
    };

    if (!staged || npanels == 1) {
        for (int64_t r = 0; r <= R; ++r) segptr[r] = h.ptr[r];
        if (staged) idx16.resize(nnz); else idx32.resize(nnz);
        parallel_rows(h.ptr, R, [&](int64_t b, int64_t e, int) {
            for (int64_t s = h.ptr[b]; s < h.ptr[e]; ++s) {
                if (staged) idx16[s] = static_cast<uint16_t>(h.idx[s]);
                else idx32[s] = h.idx[s];
                put_value(s, s);
            }
        });
    } else {
        // Count entries per (panel, row) then lay segments out panel-major.
        std::vector<int64_t> cnt(nseg, 0);
        parallel_rows(h.ptr, R, [&](int64_t b, int64_t e, int) {
            for (int64_t r = b; r < e; ++r)
                for (int64_t s = h.ptr[r]; s < h.ptr[r + 1]; ++s) ++cnt[(h.idx[s] / pw) * R + r];
        });
        for (int64_t sg = 0; sg < nseg; ++sg) segptr[sg + 1] = segptr[sg] + cnt[sg];
        idx16.resize(nnz);
        parallel_rows(h.ptr, R, [&](int64_t b, int64_t e, int) {
            std::vector<int64_t> fill(npanels);
            for (int64_t r = b; r < e; ++r) {
                for (int64_t p = 0; p < npanels; ++p) fill[p] = segptr[p * R + r];
                for (int64_t s = h.ptr[r]; s < h.ptr[r + 1]; ++s) {
                    const int64_t c = h.idx[s];
                    const int64_t p = c / pw;
                    const int64_t dst = fill[p]++;
                    idx16[dst] = static_cast<uint16_t>(c - p * pw);
                    put_value(dst, s);
                }
            }
        });
    }

    // Balance CTAs over segments by cost = nnz + kSegCost per segment.
    d.smem_bytes = staged ? static_cast<size_t>(d.panel_width) * xbytes : 0;
    TRACE("build_plan: occupancy query");
    d.group_lanes = plan_group_lanes(nnz, nseg, store_f64, x_f64);
    d.shape = plan_shape(staged, store_f64, x_f64);
    const int per_sm = spmv_blocks_per_sm(staged, store_f64, x_f64, d.smem_bytes, d.group_lanes, d.shape);
    TRACE("build_plan: %d blocks per SM", per_sm);
    int64_t nblocks = static_cast<int64_t>(di.sms) * per_sm;
    const int64_t total_cost = nnz + kSegCost * nseg;
    nblocks = std::max<int64_t>(1, std::min<int64_t>(nblocks, std::max<int64_t>(1, total_cost / 2048)));
    std::vector<int64_t> bseg(nblocks + 1, 0);
    {
        int64_t s = 0;
        for (int64_t b = 1; b < nblocks; ++b) {
            const int64_t target = total_cost * b / nblocks;
            while (s < nseg && segptr[s] + kSegCost * s < target) ++s;
            bseg[b] = s;
        }
        bseg[nblocks] = nseg;
    }
    d.nblocks = static_cast<int32_t>(nblocks);

    TRACE("build_plan: upload (%lld segments, %lld nnz, %lld blocks)", (long long)nseg, (long long)nnz, (long long)nblocks);
    plan.segptr = upload(segptr.data(), segptr.size());
    if (staged) plan.idx = upload(idx16.data(), idx16.size());
    else plan.idx = upload(idx32.data(), idx32.size());
    if (store_f64) plan.val = upload(v64.data(), v64.size());
    else plan.val = upload(v32.data(), v32.size());
    plan.block_seg = upload(bseg.data(), bseg.size());
    d.segptr = plan.segptr.as<int64_t>();
    d.idx16 = staged ? plan.idx.as<uint16_t>() : nullptr;
    d.idx32 = staged ? nullptr : plan.idx.as<int32_t>();
    d.val = plan.val.ptr;
    d.block_seg = plan.block_seg.as<int64_t>();
}

// ---------------------------------------------------------------------------
// Device-side ingestion: the same plans built on the GPU from the uploaded
// compressed arrays (ingest.cu). Rows must be sorted; pointers are checked on
// the host first, so every device read stays inside the uploaded arrays.
// ---------------------------------------------------------------------------
static bool g_device_ingest = true;

struct DevCompressed {
    int64_t rows = 0, cols = 0, nnz = 0;
    const int64_t* ptr = nullptr;
    const int32_t* idx = nullptr;
    const void* val = nullptr;
    bool f64 = false;
};

static void build_plan_device(const DevCompressed& h, bool store_f64, bool x_f64, DirPlan& plan, cudaStream_t s) {
    const DeviceInfo& di = device_info();
    DirPlanDev& d = plan.dev;
    d.nrows = h.rows;
    d.ncols = h.cols;
    d.nnz = h.nnz;
    d.val_f64 = store_f64 ? 1 : 0;
    const size_t xbytes = x_f64 ? 8 : 4;
    const int64_t pw_max = static_cast<int64_t>(kPanelBytes / xbytes);
    int64_t npanels = 1;
    bool staged = true;
    const int64_t pw = std::max<int64_t>(1, std::min<int64_t>(h.cols, pw_max));
    if (h.cols > pw_max) {
        npanels = (h.cols + pw_max - 1) / pw_max;
        const double avg = static_cast<double>(d.nnz) / (static_cast<double>(h.rows) * static_cast<double>(npanels));
        if (avg < 4.0 || npanels > (1 << 20)) {
            staged = false;
            npanels = 1;
        }
    }
    d.staged = staged ? 1 : 0;
    d.npanels = static_cast<int32_t>(npanels);
    d.panel_width = staged ? pw : h.cols;
    d.nseg = npanels * h.rows;
    const int64_t R = h.rows, nnz = d.nnz, nseg = d.nseg;
    plan.segptr.alloc(sizeof(int64_t) * (nseg + 1));
    plan.idx.alloc(std::max<size_t>((staged ? sizeof(uint16_t) : sizeof(int32_t)) * nnz, 16));
    plan.val.alloc(std::max<size_t>((store_f64 ? sizeof(double) : sizeof(float)) * nnz, 16));
    uint16_t* idx16 = staged ? plan.idx.as<uint16_t>() : nullptr;
    int32_t* idx32 = staged ? nullptr : plan.idx.as<int32_t>();
    if (!staged || npanels == 1) {
        CUDA_TRY(cudaMemcpyAsync(plan.segptr.ptr, h.ptr, sizeof(int64_t) * (R + 1), cudaMemcpyDeviceToDevice, s));
        launch_copy_entries(nnz, h.idx, h.val, h.f64, idx16, idx32, plan.val.ptr, store_f64, s);
    } else {
        DevBuf cnt(sizeof(int64_t) * std::max<int64_t>(nseg, 1)), scr(sizeof(int64_t) * scan_scratch_elems(nseg));
        launch_panel_count(R, static_cast<int32_t>(npanels), pw, h.ptr, h.idx, cnt.as<int64_t>(), s);
        launch_exclusive_scan(cnt.as<int64_t>(), nseg, plan.segptr.as<int64_t>(), plan.segptr.as<int64_t>() + nseg,
                              scr.as<int64_t>(), s);
        launch_panel_scatter(R, static_cast<int32_t>(npanels), pw, h.ptr, h.idx, h.val, h.f64,
                             plan.segptr.as<int64_t>(), idx16, plan.val.ptr, store_f64, s);
        CUDA_TRY(cudaStreamSynchronize(s));
    }
    d.smem_bytes = staged ? static_cast<size_t>(d.panel_width) * xbytes : 0;
    d.group_lanes = plan_group_lanes(nnz, nseg, store_f64, x_f64);
    d.shape = plan_shape(staged, store_f64, x_f64);
    const int per_sm = spmv_blocks_per_sm(staged, store_f64, x_f64, d.smem_bytes, d.group_lanes, d.shape);
    int64_t nblocks = static_cast<int64_t>(di.sms) * per_sm;
    const int64_t total_cost = nnz + kSegCost * nseg;
    nblocks = std::max<int64_t>(1, std::min<int64_t>(nblocks, std::max<int64_t>(1, total_cost / 2048)));
    plan.block_seg.alloc(sizeof(int64_t) * (nblocks + 1));
    launch_block_seg(plan.segptr.as<int64_t>(), nseg, kSegCost, nblocks, plan.block_seg.as<int64_t>(), s);
    d.nblocks = static_cast<int32_t>(nblocks);
    d.segptr = plan.segptr.as<int64_t>();
    d.idx16 = idx16;
    d.idx32 = idx32;
    d.val = plan.val.ptr;
    d.block_seg = plan.block_seg.as<int64_t>();
}

// ---------------------------------------------------------------------------
// Dictionary-coded values (off by default). The SpMV moves 6 bytes per FP32
// entry (value + u16 panel offset); matrices with at most kMaxDict distinct
// values (count data such as log1p-transformed single-cell counts have a few
// hundred) can store each value as a u16 code into a dictionary of the exact
// FP32 values, 4 bytes per entry, decoded from shared memory by the gather.
// Lossless: products see the stored values bit for bit. The raw values stay
// for the other kernels (statistics, realization, adjoint products). On the
// 2,000 x 1.3M bench matrix the coded gather moves a third fewer bytes but is
// no faster (multiply 0.280 vs 0.284 ms, adjoint 0.309 vs 0.283 ms): the
// dictionary lookup adds a shared-memory access per entry to a gather whose
// shared-memory x reads already bound it, so the plain layout stays the default.
// ---------------------------------------------------------------------------
static bool g_value_coding = false;
constexpr int kDictLog2Slots = 12;   // 4,096 hash slots for at most 2,048 values

static void encode_values(BaseMatrix& b, cudaStream_t s) {
    // FP32 vectors only (the FP64 form stages FP64 panels even for FP32 values).
    if (!g_value_coding || b.store_f64 || b.form != IRLBA_GB300_FORM_FP32_FP64STEPS) return;
    DirPlan* plans[2] = {&b.mul, &b.adj};
    for (DirPlan* p : plans)
        if (!p->dev.staged || p->dev.nnz == 0 || p->dev.val_f64) return;
    const int64_t nnz = b.mul.dev.nnz;
    const size_t nslots = size_t{1} << kDictLog2Slots;
    DevBuf slots(sizeof(unsigned long long) * nslots), flags(sizeof(uint32_t) * 2);
    CUDA_TRY(cudaMemsetAsync(slots.ptr, 0, slots.bytes, s));
    CUDA_TRY(cudaMemsetAsync(flags.ptr, 0, flags.bytes, s));
    uint32_t* count = flags.as<uint32_t>();
    int32_t* overflow = reinterpret_cast<int32_t*>(count + 1);
    launch_dict_insert(static_cast<const float*>(b.mul.dev.val), nnz, slots.as<unsigned long long>(), kDictLog2Slots,
                       count, overflow, static_cast<uint32_t>(kMaxDict), s);
    uint32_t hf[2] = {0, 0};
    CUDA_TRY(d2h_async(hf, flags.ptr, sizeof(hf), s));
    CUDA_TRY(cudaStreamSynchronize(s));
    if (hf[1] || hf[0] == 0 || hf[0] > static_cast<uint32_t>(kMaxDict)) return;
    const int32_t ndict = static_cast<int32_t>(hf[0]);
    DevBuf slot_code(sizeof(uint16_t) * nslots);
    b.dict.alloc(sizeof(float) * ndict);
    launch_dict_compact(slots.as<unsigned long long>(), kDictLog2Slots, slot_code.as<uint16_t>(), b.dict.as<float>(),
                        s);
    const DeviceInfo& di = device_info();
    for (DirPlan* p : plans) {
        DirPlanDev& d = p->dev;
        p->code.alloc(std::max<size_t>(sizeof(uint16_t) * d.nnz, 16));
        launch_dict_encode(static_cast<const float*>(d.val), d.nnz, slots.as<unsigned long long>(),
                           slot_code.as<uint16_t>(), kDictLog2Slots, p->code.as<uint16_t>(), s);
        d.code = p->code.as<uint16_t>();
        d.dict = b.dict.as<float>();
        d.ndict = ndict;
        d.dict_offset = static_cast<int32_t>((d.panel_width + 3) / 4 * 4);
        d.smem_bytes = sizeof(float) * (static_cast<size_t>(d.dict_offset) + static_cast<size_t>(ndict));
        // The coded kernel has its own occupancy: rebalance the CTA ranges for it.
        const int per_sm = spmv_blocks_per_sm(true, false, false, d.smem_bytes, d.group_lanes, d.shape, true);
        int64_t nblocks = static_cast<int64_t>(di.sms) * per_sm;
        const int64_t total_cost = d.nnz + kSegCost * d.nseg;
        nblocks = std::max<int64_t>(1, std::min<int64_t>(nblocks, std::max<int64_t>(1, total_cost / 2048)));
        p->block_seg.alloc(sizeof(int64_t) * (nblocks + 1));
        launch_block_seg(d.segptr, d.nseg, kSegCost, nblocks, p->block_seg.as<int64_t>(), s);
        d.nblocks = static_cast<int32_t>(nblocks);
        d.block_seg = p->block_seg.as<int64_t>();
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    CUDA_TRY(cudaGetLastError());
}

// Stable transpose of a device compressed matrix (entries of each output row
// in increasing input-row order); hptr: the input pointers on the host, for
// nnz-balanced chunks of input rows.
static void transpose_device(const DevCompressed& in, const int64_t* hptr, bool out_f64, DevBuf& tptr, DevBuf& tidx,
                             DevBuf& tval, cudaStream_t s) {
    const int64_t R = in.rows, C = in.cols, nnz = in.nnz;
    // Bytes of chunk counters (int32 counts + int64 cursors): up to 2 GiB or an
    // eighth of the free device memory; more chunks keep more SMs scattering.
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const int64_t budget = std::min<int64_t>(2ll << 30, static_cast<int64_t>(free_b / 8));
    int nchunks = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>({304, std::max<int64_t>(R, 1),
                                                                          budget / (12 * std::max<int64_t>(C, 1))})));
    std::vector<int64_t> chunk_rows(nchunks + 1, 0);
    for (int c = 1; c < nchunks; ++c) {
        const int64_t target = nnz * c / nchunks;
        chunk_rows[c] = std::lower_bound(hptr, hptr + R + 1, target) - hptr;
        chunk_rows[c] = std::max(chunk_rows[c], chunk_rows[c - 1]);
    }
    chunk_rows[nchunks] = R;
    DevBuf dchunks = upload(chunk_rows.data(), chunk_rows.size());
    tptr.alloc(sizeof(int64_t) * (C + 1));
    tidx.alloc(std::max<size_t>(sizeof(int32_t) * nnz, 16));
    tval.alloc(std::max<size_t>((out_f64 ? sizeof(double) : sizeof(float)) * nnz, 16));
    DevBuf count(sizeof(int32_t) * std::max<int64_t>(nchunks * C, 1)),
        cursor(sizeof(int64_t) * std::max<int64_t>(nchunks * C, 1)), scr(sizeof(int64_t) * scan_scratch_elems(C));
    CUDA_TRY(cudaMemsetAsync(count.ptr, 0, count.bytes, s));
    launch_transpose_count(in.ptr, in.idx, dchunks.as<int64_t>(), nchunks, C, count.as<int32_t>(), s);
    launch_transpose_totals(count.as<int32_t>(), nchunks, C, tptr.as<int64_t>(), s);
    launch_exclusive_scan(tptr.as<int64_t>(), C, tptr.as<int64_t>(), tptr.as<int64_t>() + C, scr.as<int64_t>(), s);
    launch_transpose_cursors(count.as<int32_t>(), nchunks, C, tptr.as<int64_t>(), cursor.as<int64_t>(), s);
    launch_transpose_scatter(in.ptr, in.idx, in.val, in.f64, dchunks.as<int64_t>(), nchunks, C,
                             cursor.as<int64_t>(), tidx.as<int32_t>(), tval.ptr, out_f64, s);
    CUDA_TRY(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// Matrix handles
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Optional per-kernel-class timing with CUDA events on the engine stream.
// ---------------------------------------------------------------------------
enum TimeClass { kTSpmvMul = 0, kTSpmvAdj, kTCgs, kTRestart, kTRotate, kTOther, kTNum };

struct Timer {
    bool on = false;
    cudaStream_t stream = nullptr;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    int64_t launches[kTNum] = {0};
    void begin(int cls, cudaEvent_t* out) {
        launches[cls]++;
        if (!on) return;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, stream);
        marks.push_back({cls, {a, b}});
        *out = b;
    }
    void end(cudaEvent_t e) {
        if (on) cudaEventRecord(e, stream);
    }
    void collect(double* ms) {
        for (int i = 0; i < kTNum; ++i) ms[i] = 0;
        for (auto& m : marks) {
            float t = 0;
            cudaEventElapsedTime(&t, m.second.first, m.second.second);
            ms[m.first] += t;
            cudaEventDestroy(m.second.first);
            cudaEventDestroy(m.second.second);
        }
        marks.clear();
    }
};

struct Scoped {
    Timer& t;
    cudaEvent_t e = nullptr;
    Scoped(Timer& tt, int cls) : t(tt) { t.begin(cls, &e); }
    ~Scoped() {
        if (e) t.end(e);
    }
};

static bool g_profile = false;
static double g_last_ms[kTNum] = {0};
static int64_t g_last_launches[kTNum] = {0};

// ---------------------------------------------------------------------------
// Engine: one compute() call
// ---------------------------------------------------------------------------

// Raw product of a user-defined operator: y = A x (adjoint = false) or A^T x.
// A device product is enqueued on `s`; a host product synchronizes `s`, runs on
// FP64 host copies of the vectors and copies y back before returning.
template <typename T>
static void operator_product(const BaseMatrix& A, bool adjoint, const T* x, T* y, cudaStream_t s) {
    const int64_t lin = adjoint ? A.nrow : A.ncol, lout = adjoint ? A.ncol : A.nrow;
    int32_t rc = 0;
    if (A.op.device) {
        rc = A.op.device(A.op.user, adjoint ? 1 : 0, x, y, s);
    } else {
        std::vector<T> xt(static_cast<size_t>(lin));
        CUDA_TRY(d2h_async(xt.data(), x, sizeof(T) * lin, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        std::vector<double> xd(xt.begin(), xt.end()), yd(static_cast<size_t>(lout), 0.0);
        rc = A.op.host(A.op.user, adjoint ? 1 : 0, xd.data(), yd.data());
        if (rc == 0) {
            std::vector<T> yt(yd.begin(), yd.end());
            CUDA_TRY(h2d_async(y, yt.data(), sizeof(T) * lout, s));
            CUDA_TRY(cudaStreamSynchronize(s));
        }
    }
    if (rc != 0) invalid("user-defined product failed (status " + std::to_string(rc) + ")");
}

static void gesvd_device(const double* A, int64_t mm, int64_t nn, double* U, double* S, double* V,
                         cudaStream_t stream);

template <typename T>
struct Engine {
    const Chain& ch;
    const BaseMatrix& A;
    cudaStream_t stream;
    int64_t m, n;        // rows, cols of the operator
    int64_t ldv, ldw;    // leading dims of V (n x work) and W (m x work)
    int work = 0;
    Timer timer;

    // Device buffers.
    DevBuf V, W, F, Wn, xtmp, partial, part, t, B, BU, BV, BS, prevS, res, svd_scratch, ctrl_buf;
    DevBuf center_d, scale_d;
    Ctrl* ctrl = nullptr;

    // FP32 form: the first product of the next Lanczos run, A'(F / ||F||) =
    // (A'F) / ||F||, is formed on a side stream while the restart kernel runs
    // (it needs F, not the small SVD). pre_ready: Wn holds A'F.
    cudaStream_t side = nullptr;
    cudaEvent_t ev_f = nullptr, ev_pre = nullptr;
    bool pre_ready = false;

    // Chain vectors in T precision.
    const T* cvec = nullptr;   // centre (length n)
    const T* svec = nullptr;   // scale (length n or m)

    Engine(const Chain& c, cudaStream_t s) : ch(c), A(*c.base), stream(s), m(c.base->nrow), n(c.base->ncol) {
        timer.stream = s;
        timer.on = g_profile;
    }
    ~Engine() {
        if (side) {
            cudaStreamSynchronize(side);
            cudaStreamDestroy(side);
        }
        if (ev_f) cudaEventDestroy(ev_f);
        if (ev_pre) cudaEventDestroy(ev_pre);
    }

    void upload_chain() {
        if (ch.center) {
            std::vector<T> tmp(ch.center->begin(), ch.center->end());
            center_d = upload(tmp.data(), tmp.size());
            cvec = center_d.as<T>();
        }
        if (ch.scale) {
            std::vector<T> tmp(ch.scale->begin(), ch.scale->end());
            scale_d = upload(tmp.data(), tmp.size());
            svec = scale_d.as<T>();
        }
    }

    void alloc_common() {
        ctrl_buf.alloc(sizeof(Ctrl));
        ctrl = ctrl_buf.as<Ctrl>();
        CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), stream));
        const int64_t Lmax = std::max(m, n);
        const int64_t pmax = std::max<int64_t>(A.mul.dev.npanels > 1 ? A.mul.dev.npanels * m : 0,
                                               A.adj.dev.npanels > 1 ? A.adj.dev.npanels * n : 0);
        partial.alloc(sizeof(T) * std::max<int64_t>(pmax, 1));
        xtmp.alloc(sizeof(T) * std::max<int64_t>(Lmax, 1));
        const int64_t wmax = std::max(work, 1);
        const int64_t part_sz = std::max<int64_t>(static_cast<int64_t>(cgs_dot_grid(Lmax)) * wmax,
                                                  static_cast<int64_t>(cgs_update_grid(Lmax))) + 64;
        part.alloc(sizeof(double) * part_sz);
        t.alloc(sizeof(double) * std::max<int64_t>(wmax, 1));
    }

    // ---- the fused matvecs ----------------------------------------------------
    // multiply: y (m) = Op x (n).  beta_mul must already hold the centring scalar.
    // st: the stream (NULL = the engine stream).
    void multiply(const T* x, T* y, const double* alpha, const T* q, cudaStream_t st = nullptr) {
        const cudaStream_t ms = st ? st : stream;
        // The per-class timer records on the engine stream: side-stream
        // products are left out of it (they overlap the restart kernel).
        Timer untimed;
        Scoped sc(st ? untimed : timer, kTSpmvMul);
        Epilogue<T> e;
        const bool col_scale = ch.scale && ch.scale_column;
        if (ch.center) {
            e.beta = &ctrl->beta_mul;
            e.center_after = ch.center_outer;
        }
        if (ch.scale && !ch.scale_column) {
            e.oscale = svec;
            e.odivide = ch.scale_divide;
        }
        e.alpha = alpha;
        e.q = q;
        const T* xin = x;
        if (A.is_operator()) {
            if (col_scale) {
                launch_scale_vector<T>(x, svec, ch.scale_divide, n, xtmp.as<T>(), ms);
                xin = xtmp.as<T>();
            }
            operator_product<T>(A, false, xin, y, ms);
            launch_epilogue<T>(y, m, e, &ctrl->abort, ms);
            return;
        }
        if (col_scale) {
            // FP32: scaled while staging. FP64: scaled once into xtmp (the same
            // division per entry), so the CTAs that stage the same panel do not
            // repeat it on the narrow FP64 pipe.
            if (A.mul.dev.staged && std::is_same<T, float>::value) {
                e.iscale = svec;
                e.idivide = ch.scale_divide;
            } else {
                launch_scale_vector<T>(x, svec, ch.scale_divide, n, xtmp.as<T>(), ms);
                xin = xtmp.as<T>();
            }
        }
        launch_spmv<T>(A.mul.dev, xin, y, partial.as<T>(), e, &ctrl->abort, ms);
    }

    // adjoint: y (n) = Op^T x (m).  beta_adj must already hold the centring scalar.
    void adjoint(const T* x, T* y, const double* alpha, const T* q) {
        Scoped sc(timer, kTSpmvAdj);
        Epilogue<T> e;
        const bool row_scale = ch.scale && !ch.scale_column;
        if (ch.center) {
            e.beta = &ctrl->beta_adj;
            e.cvec = cvec;
            e.center_after = ch.center_outer;
        }
        if (ch.scale && ch.scale_column) {
            e.oscale = svec;
            e.odivide = ch.scale_divide;
        }
        e.alpha = alpha;
        e.q = q;
        const T* xin = x;
        if (A.is_operator()) {
            if (row_scale) {
                launch_scale_vector<T>(x, svec, ch.scale_divide, m, xtmp.as<T>(), stream);
                xin = xtmp.as<T>();
            }
            operator_product<T>(A, true, xin, y, stream);
            launch_epilogue<T>(y, n, e, &ctrl->abort, stream);
            return;
        }
        if (row_scale) {
            if (A.adj.dev.staged && std::is_same<T, float>::value) {
                e.iscale = svec;
                e.idivide = ch.scale_divide;
            } else {
                launch_scale_vector<T>(x, svec, ch.scale_divide, m, xtmp.as<T>(), stream);
                xin = xtmp.as<T>();
            }
        }
        launch_spmv<T>(A.adj.dev, xin, y, partial.as<T>(), e, &ctrl->abort, stream);
    }

    // Scale/centre vectors that define the centring scalars.
    const T* beta_mul_fscale() const { return (ch.scale && ch.scale_column && !ch.center_outer) ? svec : nullptr; }
    const T* beta_adj_fscale() const { return (ch.scale && !ch.scale_column && !ch.center_outer) ? svec : nullptr; }

    void beta_mul_of(const T* x, cudaStream_t st = nullptr) {
        if (!ch.center) return;
        launch_beta<T>(x, n, beta_mul_fscale(), ch.scale_divide, cvec, &ctrl->beta_mul, part.as<double>(), ctrl,
                       st ? st : stream);
    }
    void beta_adj_of(const T* x) {
        if (!ch.center) return;
        launch_beta<T>(x, m, beta_adj_fscale(), ch.scale_divide, nullptr, &ctrl->beta_adj, part.as<double>(), ctrl,
                       stream);
    }

    // Reorthogonalize v against the first c columns of Q; norm -> *norm_out.
    void cgs(const T* Q, int64_t L, int64_t ldq, int c, T* v, double* norm_out, int check_eps, int check_null) {
        Scoped sc(timer, kTCgs);
        if (c > 0) launch_cgs_dot<T>(Q, L, ldq, c, v, part.as<double>(), t.as<double>(), ctrl, stream);
        launch_cgs_update<T>(Q, L, ldq, c, t.as<double>(), v, part.as<double>(), norm_out, check_eps, check_null,
                             ctrl, stream);
    }

    void normalize_F(int j) {
        Scoped sc(timer, kTOther);
        launch_normalize<T>(F.as<T>(), n, &ctrl->R_F, Vcol(j + 1), beta_mul_fscale(), ch.scale_divide,
                            ch.center ? cvec : nullptr, ch.center ? &ctrl->beta_mul : nullptr, part.as<double>(),
                            B.as<double>(), j + static_cast<int64_t>(j) * work, work, ctrl, stream);
    }
    void normalize_W(int j, const double* norm) {
        Scoped sc(timer, kTOther);
        launch_normalize<T>(Wn.as<T>(), m, norm, Wcol(j), beta_adj_fscale(), ch.scale_divide, nullptr,
                            ch.center ? &ctrl->beta_adj : nullptr, part.as<double>(), nullptr, -1, 0, ctrl, stream);
    }

    T* Vcol(int j) { return V.as<T>() + j * ldv; }
    T* Wcol(int j) { return W.as<T>() + j * ldw; }

    void sync_ctrl(Ctrl& h) {
        CUDA_TRY(d2h_async(&h, ctrl, sizeof(Ctrl), stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
    }
    void set_scalar(double* dptr, double v) {
        CUDA_TRY(h2d_async(dptr, &v, sizeof(double), stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
    }

    // Replace v (length L) by random normals from the host engine, then
    // orthogonalize against Q[:, :c] and normalize; the recurrence scalar at
    // *scalar becomes 0 (lanczos.hpp:101-106, 124-129).
    void refill(T* v, int64_t L, const T* Q, int64_t ldq, int c, std::mt19937_64& eng, double* scalar, bool is_F,
                int j) {
        std::vector<double> r(L);
        fill_normals(r, eng);
        std::vector<T> rt(r.begin(), r.end());
        CUDA_TRY(h2d_async(v, rt.data(), sizeof(T) * L, stream));
        cgs(Q, L, ldq, c, v, &ctrl->tmp[0], 0, 0);
        CUDA_TRY(cudaStreamSynchronize(stream));
        set_scalar(scalar, 0.0);
        if (is_F) {
            Scoped sc(timer, kTOther);
            launch_normalize<T>(F.as<T>(), n, &ctrl->tmp[0], Vcol(j + 1), beta_mul_fscale(), ch.scale_divide,
                                ch.center ? cvec : nullptr, ch.center ? &ctrl->beta_mul : nullptr, part.as<double>(),
                                B.as<double>(), j + static_cast<int64_t>(j) * work, work, ctrl, stream);
        } else {
            normalize_W(j + 1, &ctrl->tmp[0]);
        }
        (void)v;
    }

    // run_lanczos_bidiagonalization from column `start` (lanczos.hpp:54-143).
    // Fast mode raises ctrl->invariant and stops on a tiny norm; careful mode
    // synchronizes after each norm and refills from the host engine.
    void lanczos(int start, bool careful, std::mt19937_64& eng, int64_t& matvecs) {
        // W_next = A * V[:, start]
        if (pre_ready && !careful) {
            // Wn = (A'F) / ||F|| from the side stream; V[:, start] = F / ||F||.
            CUDA_TRY(cudaStreamWaitEvent(stream, ev_pre, 0));
            launch_normalize<T>(Wn.as<T>(), m, &ctrl->norm_F, nullptr, nullptr, 0, nullptr, nullptr,
                                part.as<double>(), nullptr, -1, 0, ctrl, stream);
        } else {
            beta_mul_of(Vcol(start));
            multiply(Vcol(start), Wn.as<T>(), nullptr, nullptr);
            ++matvecs;
        }
        pre_ready = false;
        cgs(W.as<T>(), m, ldw, start, Wn.as<T>(), &ctrl->S, 0, 1);
        normalize_W(start, &ctrl->S);
        for (int j = start; j < work; ++j) {
            // F = A^T W_next - S V[:, j], reorthogonalized against V[:, :j+1]
            adjoint(Wn.as<T>(), F.as<T>(), &ctrl->S, Vcol(j));
            ++matvecs;
            const bool more = j + 1 < work;
            cgs(V.as<T>(), n, ldv, j + 1, F.as<T>(), more ? &ctrl->R_F : &ctrl->norm_F, more && !careful ? 1 : 0, 0);
            if (more) {
                bool refilled = false;
                if (careful) {
                    Ctrl h;
                    sync_ctrl(h);
                    if (h.R_F < h.eps) {
                        refill(F.as<T>(), n, V.as<T>(), ldv, j + 1, eng, &ctrl->R_F, true, j);
                        refilled = true;
                    }
                }
                if (!refilled) normalize_F(j);
                // W_next = A F - R_F W[:, j], reorthogonalized against W[:, :j+1]
                multiply(Vcol(j + 1), Wn.as<T>(), &ctrl->R_F, Wcol(j));
                ++matvecs;
                cgs(W.as<T>(), m, ldw, j + 1, Wn.as<T>(), &ctrl->S, careful ? 0 : 1, 0);
                bool refilledW = false;
                if (careful) {
                    Ctrl h;
                    sync_ctrl(h);
                    if (h.S < h.eps) {
                        refill(Wn.as<T>(), m, W.as<T>(), ldw, j + 1, eng, &ctrl->S, false, j);
                        refilledW = true;
                    }
                }
                if (!refilledW) normalize_W(j + 1, &ctrl->S);
            } else {
                // B(j, j) = S (lanczos.hpp:140)
                CUDA_TRY(cudaMemcpyAsync(B.as<double>() + j + static_cast<int64_t>(j) * work, &ctrl->S,
                                         sizeof(double), cudaMemcpyDeviceToDevice, stream));
            }
        }
    }

    // The restart step (compute.hpp:225-293). Working subspaces above 1024
    // (beyond the one-CTA Jacobi kernel's shared arrays) take the SVD of B
    // from cuSOLVER, after checking that the Lanczos run was not aborted, and
    // the rest of the step from the tail kernel.
    void restart(const RestartArgs& ra, size_t smem) {
        if (ra.work <= 1024) {
            launch_restart(ra, stream, smem);
            return;
        }
        Ctrl h;
        CUDA_TRY(d2h_async(&h, ctrl, sizeof(Ctrl), stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (h.abort) return;
        gesvd_device(ra.B, ra.work, ra.work, ra.BU, ra.BS, ra.BV, stream);
        launch_restart_tail(ra, stream);
    }

    struct Result {
        bool converged = false;
        int iterations = 0;
    };

    // compute.hpp:172-307 with outputs written to device buffers U (m x r), Vout (n x r), D (r).
    Result run(int64_t requested, const irlba_gb300_options& opt, double* dU, double* dV, double* dD,
               irlba_gb300_stats* stats) {
        const int64_t smaller = std::min(m, n);
        const int64_t w64 = (requested >= smaller) ? smaller : requested + std::min<int64_t>(smaller - requested, opt.extra_work);
        if (w64 == 0) invalid("number of requested dimensions must be positive");
        work = static_cast<int>(w64);
        ldv = round_up(std::max<int64_t>(n, 1), 32);
        ldw = round_up(std::max<int64_t>(m, 1), 32);

        const int64_t launches0 = g_launch_count.load();
        cudaEvent_t ev0, ev1;
        CUDA_TRY(cudaEventCreate(&ev0));
        CUDA_TRY(cudaEventCreate(&ev1));
        CUDA_TRY(cudaEventRecord(ev0, stream));
        upload_chain();
        alloc_common();
        V.alloc(sizeof(T) * ldv * work);
        W.alloc(sizeof(T) * ldw * work);
        F.alloc(sizeof(T) * std::max<int64_t>(n, 1));
        Wn.alloc(sizeof(T) * std::max<int64_t>(m, 1));
        B.alloc(sizeof(double) * work * work);
        BU.alloc(sizeof(double) * work * work);
        BV.alloc(sizeof(double) * work * work);
        BS.alloc(sizeof(double) * work);
        prevS.alloc(sizeof(double) * work);
        res.alloc(sizeof(double) * work);
        svd_scratch.alloc(restart_smem_bytes(work));
        CUDA_TRY(cudaMemsetAsync(V.ptr, 0, V.bytes, stream));
        CUDA_TRY(cudaMemsetAsync(W.ptr, 0, W.bytes, stream));
        CUDA_TRY(cudaMemsetAsync(B.ptr, 0, B.bytes, stream));
        CUDA_TRY(cudaMemsetAsync(BU.ptr, 0, BU.bytes, stream));
        CUDA_TRY(cudaMemsetAsync(BV.ptr, 0, BV.bytes, stream));
        CUDA_TRY(cudaMemsetAsync(BS.ptr, 0, BS.bytes, stream));
        CUDA_TRY(cudaMemsetAsync(prevS.ptr, 0, prevS.bytes, stream));

        // Start vector (compute.hpp:179-190), normalized on the host in FP64.
        std::mt19937_64 eng(opt.seed);
        std::vector<double> v0(n);
        if (opt.initial) {
            if (opt.initial_size != n) invalid("initialization vector does not have expected number of rows");
            std::copy(opt.initial, opt.initial + n, v0.begin());
        } else {
            fill_normals(v0, eng);
        }
        {
            double s = 0;
            for (double x : v0) s += x * x;
            s = std::sqrt(s);
            for (double& x : v0) x /= s;
            std::vector<T> vt(v0.begin(), v0.end());
            CUDA_TRY(h2d_async(V.ptr, vt.data(), sizeof(T) * n, stream));
        }
        const double raw_eps = opt.invariant_subspace_tolerance;
        const double eps = raw_eps < 0 ? std::pow(std::numeric_limits<double>::epsilon(), 0.8) : raw_eps;
        {
            Ctrl h;
            std::memset(&h, 0, sizeof(h));
            h.eps = eps;
            CUDA_TRY(h2d_async(ctrl, &h, sizeof(Ctrl), stream));
        }

        const double tol = opt.convergence_tolerance;
        const double svtol = opt.singular_value_ratio_tolerance >= 0 ? opt.singular_value_ratio_tolerance : tol;
        Result out;
        int iter = 0;
        int k = 0;
        int64_t matvecs = 0, steps = 0, careful_restarts = 0, svd_sweeps = 0;
        const DeviceInfo& di = device_info();
        const size_t restart_smem = di.max_smem_optin - 16384;
        // FP32 form only: the FP64 form keeps the reference's order of operations.
        // Host-side products synchronize the stream they are given, so they
        // stay on the engine stream.
        const bool overlap = std::is_same<T, float>::value && !A.op.host;
        if (overlap && !side) {
            CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
            CUDA_TRY(cudaEventCreateWithFlags(&ev_f, cudaEventDisableTiming));
            CUDA_TRY(cudaEventCreateWithFlags(&ev_pre, cudaEventDisableTiming));
        }

        auto reset_flags = [&]() {
            // abort, invariant, null_start back to zero (contiguous int32 fields).
            CUDA_TRY(cudaMemsetAsync(&ctrl->abort, 0, 3 * sizeof(int32_t), stream));
        };

        for (; iter < opt.max_iterations; ++iter) {
            reset_flags();
            lanczos(k, false, eng, matvecs);
            RestartArgs ra;
            ra.B = B.as<double>();
            ra.BS = BS.as<double>();
            ra.BU = BU.as<double>();
            ra.BV = BV.as<double>();
            ra.prevS = prevS.as<double>();
            ra.res = res.as<double>();
            ra.scratch = svd_scratch.as<double>();
            ra.work = work;
            ra.k = k;
            ra.requested = static_cast<int>(requested);
            ra.iter = iter;
            ra.tol = tol;
            ra.svtol = svtol;
            ra.ctrl = ctrl;
            if (overlap) CUDA_TRY(cudaEventRecord(ev_f, stream));
            {
                Scoped sc(timer, kTRestart);
                restart(ra, restart_smem);
            }
            if (overlap) {
                // Behind the restart kernel: Wn = A'F on the side stream.
                CUDA_TRY(cudaStreamWaitEvent(side, ev_f, 0));
                beta_mul_of(F.as<T>(), side);
                multiply(F.as<T>(), Wn.as<T>(), nullptr, nullptr, side);
                CUDA_TRY(cudaEventRecord(ev_pre, side));
                ++matvecs;
                pre_ready = true;
            }
            Ctrl h;
            sync_ctrl(h);
            if (overlap && (h.invariant || h.converged)) {
                // The side product is not used: order it before what follows.
                CUDA_TRY(cudaStreamWaitEvent(stream, ev_pre, 0));
                if (pre_ready) --matvecs;
                pre_ready = false;
            }
            if (h.null_start) throw Error(IRLBA_GB300_ERROR_NUMERICAL, "starting vector near the null space of the input matrix");
            if (h.invariant) {
                ++careful_restarts;
                reset_flags();
                lanczos(k, true, eng, matvecs);
                {
                    Scoped sc(timer, kTRestart);
                    restart(ra, restart_smem);
                }
                sync_ctrl(h);
                if (h.null_start) throw Error(IRLBA_GB300_ERROR_NUMERICAL, "starting vector near the null space of the input matrix");
            }
            steps += work - k;
            svd_sweeps += h.svd_sweeps;
            if (h.converged) {
                out.converged = true;
                break;
            }
            const int kn = h.k_next;
            if (kn >= work)
                throw Error(IRLBA_GB300_ERROR_UNSUPPORTED,
                            "the working subspace (number + extra_work) is too small to restart the iterations");
            {
                Scoped sc(timer, kTRotate);
                // V[:, :kn] = V BV[:, :kn]; V[:, kn] = F / ||F||  (compute.hpp:268-277)
                launch_rotate<T>(V.as<T>(), n, ldv, work, BV.as<double>(), work, kn, V.as<T>(), ldv, F.as<T>(),
                                 &ctrl->norm_F, nullptr, stream);
                // W[:, :kn] = W BU[:, :kn]  (compute.hpp:279-280)
                launch_rotate<T>(W.as<T>(), m, ldw, work, BU.as<double>(), work, kn, W.as<T>(), ldw, nullptr, nullptr,
                                 nullptr, stream);
            }
            k = kn;
        }
        out.iterations = out.converged ? iter + 1 : iter;

        // Output assembly (compute.hpp:298-305).
        {
            Scoped sc(timer, kTOther);
            CUDA_TRY(cudaMemcpyAsync(dD, BS.ptr, sizeof(double) * requested, cudaMemcpyDeviceToDevice, stream));
            launch_rotate_out<T>(W.as<T>(), m, ldw, work, BU.as<double>(), work, static_cast<int>(requested), dU, m,
                                 stream);
            launch_rotate_out<T>(V.as<T>(), n, ldv, work, BV.as<double>(), work, static_cast<int>(requested), dV, n,
                                 stream);
        }
        CUDA_TRY(cudaEventRecord(ev1, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        CUDA_TRY(cudaGetLastError());
        if (rotate_tc_take_error() != 0)
            throw Error(IRLBA_GB300_ERROR_CUDA, "a tensor-core basis rotation timed out on a wait");
        float dev_ms = 0;
        cudaEventElapsedTime(&dev_ms, ev0, ev1);
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        if (stats) {
            stats->device_ms = dev_ms;
            stats->kernel_launches = g_launch_count.load() - launches0;
            stats->matvecs = matvecs;
            stats->lanczos_steps = steps;
            stats->restarts = iter + (out.converged ? 1 : 0);
            stats->careful_restarts = careful_restarts;
            stats->svd_sweeps = svd_sweeps;
        }
        timer.collect(g_last_ms);
        for (int i = 0; i < kTNum; ++i) g_last_launches[i] = timer.launches[i];
        return out;
    }
};

// ---------------------------------------------------------------------------
// Realize (dense FP64, column-major m x n) on the device.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void unit_vector_kernel(T* x, int64_t len, int64_t pos) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < len;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        x[i] = (i == pos) ? T(1) : T(0);
}

__global__ void transpose_kernel(const double* in, int64_t m, int64_t n, double* out);

// Dense FP64 column-major realization of a user-defined operator: one product
// per unit vector along the smaller dimension (columns A e_c, or rows A^T e_r
// gathered into the transpose and transposed back).
template <typename T>
static void realize_operator(const BaseMatrix& A, double* out, cudaStream_t stream) {
    const int64_t m = A.nrow, n = A.ncol;
    if (m == 0 || n == 0) return;
    const bool by_cols = n <= m;
    const int64_t count = by_cols ? n : m, lin = by_cols ? n : m, lout = by_cols ? m : n;
    DevBuf x(sizeof(T) * lin), y(sizeof(T) * lout), tr;
    double* dst = out;
    if (!by_cols) {
        tr.alloc(sizeof(double) * m * n);
        dst = tr.as<double>();
    }
    const int grid = static_cast<int>(std::min<int64_t>((std::max(lin, lout) + 255) / 256, 152 * 8));
    for (int64_t c = 0; c < count; ++c) {
        unit_vector_kernel<T><<<grid, 256, 0, stream>>>(x.as<T>(), lin, c); count_launch();
        operator_product<T>(A, !by_cols, x.as<T>(), y.as<T>(), stream);
        launch_convert<T, double>(y.as<T>(), dst + c * lout, lout, stream);
    }
    if (!by_cols) {
        // dst is n x m (column r = row r of A); out = its transpose.
        transpose_kernel<<<152 * 8, 256, 0, stream>>>(dst, n, m, out); count_launch();
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
}

static void realize_device(const Chain& ch, double* out, cudaStream_t stream) {
    const BaseMatrix& A = *ch.base;
    CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * A.nrow * A.ncol, stream));
    if (A.is_operator()) {
        if (A.form == IRLBA_GB300_FORM_FP32_FP64STEPS) realize_operator<float>(A, out, stream);
        else realize_operator<double>(A, out, stream);
    } else {
        launch_realize(A.mul.dev, out, A.nrow, 0, stream);
    }
    DevBuf c, s;
    if (ch.center) c = upload(ch.center->data(), ch.center->size());
    if (ch.scale) s = upload(ch.scale->data(), ch.scale->size());
    launch_realize_ops(out, A.nrow, A.ncol, c.as<double>(), s.as<double>(), ch.scale_column, ch.scale_divide,
                       ch.center_outer, stream);
    CUDA_TRY(cudaStreamSynchronize(stream));
}

__global__ void transpose_kernel(const double* in, int64_t m, int64_t n, double* out) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < m * n;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = e % m, c = e / m;
        out[r * n + c] = in[e];
    }
}

__global__ void scale_columns_kernel(double* A, int64_t m, int64_t r, const double* d) {
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < m * r;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        A[e] *= d[e / m];
}

// Exact SVD (compute.hpp:30-46) on the device: realize, then one-sided Jacobi.
// cuSOLVER's dense SVD (cusolverDnDgesvd), loaded on first use for SVDs
// whose smaller dimension is above what the one-CTA Jacobi kernel holds (1024
// columns); the engine library does not link it.
struct CusolverApi {
    decltype(&cusolverDnCreate) create = nullptr;
    decltype(&cusolverDnDestroy) destroy = nullptr;
    decltype(&cusolverDnSetStream) set_stream = nullptr;
    decltype(&cusolverDnDgesvd_bufferSize) buffer_size = nullptr;
    decltype(&cusolverDnDgesvd) gesvd = nullptr;
    bool ok = false;
};
static const CusolverApi& cusolver_api() {
    static const CusolverApi api = [] {
        CusolverApi a;
        void* h = nullptr;
        for (const char* name : {"libcusolver.so", "libcusolver.so.12", "libcusolver.so.11",
                                 "/usr/local/cuda/lib64/libcusolver.so"}) {
            h = dlopen(name, RTLD_NOW | RTLD_LOCAL);
            if (h) break;
        }
        if (!h) return a;
        a.create = reinterpret_cast<decltype(a.create)>(dlsym(h, "cusolverDnCreate"));
        a.destroy = reinterpret_cast<decltype(a.destroy)>(dlsym(h, "cusolverDnDestroy"));
        a.set_stream = reinterpret_cast<decltype(a.set_stream)>(dlsym(h, "cusolverDnSetStream"));
        a.buffer_size = reinterpret_cast<decltype(a.buffer_size)>(dlsym(h, "cusolverDnDgesvd_bufferSize"));
        a.gesvd = reinterpret_cast<decltype(a.gesvd)>(dlsym(h, "cusolverDnDgesvd"));
        a.ok = a.create && a.destroy && a.set_stream && a.buffer_size && a.gesvd;
        return a;
    }();
    return api;
}

// Canonical signs of a thin SVD (the largest-magnitude entry of each V column
// positive, the first one on ties; the U column follows), the convention of
// the Jacobi kernels and the oracle. One CTA of 256 threads per column.
__global__ void canonical_signs_kernel(double* U, int64_t m, double* V, int64_t n, int64_t ncols) {
    __shared__ double best_v[32];
    __shared__ int64_t best_i[32];
    __shared__ bool flip;
    const int64_t j = blockIdx.x;
    if (j >= ncols) return;
    double* v = V + j * n;
    double best = -1.0;
    int64_t arg = n;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double a = fabs(v[i]);
        if (a > best) {
            best = a;
            arg = i;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int64_t oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob > best || (ob == best && oa < arg)) {
            best = ob;
            arg = oa;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        best_v[warp] = best;
        best_i[warp] = arg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = -1.0;
        int64_t a = n;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w)
            if (best_v[w] > b || (best_v[w] == b && best_i[w] < a)) {
                b = best_v[w];
                a = best_i[w];
            }
        flip = a < n && v[a] < 0;
    }
    __syncthreads();
    if (!flip) return;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) v[i] = -v[i];
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) U[i + j * m] = -U[i + j * m];
}

// Thin SVD of a tall column-major mm x nn matrix (copied first) by cuSOLVER:
// U (mm x nn), S (nn, descending), V (nn x nn), canonical signs.
static void gesvd_device(const double* A, int64_t mm, int64_t nn, double* U, double* S, double* V,
                         cudaStream_t stream) {
    const CusolverApi& api = cusolver_api();
    if (!api.ok)
        throw Error(IRLBA_GB300_ERROR_UNSUPPORTED,
                    "an SVD with more than 1024 columns needs cuSOLVER, which could not be loaded");
    if (mm > INT32_MAX || nn > INT32_MAX) invalid("matrix too large for the dense SVD");
    cusolverDnHandle_t h = nullptr;
    if (api.create(&h) != CUSOLVER_STATUS_SUCCESS) throw Error(IRLBA_GB300_ERROR_CUDA, "cusolverDnCreate failed");
    struct Guard {
        const CusolverApi& a;
        cusolverDnHandle_t h;
        ~Guard() { a.destroy(h); }
    } guard{api, h};
    api.set_stream(h, stream);
    int lwork = 0;
    if (api.buffer_size(h, static_cast<int>(mm), static_cast<int>(nn), &lwork) != CUSOLVER_STATUS_SUCCESS)
        throw Error(IRLBA_GB300_ERROR_CUDA, "cusolverDnDgesvd_bufferSize failed");
    DevBuf Acopy(sizeof(double) * mm * nn), VT(sizeof(double) * nn * nn), work(sizeof(double) * std::max(lwork, 1)),
        rwork(sizeof(double) * std::max<int64_t>(nn, 1)), info(sizeof(int));
    CUDA_TRY(cudaMemcpyAsync(Acopy.ptr, A, sizeof(double) * mm * nn, cudaMemcpyDeviceToDevice, stream));
    const cusolverStatus_t st =
        api.gesvd(h, 'S', 'S', static_cast<int>(mm), static_cast<int>(nn), Acopy.as<double>(), static_cast<int>(mm), S,
                  U, static_cast<int>(mm), VT.as<double>(), static_cast<int>(nn), work.as<double>(), lwork,
                  rwork.as<double>(), info.as<int>());
    if (st != CUSOLVER_STATUS_SUCCESS) throw Error(IRLBA_GB300_ERROR_CUDA, "cusolverDnDgesvd failed");
    int hinfo = 0;
    CUDA_TRY(cudaMemcpyAsync(&hinfo, info.ptr, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (hinfo != 0) throw Error(IRLBA_GB300_ERROR_NUMERICAL, "the dense SVD did not converge");
    transpose_kernel<<<152 * 8, 256, 0, stream>>>(VT.as<double>(), nn, nn, V); count_launch();
    canonical_signs_kernel<<<static_cast<unsigned>(nn), 256, 0, stream>>>(U, mm, V, nn, nn); count_launch();
    CUDA_TRY(cudaStreamSynchronize(stream));
}

static void exact_device(const Chain& ch, int64_t requested, double* dU, double* dV, double* dD,
                         cudaStream_t stream) {
    const int64_t m = ch.base->nrow, n = ch.base->ncol;
    DevBuf dense(sizeof(double) * std::max<int64_t>(m * n, 1));
    realize_device(ch, dense.as<double>(), stream);
    const bool tall = m >= n;
    const int64_t mm = tall ? m : n, nn = tall ? n : m;
    DevBuf At;
    const double* Ain = dense.as<double>();
    if (!tall) {
        At.alloc(sizeof(double) * m * n);
        transpose_kernel<<<152 * 8, 256, 0, stream>>>(dense.as<double>(), m, n, At.as<double>()); count_launch();
        Ain = At.as<double>();
    }
    DevBuf U(sizeof(double) * mm * nn), S(sizeof(double) * nn), V(sizeof(double) * nn * nn);
    if (nn > 1024) {
        // The one-CTA Jacobi kernel keeps per-column norms and the sort order
        // of at most 1024 columns in shared memory.
        gesvd_device(Ain, mm, nn, U.as<double>(), S.as<double>(), V.as<double>(), stream);
    } else {
        DevBuf scratch(sizeof(double) * (mm * nn + nn * nn)), ctrlb(sizeof(Ctrl));
        CUDA_TRY(cudaMemsetAsync(ctrlb.ptr, 0, sizeof(Ctrl), stream));
        launch_dense_svd(Ain, mm, nn, U.as<double>(), S.as<double>(), V.as<double>(), scratch.as<double>(),
                         ctrlb.as<Ctrl>(), stream);
        CUDA_TRY(cudaStreamSynchronize(stream));
    }
    CUDA_TRY(cudaMemcpyAsync(dD, S.ptr, sizeof(double) * requested, cudaMemcpyDeviceToDevice, stream));
    // tall: A = U S V^T, U is m x n. wide: A^T = U' S V'^T, so U = V' (m x m), V = U' (n x m).
    const double* Usrc = tall ? U.as<double>() : V.as<double>();
    const double* Vsrc = tall ? V.as<double>() : U.as<double>();
    CUDA_TRY(cudaMemcpyAsync(dU, Usrc, sizeof(double) * m * requested, cudaMemcpyDeviceToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(dV, Vsrc, sizeof(double) * n * requested, cudaMemcpyDeviceToDevice, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
}

static bool requested_ge_half(int64_t requested, int64_t smaller) {
    const int64_t half = smaller / 2;
    if (requested == half) return smaller % 2 == 0;
    return requested > half;
}

struct StreamGuard {
    cudaStream_t s = nullptr;
    StreamGuard() { CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~StreamGuard() {
        if (s) cudaStreamDestroy(s);
    }
};

// compute() on device outputs. Returns (converged, iterations); *out_number set.
static std::pair<bool, int> compute_device(const irlba_gb300_matrix* mat, int64_t number,
                                           const irlba_gb300_options& opt, double* dU, double* dV, double* dD,
                                           int64_t* out_number, irlba_gb300_stats* stats, cudaStream_t stream) {
    const Chain ch = flatten(mat);
    const int64_t m = ch.base->nrow, n = ch.base->ncol;
    const int64_t smaller = std::min(m, n);
    int64_t requested = number;
    if (number < 0) invalid("requested number of singular values must be non-negative");
    if (requested > smaller) {
        if (opt.cap_number) requested = smaller;
        else invalid("requested number of singular values cannot be greater than the smaller matrix dimension");
    } else if (requested == smaller && !opt.exact_for_large_number) {
        invalid("requested number of singular values must be less than the smaller matrix dimension for IRLBA iterations");
    }
    *out_number = requested;
    if ((opt.exact_for_small_matrix && smaller < 6) ||
        (opt.exact_for_large_number && requested_ge_half(requested, smaller))) {
        exact_device(ch, requested, dU, dV, dD, stream);
        return {true, 0};
    }
    if (ch.base->form == IRLBA_GB300_FORM_FP32_FP64STEPS) {
        Engine<float> e(ch, stream);
        auto r = e.run(requested, opt, dU, dV, dD, stats);
        return {r.converged, r.iterations};
    } else {
        Engine<double> e(ch, stream);
        auto r = e.run(requested, opt, dU, dV, dD, stats);
        return {r.converged, r.iterations};
    }
}

// A single matvec through the chain (Workspace::multiply / AdjointWorkspace::multiply).
template <typename T>
static void matvec_device(const Chain& ch, const double* x_host, double* y_host, bool adjoint, cudaStream_t stream) {
    Engine<T> e(ch, stream);
    const int64_t m = ch.base->nrow, n = ch.base->ncol;
    e.work = 1;
    e.upload_chain();
    e.alloc_common();
    const int64_t lin = adjoint ? m : n, lout = adjoint ? n : m;
    std::vector<T> xin(x_host, x_host + lin);
    DevBuf xd = upload(xin.data(), xin.size());
    DevBuf yd(sizeof(T) * std::max<int64_t>(lout, 1));
    if (adjoint) {
        e.beta_adj_of(xd.as<T>());
        e.adjoint(xd.as<T>(), yd.as<T>(), nullptr, nullptr);
    } else {
        e.beta_mul_of(xd.as<T>());
        e.multiply(xd.as<T>(), yd.as<T>(), nullptr, nullptr);
    }
    std::vector<T> yh(lout);
    CUDA_TRY(d2h_async(yh.data(), yd.ptr, sizeof(T) * lout, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    CUDA_TRY(cudaGetLastError());
    for (int64_t i = 0; i < lout; ++i) y_host[i] = static_cast<double>(yh[i]);
}

static HostCompressed dense_to_compressed(int64_t nrow, int64_t ncol, const void* values, bool f64, int64_t ld,
                                          bool row_major, bool by_rows) {
    // by_rows: rows = matrix rows, cols = matrix columns; else the transpose.
    HostCompressed h;
    const int64_t R = by_rows ? nrow : ncol, C = by_rows ? ncol : nrow;
    h.rows = R;
    h.cols = C;
    h.f64 = f64;
    auto at = [&](int64_t r, int64_t c) -> double {
        const int64_t i = row_major ? r * ld + c : c * ld + r;
        return f64 ? static_cast<const double*>(values)[i] : static_cast<double>(static_cast<const float*>(values)[i]);
    };
    h.own_ptr.assign(R + 1, 0);
    for (int64_t r = 0; r < R; ++r) {
        int64_t cnt = 0;
        for (int64_t c = 0; c < C; ++c) {
            const double v = by_rows ? at(r, c) : at(c, r);
            if (v != 0) {
                h.own_idx.push_back(static_cast<int32_t>(c));
                if (f64) h.own_f64.push_back(v); else h.own_f32.push_back(static_cast<float>(v));
                ++cnt;
            }
        }
        h.own_ptr[r + 1] = h.own_ptr[r] + cnt;
    }
    h.ptr = h.own_ptr.data();
    h.idx = h.own_idx.data();
    h.val = f64 ? static_cast<const void*>(h.own_f64.data()) : static_cast<const void*>(h.own_f32.data());
    return h;
}

__global__ void variances_kernel(double* d, int64_t r, double denom) {
    for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < r;
         j += static_cast<int64_t>(gridDim.x) * blockDim.x)
        d[j] = d[j] * d[j] / denom;
}

// pca() (pca.hpp:55-139) with outputs in device memory. Column statistics are
// computed on the device (pca.hpp:85-109); the decorator chain is
// SimpleMatrix -> CenteredMatrix -> ScaledMatrix(column, divide) (pca.hpp:113-126).
static std::pair<bool, int> pca_device_impl(const irlba_gb300_matrix* matrix, int32_t center, int32_t scale,
                                            int64_t number, const irlba_gb300_options& opt, double* dScores,
                                            double* dRot, double* dVar, double* dCenter, double* dScale,
                                            int64_t* out_number, irlba_gb300_stats* stats, cudaStream_t s) {
    if (matrix->kind != 0) invalid("pca() takes an undecorated matrix");
    require_stored(matrix->base.get(), "pca()");
    const int64_t nr = matrix->nrow, nc = matrix->ncol;
    if (center && nr < 1) invalid("cannot center with no observations");
    if (scale && nr < 2) invalid("cannot scale with fewer than two observations");
    std::vector<double> c0, s0;
    if (center || scale) {
        DevBuf cd, sd;
        if (!dCenter) {
            cd.alloc(sizeof(double) * std::max<int64_t>(nc, 1));
            dCenter = cd.as<double>();
        }
        if (!dScale) {
            sd.alloc(sizeof(double) * std::max<int64_t>(nc, 1));
            dScale = sd.as<double>();
        }
        DevBuf scratch(sizeof(double) * 4 * std::max<int64_t>(nc, 1));
        launch_feature_stats(matrix->base->adj.dev, nr, center, scale, dCenter, dScale, scratch.as<double>(), s);
        if (center) {
            c0.resize(nc);
            CUDA_TRY(d2h_async(c0.data(), dCenter, sizeof(double) * nc, s));
        }
        if (scale) {
            s0.resize(nc);
            CUDA_TRY(d2h_async(s0.data(), dScale, sizeof(double) * nc, s));
        }
        CUDA_TRY(cudaStreamSynchronize(s));
    }
    irlba_gb300_matrix cm, sm;
    const irlba_gb300_matrix* top = matrix;
    if (center) {
        cm.kind = 1;
        cm.inner = top;
        cm.nrow = nr;
        cm.ncol = nc;
        cm.form = matrix->form;
        cm.vec = c0;
        top = &cm;
    }
    if (scale) {
        sm.kind = 2;
        sm.inner = top;
        sm.nrow = nr;
        sm.ncol = nc;
        sm.form = matrix->form;
        sm.column = 1;
        sm.divide = 1;
        sm.vec = s0;
        top = &sm;
    }
    auto r = compute_device(top, number, opt, dScores, dRot, dVar, out_number, stats, s);
    const int64_t num = *out_number;
    // scores = U diag(D) (pca.hpp:130); variances = D^2 / (nr - 1) if nc > 1 (pca.hpp:131-136).
    if (num > 0 && nr > 0) {
        scale_columns_kernel<<<152 * 8, 256, 0, s>>>(dScores, nr, num, dVar);
        count_launch();
    }
    if (num > 0 && nc > 1) {
        variances_kernel<<<1, 64, 0, s>>>(dVar, num, static_cast<double>(nr - 1));
        count_launch();
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    CUDA_TRY(cudaGetLastError());
    return r;
}

}  // namespace irlba_gb300

namespace irlba_gb300 {

// ---------------------------------------------------------------------------
// Decorator chains beyond one centre and one scale (e.g. CenteredMatrix over
// ScaledMatrix over CenteredMatrix, or row and column scaling together): the
// chain runs as a device operator. Each product applies the decorators from
// the outside in, as the reference's nested workspaces do
// (centered.hpp:46-52,83-87; scaled.hpp:52-69,106-123):
//   multiply  Centered: beta = c . x, y = inner(x) - beta
//             Scaled column: y = inner(x * s or x / s)
//             Scaled row: y = inner(x), then y * s or y / s
//   adjoint   Centered: beta = sum x, y = inner^T(x) - beta c
//             Scaled column: y = inner^T(x), then y * s or y / s
//             Scaled row: y = inner^T(x * s or x / s)
// with the base's own products at the bottom. The extra passes are over
// vectors (length nrow or ncol), not over the matrix.
// ---------------------------------------------------------------------------
struct ChainOperator {
    const BaseMatrix* base = nullptr;
    std::vector<const irlba_gb300_matrix*> decos;
    bool f64 = true;
    std::vector<DevBuf> vecs;      // each decorator's vector in the form's type
    std::vector<DevBuf> tmps;      // one scratch vector per decorator level
    DevBuf betas, part, partial, ctrl_buf;
    int64_t nrow = 0, ncol = 0;

    template <typename T>
    void base_product(bool adjoint, const T* x, T* y, cudaStream_t s) {
        const Ctrl* ctrl = ctrl_buf.as<Ctrl>();
        if (base->is_operator()) {
            operator_product<T>(*base, adjoint, x, y, s);
            return;
        }
        const DirPlan& p = adjoint ? base->adj : base->mul;
        Epilogue<T> e;
        launch_spmv<T>(p.dev, x, y, partial.as<T>(), e, &ctrl->abort, s);
    }

    template <typename T>
    void apply(size_t level, bool adjoint, const T* x, T* y, cudaStream_t s) {
        if (level == decos.size()) {
            base_product<T>(adjoint, x, y, s);
            return;
        }
        Ctrl* ctrl = ctrl_buf.as<Ctrl>();
        const irlba_gb300_matrix* d = decos[level];
        const T* v = vecs[level].as<T>();
        T* tmp = tmps[level].as<T>();
        double* beta = betas.as<double>() + level;
        const int64_t lin = adjoint ? nrow : ncol, lout = adjoint ? ncol : nrow;
        Epilogue<T> e;
        if (d->kind == 1) {
            // Centering: beta from the input, then one rank-1 correction.
            launch_beta<T>(x, lin, nullptr, 0, adjoint ? nullptr : v, beta, part.as<double>(), ctrl, s);
            apply<T>(level + 1, adjoint, x, y, s);
            e.beta = beta;
            if (adjoint) e.cvec = v;
            launch_epilogue<T>(y, lout, e, &ctrl->abort, s);
        } else if (static_cast<bool>(d->column) != adjoint) {
            // Scaling on the input side (column scale of a multiply, row scale of an adjoint).
            launch_scale_vector<T>(x, v, d->divide, lin, tmp, s);
            apply<T>(level + 1, adjoint, tmp, y, s);
        } else {
            // Scaling on the output side.
            apply<T>(level + 1, adjoint, x, y, s);
            e.oscale = v;
            e.odivide = d->divide;
            launch_epilogue<T>(y, lout, e, &ctrl->abort, s);
        }
    }

    static int32_t product(void* user, int32_t adjoint, const void* x, void* y, void* stream) {
        auto* op = static_cast<ChainOperator*>(user);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        try {
            if (op->f64) op->apply<double>(0, adjoint != 0, static_cast<const double*>(x), static_cast<double*>(y), s);
            else op->apply<float>(0, adjoint != 0, static_cast<const float*>(x), static_cast<float*>(y), s);
            return cudaGetLastError() == cudaSuccess ? 0 : 1;
        } catch (const std::exception&) {
            return 1;
        }
    }
};

std::shared_ptr<BaseMatrix> make_chain_operator(const BaseMatrix* base,
                                                const std::vector<const irlba_gb300_matrix*>& decos) {
    auto op = std::make_shared<ChainOperator>();
    op->base = base;
    op->decos = decos;
    op->f64 = base->form == IRLBA_GB300_FORM_FP64;
    op->nrow = base->nrow;
    op->ncol = base->ncol;
    const size_t tsz = op->f64 ? sizeof(double) : sizeof(float);
    const int64_t lmax = std::max<int64_t>(std::max(base->nrow, base->ncol), 1);
    for (const irlba_gb300_matrix* d : decos) {
        if (op->f64) {
            op->vecs.push_back(upload(d->vec.data(), d->vec.size()));
        } else {
            std::vector<float> f(d->vec.begin(), d->vec.end());
            op->vecs.push_back(upload(f.data(), f.size()));
        }
        op->tmps.emplace_back(tsz * lmax);
    }
    op->betas.alloc(sizeof(double) * std::max<size_t>(decos.size(), 1));
    op->part.alloc(sizeof(double) * (cgs_update_grid(lmax) + 64));
    int64_t pmax = 1;
    if (!base->is_operator())
        pmax = std::max<int64_t>({pmax, base->mul.dev.npanels > 1 ? base->mul.dev.npanels * base->nrow : 0,
                                  base->adj.dev.npanels > 1 ? base->adj.dev.npanels * base->ncol : 0});
    op->partial.alloc(tsz * pmax);
    op->ctrl_buf.alloc(sizeof(Ctrl));
    CUDA_TRY(cudaMemset(op->ctrl_buf.ptr, 0, sizeof(Ctrl)));
    auto bm = std::make_shared<BaseMatrix>();
    bm->nrow = base->nrow;
    bm->ncol = base->ncol;
    bm->form = base->form;
    bm->store_f64 = base->store_f64;
    bm->op.device = &ChainOperator::product;
    bm->op.user = op.get();
    // The BaseMatrix keeps the operator alive through its deleter.
    return std::shared_ptr<BaseMatrix>(bm.get(), [bm, op](BaseMatrix*) {});
}

}  // namespace irlba_gb300

// ===========================================================================
// C ABI
// ===========================================================================
using namespace irlba_gb300;

extern "C" {

void irlba_gb300_default_options(irlba_gb300_options* o) {
    o->invariant_subspace_tolerance = -1;
    o->convergence_tolerance = 1e-5;
    o->singular_value_ratio_tolerance = -1;
    o->extra_work = 7;
    o->max_iterations = 1000;
    o->exact_for_small_matrix = 1;
    o->exact_for_large_number = 1;
    o->cap_number = 0;
    o->reserved0 = 0;
    o->seed = std::mt19937_64::default_seed;
    o->initial = nullptr;
    o->initial_size = 0;
}

const char* irlba_gb300_last_error(void) { return g_last_error.c_str(); }

int irlba_gb300_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return n;
}

irlba_gb300_status irlba_gb300_matrix_create_sparse(int64_t nrow, int64_t ncol, const void* values,
                                                    irlba_gb300_value_type value_type, const int32_t* indices,
                                                    const int64_t* pointers, int32_t column_major,
                                                    irlba_gb300_form form, irlba_gb300_matrix** out) {
    return guarded([&]() {
        if (!out) invalid("output handle pointer is NULL");
        if (nrow < 0 || ncol < 0) invalid("matrix dimensions must be non-negative");
        const int64_t primary = column_major ? ncol : nrow, secondary = column_major ? nrow : ncol;
        if (!pointers) invalid("pointers must not be NULL");
        if (pointers[0] != 0) invalid("pointers must start at zero");
        for (int64_t p = 0; p < primary; ++p)
            if (pointers[p + 1] < pointers[p]) invalid("pointers must be non-decreasing");
        const int64_t nnz = pointers[primary];
        device_info();
        auto base = std::make_shared<BaseMatrix>();
        base->nrow = nrow;
        base->ncol = ncol;
        base->form = form;
        const bool in_f64 = value_type == IRLBA_GB300_VALUE_F64;
        base->store_f64 = (form == IRLBA_GB300_FORM_FP64) && in_f64;
        const bool x_f64 = form == IRLBA_GB300_FORM_FP64;
        bool done = false;
        if (g_device_ingest && nnz > 0) {
            // Upload the compressed arrays, check them and build both plans on the device.
            StreamGuard sg;
            const cudaStream_t s = sg.s;
            DevBuf dptr(sizeof(int64_t) * (primary + 1)), didx(sizeof(int32_t) * nnz),
                dval((in_f64 ? sizeof(double) : sizeof(float)) * nnz), flags(sizeof(int32_t) * 4);
            CUDA_TRY(h2d_async(dptr.ptr, pointers, dptr.bytes, s));
            CUDA_TRY(h2d_async(didx.ptr, indices, didx.bytes, s));
            CUDA_TRY(h2d_async(dval.ptr, values, dval.bytes, s));
            CUDA_TRY(cudaMemsetAsync(flags.ptr, 0, flags.bytes, s));
            launch_validate(primary, secondary, nnz, dptr.as<int64_t>(), didx.as<int32_t>(), flags.as<int32_t>(), s);
            int32_t hf[4] = {0, 0, 0, 0};
            CUDA_TRY(d2h_async(hf, flags.ptr, sizeof(hf), s));
            CUDA_TRY(cudaStreamSynchronize(s));
            if (hf[1]) invalid("index out of range of the secondary dimension");
            if (!hf[2]) {
                DevCompressed native;
                native.rows = primary;
                native.cols = secondary;
                native.nnz = nnz;
                native.ptr = dptr.as<int64_t>();
                native.idx = didx.as<int32_t>();
                native.val = dval.ptr;
                native.f64 = in_f64;
                DevBuf tptr, tidx, tval;
                transpose_device(native, pointers, base->store_f64, tptr, tidx, tval, s);
                DevCompressed trans;
                trans.rows = secondary;
                trans.cols = primary;
                trans.nnz = nnz;
                trans.ptr = tptr.as<int64_t>();
                trans.idx = tidx.as<int32_t>();
                trans.val = tval.ptr;
                trans.f64 = base->store_f64;
                // native rows = primary. column_major: primary = columns -> adjoint gather.
                build_plan_device(native, base->store_f64, x_f64, column_major ? base->adj : base->mul, s);
                build_plan_device(trans, base->store_f64, x_f64, column_major ? base->mul : base->adj, s);
                CUDA_TRY(cudaStreamSynchronize(s));
                CUDA_TRY(cudaGetLastError());
                done = true;
            }
        }
        if (!done) {
            // Host ingestion (unsorted rows, or device ingestion switched off).
            std::atomic<int> bad_index{0};
            parallel_rows(pointers, primary, [&](int64_t b, int64_t e, int) {
                for (int64_t s = pointers[b]; s < pointers[e]; ++s)
                    if (indices[s] < 0 || indices[s] >= secondary) {
                        bad_index.store(1);
                        break;
                    }
            });
            if (bad_index.load()) invalid("index out of range of the secondary dimension");
            HostCompressed native;
            native.rows = primary;
            native.cols = secondary;
            native.ptr = pointers;
            native.idx = indices;
            native.val = values;
            native.f64 = in_f64;
            HostCompressed trans;
            transpose_host(native, trans);
            // native rows = primary. column_major: primary = columns -> adjoint gather.
            if (column_major) {
                build_plan(native, base->store_f64, x_f64, base->adj);
                build_plan(trans, base->store_f64, x_f64, base->mul);
            } else {
                build_plan(native, base->store_f64, x_f64, base->mul);
                build_plan(trans, base->store_f64, x_f64, base->adj);
            }
        }
        if (nnz > 0) {
            StreamGuard sg;
            encode_values(*base, sg.s);
        }
        auto* h = new irlba_gb300_matrix();
        h->kind = 0;
        h->base = base;
        h->nrow = nrow;
        h->ncol = ncol;
        h->form = form;
        *out = h;
    });
}

void irlba_gb300_set_device_ingest(int32_t on) { g_device_ingest = on != 0; }
void irlba_gb300_set_rotation_engine(int32_t engine) { set_rotate_engine(engine); }

void irlba_gb300_set_value_coding(int32_t on) { g_value_coding = on != 0; }

irlba_gb300_status irlba_gb300_rotate_device(int32_t fp64, const void* Q, int64_t L, int64_t ldq, int32_t w,
                                             const double* R, int32_t ldr, int32_t k, void* out, int64_t ldo,
                                             const void* fcol, const double* fnorm, int32_t engine, void* stream) {
    return guarded([&]() {
        if (L < 0 || w < 0 || k < 0) invalid("sizes must be non-negative");
        if (!Q || !R || !out) invalid("NULL argument");
        if (ldq < L || ldo < L || ldr < w) invalid("leading dimension is smaller than the extent");
        if (fcol && !fnorm) invalid("fcol needs fnorm");
        if (engine == 1 && (w < 1 || w > 64 || k > 64))
            throw Error(IRLBA_GB300_ERROR_UNSUPPORTED, "tensor-core rotations take 1 <= w <= 64, k <= 64");
        device_info();
        if (engine == 1 && !(fp64 ? rotate_tc64_available() : rotate_tc32_available()))
            throw Error(IRLBA_GB300_ERROR_UNSUPPORTED, "tensor-core rotation not available on this device");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (fp64) {
            const double* q = static_cast<const double*>(Q);
            double* o = static_cast<double*>(out);
            const double* f = static_cast<const double*>(fcol);
            if (engine == 1) launch_rotate_tc64(q, L, ldq, w, R, ldr, k, o, ldo, f, fnorm, nullptr, nullptr, 0, s);
            else launch_rotate_cores<double>(q, L, ldq, w, R, ldr, k, o, ldo, f, fnorm, nullptr, s);
        } else {
            const float* q = static_cast<const float*>(Q);
            float* o = static_cast<float*>(out);
            const float* f = static_cast<const float*>(fcol);
            if (engine == 1) launch_rotate_tc32(q, L, ldq, w, R, ldr, k, o, ldo, f, fnorm, nullptr, nullptr, 0, s);
            else launch_rotate_cores<float>(q, L, ldq, w, R, ldr, k, o, ldo, f, fnorm, nullptr, s);
        }
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamSynchronize(s));
        if (rotate_tc_take_error() != 0) throw Error(IRLBA_GB300_ERROR_CUDA, "a tensor-core rotation timed out on a wait");
    });
}

void irlba_gb300_set_spmv_shape(int32_t shape) { g_spmv_shape = shape >= 0 && shape <= 2 ? shape : 2; }

irlba_gb300_status irlba_gb300_matrix_create_dense(int64_t nrow, int64_t ncol, const void* values,
                                                   irlba_gb300_value_type value_type, int64_t ld, int32_t row_major,
                                                   irlba_gb300_form form, irlba_gb300_matrix** out) {
    return guarded([&]() {
        if (!out) invalid("output handle pointer is NULL");
        if (nrow < 0 || ncol < 0) invalid("matrix dimensions must be non-negative");
        if (ld < (row_major ? ncol : nrow)) invalid("leading dimension is smaller than the matrix extent");
        device_info();
        auto base = std::make_shared<BaseMatrix>();
        base->nrow = nrow;
        base->ncol = ncol;
        base->form = form;
        const bool in_f64 = value_type == IRLBA_GB300_VALUE_F64;
        base->store_f64 = (form == IRLBA_GB300_FORM_FP64) && in_f64;
        const bool x_f64 = form == IRLBA_GB300_FORM_FP64;
        HostCompressed byrow = dense_to_compressed(nrow, ncol, values, in_f64, ld, row_major != 0, true);
        TRACE("create_dense: by rows done");
        HostCompressed bycol = dense_to_compressed(nrow, ncol, values, in_f64, ld, row_major != 0, false);
        build_plan(byrow, base->store_f64, x_f64, base->mul);
        build_plan(bycol, base->store_f64, x_f64, base->adj);
        if (base->mul.dev.nnz > 0) {
            StreamGuard sg;
            encode_values(*base, sg.s);
        }
        auto* h = new irlba_gb300_matrix();
        h->kind = 0;
        h->base = base;
        h->nrow = nrow;
        h->ncol = ncol;
        h->form = form;
        *out = h;
    });
}

static irlba_gb300_matrix* operator_handle(int64_t nrow, int64_t ncol, irlba_gb300_form form, UserOperator op) {
    if (nrow < 0 || ncol < 0) invalid("matrix dimensions must be non-negative");
    if (form != IRLBA_GB300_FORM_FP64 && form != IRLBA_GB300_FORM_FP32_FP64STEPS) invalid("unknown arithmetic form");
    device_info();
    auto base = std::make_shared<BaseMatrix>();
    base->nrow = nrow;
    base->ncol = ncol;
    base->form = form;
    base->store_f64 = form == IRLBA_GB300_FORM_FP64;
    base->op = op;
    auto* h = new irlba_gb300_matrix();
    h->kind = 0;
    h->base = base;
    h->nrow = nrow;
    h->ncol = ncol;
    h->form = form;
    return h;
}

irlba_gb300_status irlba_gb300_matrix_create_device_operator(int64_t nrow, int64_t ncol,
                                                             irlba_gb300_device_product product, void* user,
                                                             irlba_gb300_form form, irlba_gb300_matrix** out) {
    return guarded([&]() {
        if (!out) invalid("output handle pointer is NULL");
        if (!product) invalid("product function must not be NULL");
        UserOperator op;
        op.device = product;
        op.user = user;
        *out = operator_handle(nrow, ncol, form, op);
    });
}

irlba_gb300_status irlba_gb300_matrix_create_host_operator(int64_t nrow, int64_t ncol,
                                                           irlba_gb300_host_product product, void* user,
                                                           irlba_gb300_form form, irlba_gb300_matrix** out) {
    return guarded([&]() {
        if (!out) invalid("output handle pointer is NULL");
        if (!product) invalid("product function must not be NULL");
        UserOperator op;
        op.host = product;
        op.user = user;
        *out = operator_handle(nrow, ncol, form, op);
    });
}

irlba_gb300_status irlba_gb300_matrix_center(const irlba_gb300_matrix* inner, const double* center,
                                             irlba_gb300_matrix** out) {
    return guarded([&]() {
        if (!inner || !out || !center) invalid("NULL argument");
        auto* h = new irlba_gb300_matrix();
        h->kind = 1;
        h->inner = inner;
        h->nrow = inner->nrow;
        h->ncol = inner->ncol;
        h->form = inner->form;
        h->vec.assign(center, center + inner->ncol);
        *out = h;
    });
}

irlba_gb300_status irlba_gb300_matrix_scale(const irlba_gb300_matrix* inner, const double* scale, int32_t column,
                                            int32_t divide, irlba_gb300_matrix** out) {
    return guarded([&]() {
        if (!inner || !out || !scale) invalid("NULL argument");
        auto* h = new irlba_gb300_matrix();
        h->kind = 2;
        h->inner = inner;
        h->nrow = inner->nrow;
        h->ncol = inner->ncol;
        h->form = inner->form;
        h->column = column ? 1 : 0;
        h->divide = divide ? 1 : 0;
        const int64_t len = column ? inner->ncol : inner->nrow;
        h->vec.assign(scale, scale + len);
        *out = h;
    });
}

irlba_gb300_status irlba_gb300_matrix_destroy(irlba_gb300_matrix* matrix) {
    return guarded([&]() { delete matrix; });
}

irlba_gb300_status irlba_gb300_matrix_dims(const irlba_gb300_matrix* matrix, int64_t* nrow, int64_t* ncol) {
    return guarded([&]() {
        if (!matrix) invalid("NULL matrix");
        *nrow = matrix->nrow;
        *ncol = matrix->ncol;
    });
}

irlba_gb300_status irlba_gb300_multiply(const irlba_gb300_matrix* matrix, const double* right, double* output) {
    return guarded([&]() {
        const Chain ch = flatten(matrix);
        StreamGuard sg;
        if (ch.base->form == IRLBA_GB300_FORM_FP32_FP64STEPS) matvec_device<float>(ch, right, output, false, sg.s);
        else matvec_device<double>(ch, right, output, false, sg.s);
    });
}

irlba_gb300_status irlba_gb300_adjoint_multiply(const irlba_gb300_matrix* matrix, const double* right,
                                                double* output) {
    return guarded([&]() {
        const Chain ch = flatten(matrix);
        StreamGuard sg;
        if (ch.base->form == IRLBA_GB300_FORM_FP32_FP64STEPS) matvec_device<float>(ch, right, output, true, sg.s);
        else matvec_device<double>(ch, right, output, true, sg.s);
    });
}

irlba_gb300_status irlba_gb300_realize(const irlba_gb300_matrix* matrix, double* output) {
    return guarded([&]() {
        const Chain ch = flatten(matrix);
        StreamGuard sg;
        const int64_t total = ch.base->nrow * ch.base->ncol;
        DevBuf d(sizeof(double) * std::max<int64_t>(total, 1));
        realize_device(ch, d.as<double>(), sg.s);
        CUDA_TRY(d2h_sync(output, d.ptr, sizeof(double) * total));
    });
}

irlba_gb300_status irlba_gb300_compute(const irlba_gb300_matrix* matrix, int64_t number,
                                       const irlba_gb300_options* options, double* U, double* V, double* D,
                                       int64_t* out_number, int32_t* converged, int32_t* iterations,
                                       irlba_gb300_stats* stats) {
    return guarded([&]() {
        if (!matrix) invalid("NULL matrix");
        irlba_gb300_options opt;
        if (options) opt = *options; else irlba_gb300_default_options(&opt);
        auto t0 = std::chrono::steady_clock::now();
        StreamGuard sg;
        const int64_t m = matrix->nrow, n = matrix->ncol;
        const int64_t cap = std::max<int64_t>(std::min(number, std::min(m, n)), 0);
        DevBuf dU(sizeof(double) * std::max<int64_t>(m * cap, 1)), dV(sizeof(double) * std::max<int64_t>(n * cap, 1)),
            dD(sizeof(double) * std::max<int64_t>(cap, 1));
        int64_t num = 0;
        auto r = compute_device(matrix, number, opt, dU.as<double>(), dV.as<double>(), dD.as<double>(), &num, stats,
                                sg.s);
        CUDA_TRY(d2h_sync(U, dU.ptr, sizeof(double) * m * num));
        CUDA_TRY(d2h_sync(V, dV.ptr, sizeof(double) * n * num));
        CUDA_TRY(d2h_sync(D, dD.ptr, sizeof(double) * num));
        if (out_number) *out_number = num;
        if (converged) *converged = r.first ? 1 : 0;
        if (iterations) *iterations = r.second;
        if (stats) stats->seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
}

// Same as irlba_gb300_compute with U, V, D in device memory (sized for `number`).
irlba_gb300_status irlba_gb300_compute_device(const irlba_gb300_matrix* matrix, int64_t number,
                                              const irlba_gb300_options* options, double* U_device,
                                              double* V_device, double* D_device, int64_t* out_number,
                                              int32_t* converged, int32_t* iterations, irlba_gb300_stats* stats,
                                              void* stream) {
    return guarded([&]() {
        if (!matrix) invalid("NULL matrix");
        irlba_gb300_options opt;
        if (options) opt = *options; else irlba_gb300_default_options(&opt);
        auto t0 = std::chrono::steady_clock::now();
        std::unique_ptr<StreamGuard> own;
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (!s) {
            own.reset(new StreamGuard());
            s = own->s;
        }
        int64_t num = 0;
        auto r = compute_device(matrix, number, opt, U_device, V_device, D_device, &num, stats, s);
        if (out_number) *out_number = num;
        if (converged) *converged = r.first ? 1 : 0;
        if (iterations) *iterations = r.second;
        if (stats) stats->seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
}

irlba_gb300_status irlba_gb300_pca(const irlba_gb300_matrix* matrix, int32_t center, int32_t scale, int64_t number,
                                   const irlba_gb300_options* options, double* scores, double* rotation,
                                   double* variances, int64_t* out_number, int32_t* converged, int32_t* iterations,
                                   double* center_out, double* scale_out, irlba_gb300_stats* stats) {
    return guarded([&]() {
        if (!matrix) invalid("NULL matrix");
        irlba_gb300_options opt;
        if (options) opt = *options; else irlba_gb300_default_options(&opt);
        auto t0 = std::chrono::steady_clock::now();
        const int64_t nr = matrix->nrow, nc = matrix->ncol;
        StreamGuard sg;
        const int64_t cap = std::max<int64_t>(std::min(number, std::min(nr, nc)), 0);
        DevBuf dS(sizeof(double) * std::max<int64_t>(nr * cap, 1)), dR(sizeof(double) * std::max<int64_t>(nc * cap, 1)),
            dVar(sizeof(double) * std::max<int64_t>(cap, 1)), dC(sizeof(double) * std::max<int64_t>(nc, 1)),
            dSc(sizeof(double) * std::max<int64_t>(nc, 1));
        int64_t num = 0;
        auto r = pca_device_impl(matrix, center, scale, number, opt, dS.as<double>(), dR.as<double>(),
                                 dVar.as<double>(), dC.as<double>(), dSc.as<double>(), &num, stats, sg.s);
        CUDA_TRY(d2h_sync(scores, dS.ptr, sizeof(double) * nr * num));
        CUDA_TRY(d2h_sync(rotation, dR.ptr, sizeof(double) * nc * num));
        CUDA_TRY(d2h_sync(variances, dVar.ptr, sizeof(double) * num));
        if (center_out && center) CUDA_TRY(d2h_sync(center_out, dC.ptr, sizeof(double) * nc));
        if (scale_out && scale) CUDA_TRY(d2h_sync(scale_out, dSc.ptr, sizeof(double) * nc));
        if (out_number) *out_number = num;
        if (converged) *converged = r.first ? 1 : 0;
        if (iterations) *iterations = r.second;
        if (stats) stats->seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
}

irlba_gb300_status irlba_gb300_pca_device(const irlba_gb300_matrix* matrix, int32_t center, int32_t scale,
                                          int64_t number, const irlba_gb300_options* options, double* scores_device,
                                          double* rotation_device, double* variances_device, int64_t* out_number,
                                          int32_t* converged, int32_t* iterations, irlba_gb300_stats* stats,
                                          void* stream) {
    return guarded([&]() {
        if (!matrix) invalid("NULL matrix");
        irlba_gb300_options opt;
        if (options) opt = *options; else irlba_gb300_default_options(&opt);
        auto t0 = std::chrono::steady_clock::now();
        std::unique_ptr<StreamGuard> own;
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (!s) {
            own.reset(new StreamGuard());
            s = own->s;
        }
        int64_t num = 0;
        auto r = pca_device_impl(matrix, center, scale, number, opt, scores_device, rotation_device,
                                 variances_device, nullptr, nullptr, &num, stats, s);
        if (out_number) *out_number = num;
        if (converged) *converged = r.first ? 1 : 0;
        if (iterations) *iterations = r.second;
        if (stats) stats->seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
}

irlba_gb300_status irlba_gb300_orthogonalize_vector_device(const double* Q, int64_t L, int64_t ldq, int64_t ncols,
                                                           double* vec, void* stream) {
    return guarded([&]() {
        if (ncols < 0 || ncols > 1024) invalid("ncols must be in [0, 1024]");
        if (ldq < L) invalid("ldq is smaller than L");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const int64_t part_sz = std::max<int64_t>(static_cast<int64_t>(cgs_dot_grid(L)) * std::max<int64_t>(ncols, 1),
                                                  cgs_update_grid(L)) + 64;
        DevBuf part(sizeof(double) * part_sz), t(sizeof(double) * std::max<int64_t>(ncols, 1)),
            ctrlb(sizeof(Ctrl)), nrm(sizeof(double));
        CUDA_TRY(cudaMemsetAsync(ctrlb.ptr, 0, sizeof(Ctrl), s));
        if (ncols > 0) {
            launch_cgs_dot<double>(Q, L, ldq, static_cast<int32_t>(ncols), vec, part.as<double>(), t.as<double>(),
                                   ctrlb.as<Ctrl>(), s);
            launch_cgs_update<double>(Q, L, ldq, static_cast<int32_t>(ncols), t.as<double>(), vec, part.as<double>(),
                                      nrm.as<double>(), 0, 0, ctrlb.as<Ctrl>(), s);
        }
        CUDA_TRY(cudaStreamSynchronize(s));
        CUDA_TRY(cudaGetLastError());
    });
}

// ---------------------------------------------------------------------------
// orthogonalize_vector without any device allocation.
//
// Some callers cannot call cudaMalloc/cudaFree: code that runs inside another
// framework's memory budget (a caching allocator that has already reserved the
// device memory), or a latency-critical loop in which cudaMalloc/cudaFree would
// synchronize the whole device and stall other streams. For them this variant
// keeps its scratch (the per-CTA partial dot products, the coefficients, the
// reduction tickets and the norm) in one file-scope device array of fixed size,
// which every GPU that loads this library holds until the process exits.
// ---------------------------------------------------------------------------
namespace irlba_gb300 {

// 1 MiB of scratch per device.
constexpr int64_t kNoAllocScratchDoubles = 131072;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Layout of the scratch, in doubles: control block at 0 (reduction tickets and
// abort flag, cleared on every call), the norm at 64, the coefficients t at 128,
// then the per-CTA partials.
constexpr int64_t kNoAllocCtrlOffset = 0;
constexpr int64_t kNoAllocNormOffset = 64;
constexpr int64_t kNoAllocCoefOffset = 128;
static_assert(sizeof(Ctrl) <= 64 * sizeof(double), "control block must fit its scratch slot");

static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[256] = {nullptr};

// Device address of the scratch array for the current device, looked up once
// per device (with that device current) and cached.
static double* noalloc_scratch_for_current_device() {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) invalid("device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    return g_noalloc_ptr[dev];
}

}  // namespace irlba_gb300

// Same operation as irlba_gb300_orthogonalize_vector_device, with no device
// allocation. The first call on each device looks up the scratch array's
// device address (make that first call before any stream capture). The call
// synchronizes `stream` before it returns. Calls share the array: calls that
// overlap on the GPU (other streams, other host threads) race on it. Sizes
// beyond the scratch are rejected: it needs
// 128 + round_up(max(ncols, 1), 32) + min(ceil(L / 256), 1216) * max(ncols, 1)
// doubles out of 131072 (1 MiB), so any L is accepted for ncols <= 107.
irlba_gb300_status irlba_gb300_orthogonalize_vector_device_noalloc(const double* Q, int64_t L, int64_t ldq,
                                                                   int64_t ncols, double* vec, void* stream) {
    return guarded([&]() {
        if (ncols < 0 || ncols > 1024) invalid("ncols must be in [0, 1024]");
        if (L < 0) invalid("L must be non-negative");
        if (ldq < L) invalid("ldq is smaller than L");
        const int64_t part_off = kNoAllocCoefOffset + round_up(std::max<int64_t>(ncols, 1), 32);
        const int64_t part_sz = std::max<int64_t>(static_cast<int64_t>(cgs_dot_grid(L)) * std::max<int64_t>(ncols, 1),
                                                  cgs_update_grid(L));
        if (part_off + part_sz > kNoAllocScratchDoubles)
            invalid("orthogonalize_vector_device_noalloc: L and ncols need " + std::to_string(part_off + part_sz) +
                    " doubles of scratch, more than the fixed " + std::to_string(kNoAllocScratchDoubles));
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        double* scratch = noalloc_scratch_for_current_device();
        Ctrl* ctrl = reinterpret_cast<Ctrl*>(scratch + kNoAllocCtrlOffset);
        double* nrm = scratch + kNoAllocNormOffset;
        double* t = scratch + kNoAllocCoefOffset;
        double* part = scratch + part_off;
        // The tickets and the abort flag must start at zero; the array keeps the
        // previous call's contents.
        CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), s));
        if (ncols > 0) {
            launch_cgs_dot<double>(Q, L, ldq, static_cast<int32_t>(ncols), vec, part, t, ctrl, s);
            launch_cgs_update<double>(Q, L, ldq, static_cast<int32_t>(ncols), t, vec, part, nrm, 0, 0, ctrl, s);
        }
        CUDA_TRY(cudaStreamSynchronize(s));
        CUDA_TRY(cudaGetLastError());
    });
}

// The restart kernel's update_k (compute.hpp:78-111) on the device, for
// `count` quadruples (k, requested, n_converged, work) in host memory.
irlba_gb300_status irlba_gb300_update_k_device(const int32_t* args, int64_t count, int32_t* out) {
    return guarded([&]() {
        if (count < 0 || (count > 0 && (!args || !out))) invalid("NULL argument");
        if (count == 0) return;
        DevBuf da(sizeof(int32_t) * 4 * count), dout(sizeof(int32_t) * count);
        CUDA_TRY(cudaMemcpy(da.ptr, args, sizeof(int32_t) * 4 * count, cudaMemcpyHostToDevice));
        launch_update_k(da.as<int32_t>(), count, dout.as<int32_t>(), nullptr);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpy(out, dout.ptr, sizeof(int32_t) * count, cudaMemcpyDeviceToHost));
    });
}

// Replaces the centre (CenteredMatrix) or scale (ScaledMatrix) vector of a
// decorator handle, same length as at creation. The reference's decorators
// read the caller's vector through a pointer at every product
// (centered.hpp:139-160, scaled.hpp:195-223); callers that keep that pointer
// semantics pass the vector's current contents here before a compute call.
irlba_gb300_status irlba_gb300_matrix_set_vector(irlba_gb300_matrix* matrix, const double* values) {
    return guarded([&]() {
        if (!matrix || !values) invalid("NULL argument");
        if (matrix->kind != 1 && matrix->kind != 2) invalid("set_vector takes a centred or scaled matrix");
        std::copy(values, values + matrix->vec.size(), matrix->vec.begin());
    });
}

// Per-kernel-class timing of the last compute call (ms) when profiling is on.
// Classes: 0 SpMV multiply, 1 SpMV adjoint, 2 reorthogonalization,
// 3 restart (small SVD), 4 rotation, 5 other. launches may be NULL.
void irlba_gb300_set_profiling(int32_t on) { g_profile = on != 0; }
int64_t irlba_gb300_launch_count(void) { return g_launch_count.load(); }
void irlba_gb300_transfer_bytes(int64_t* h2d, int64_t* d2h) {
    if (h2d) *h2d = g_h2d_bytes.load();
    if (d2h) *d2h = g_d2h_bytes.load();
}
void irlba_gb300_last_profile(double* ms, int64_t* launches) {
    for (int i = 0; i < kTNum; ++i) {
        if (ms) ms[i] = g_last_ms[i];
        if (launches) launches[i] = g_last_launches[i];
    }
}

// Single-direction SpMV of a base matrix on device vectors (no centring or
// scaling), for bandwidth measurement: y = A x (adjoint = 0) or A^T x. Vectors
// are FP64 for FP64-form matrices and FP32 otherwise.
irlba_gb300_status irlba_gb300_spmv_device(const irlba_gb300_matrix* matrix, int32_t adjoint, const void* x,
                                           void* y, void* stream) {
    return guarded([&]() {
        if (!matrix || matrix->kind != 0) invalid("spmv_device takes an undecorated matrix");
        require_stored(matrix->base.get(), "spmv_device");
        const BaseMatrix& A = *matrix->base;
        const DirPlan& p = adjoint ? A.adj : A.mul;
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        // The abort flag (zero) and the panel partials live in one stream-ordered
        // allocation on the caller's stream, so calls on different devices or
        // streams never share scratch.
        const size_t vbytes = A.form == IRLBA_GB300_FORM_FP64 ? 8 : 4;
        const size_t pbytes = p.dev.npanels > 1 ? vbytes * static_cast<size_t>(p.dev.npanels * p.dev.nrows) : 0;
        void* scratch = nullptr;
        CUDA_TRY(cudaMallocAsync(&scratch, 256 + pbytes, s));
        int32_t* zero_flag = static_cast<int32_t*>(scratch);
        void* partial = static_cast<char*>(scratch) + 256;
        cudaError_t err = cudaMemsetAsync(zero_flag, 0, sizeof(int32_t), s);
        if (err == cudaSuccess) {
            if (A.form == IRLBA_GB300_FORM_FP64) {
                Epilogue<double> e;
                launch_spmv<double>(p.dev, static_cast<const double*>(x), static_cast<double*>(y),
                                    static_cast<double*>(partial), e, zero_flag, s);
            } else {
                Epilogue<float> e;
                launch_spmv<float>(p.dev, static_cast<const float*>(x), static_cast<float*>(y),
                                   static_cast<float*>(partial), e, zero_flag, s);
            }
            err = cudaGetLastError();
        }
        const cudaError_t ferr = cudaFreeAsync(scratch, s);
        CUDA_TRY(err);
        CUDA_TRY(ferr);
    });
}

// Layout facts of a base matrix for byte accounting: nnz, stored value bytes,
// index bytes (per direction), panels (per direction).
irlba_gb300_status irlba_gb300_matrix_layout(const irlba_gb300_matrix* matrix, int64_t* nnz, int32_t* value_bytes,
                                             int32_t* index_bytes_mul, int32_t* index_bytes_adj, int32_t* panels_mul,
                                             int32_t* panels_adj) {
    return guarded([&]() {
        if (!matrix || matrix->kind != 0) invalid("matrix_layout takes an undecorated matrix");
        require_stored(matrix->base.get(), "matrix_layout");
        const BaseMatrix& A = *matrix->base;
        *nnz = A.mul.dev.nnz;
        *value_bytes = A.store_f64 ? 8 : (A.mul.dev.code ? 2 : 4);
        *index_bytes_mul = A.mul.dev.staged ? 2 : 4;
        *index_bytes_adj = A.adj.dev.staged ? 2 : 4;
        *panels_mul = A.mul.dev.npanels;
        *panels_adj = A.adj.dev.npanels;
    });
}

}  // extern "C"
