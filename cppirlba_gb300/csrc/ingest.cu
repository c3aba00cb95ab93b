// Device-side ingestion of a compressed matrix into the two gather plans
// (the layout the host builder makes, built from the uploaded compressed
// arrays): validation, a stable transpose (counting sort over chunks of input
// rows), the panel layout with u16 offsets, and the CTA segment ranges.
// sparse.hpp:35-115 (ParallelSparseMatrixCore) partitions the same data for
// its threads; here the partitions are the gather plans of both directions.

#include <type_traits>

#include "kernels.cuh"

namespace irlba_gb300 {

namespace {

constexpr int kT = 256;

int grid_of(int64_t work, int cap) {
    int64_t g = (work + kT - 1) / kT;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return static_cast<int>(g);
}

// flags[1]: an index is outside [0, cols); flags[2]: a row is not sorted
// (non-decreasing). Element-parallel: entry s breaks the order when
// idx[s] < idx[s - 1] and s does not start a row (checked by binary search on
// the pointers, which the host has already checked).
__global__ void validate_kernel(int64_t rows, int64_t cols, int64_t nnz, const int64_t* __restrict__ ptr,
                                const int32_t* __restrict__ idx, int32_t* flags) {
    for (int64_t s = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; s < nnz;
         s += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t c = idx[s];
        if (c < 0 || c >= cols) flags[1] = 1;
        if (s > 0 && c < idx[s - 1]) {
            int64_t lo = 0, hi = rows;   // is there a row r with ptr[r] == s?
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (ptr[mid] < s) lo = mid + 1;
                else hi = mid;
            }
            if (ptr[lo] != s) flags[2] = 1;
        }
    }
}

// ---- exclusive scan of int64 (three passes over blocks of 1024) -------------
constexpr int kScanBlock = 1024;

__global__ void scan_block_sums_kernel(const int64_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
    __shared__ int64_t red[kT / 32];
    const int64_t b0 = static_cast<int64_t>(blockIdx.x) * kScanBlock;
    int64_t s = 0;
    for (int64_t i = b0 + threadIdx.x; i < b0 + kScanBlock && i < n; i += kT) s += in[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kT / 32; ++w) t += red[w];
        sums[blockIdx.x] = t;
    }
}

// Exclusive scan of the block sums by one CTA (sequential chunks per thread).
__global__ void scan_sums_kernel(int64_t* sums, int64_t nb, int64_t* total) {
    __shared__ int64_t part[kT];
    const int64_t per = (nb + kT - 1) / kT;
    const int64_t lo = threadIdx.x * per, hi = lo + per < nb ? lo + per : nb;
    int64_t s = 0;
    for (int64_t i = lo; i < hi; ++i) s += sums[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t run = 0;
        for (int t = 0; t < kT; ++t) {
            const int64_t v = part[t];
            part[t] = run;
            run += v;
        }
        *total = run;
    }
    __syncthreads();
    int64_t run = part[threadIdx.x];
    for (int64_t i = lo; i < hi; ++i) {
        const int64_t v = sums[i];
        sums[i] = run;
        run += v;
    }
}

// out[i] = offset(block) + exclusive prefix of in within the block; out may alias in.
__global__ void scan_apply_kernel(const int64_t* in, int64_t n, const int64_t* __restrict__ sums, int64_t* out) {
    __shared__ int64_t buf[kScanBlock];
    __shared__ int64_t warp_tot[kScanBlock / 32];
    const int64_t b0 = static_cast<int64_t>(blockIdx.x) * kScanBlock;
    for (int i = threadIdx.x; i < kScanBlock; i += kT) buf[i] = b0 + i < n ? in[b0 + i] : 0;
    __syncthreads();
    // 32 segments of 32 values: serial within a segment, then over segments.
    if (threadIdx.x < 32) {
        int64_t run = 0;
        for (int i = 0; i < 32; ++i) {
            const int64_t v = buf[threadIdx.x * 32 + i];
            buf[threadIdx.x * 32 + i] = run;
            run += v;
        }
        warp_tot[threadIdx.x] = run;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t run = sums[blockIdx.x];
        for (int w = 0; w < 32; ++w) {
            const int64_t v = warp_tot[w];
            warp_tot[w] = run;
            run += v;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kScanBlock; i += kT)
        if (b0 + i < n) out[b0 + i] = buf[i] + warp_tot[i / 32];
}

// ---- stable transpose -----------------------------------------------------
// count[c * cols + col] = entries of chunk c in column col.
__global__ void transpose_count_kernel(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                       const int64_t* __restrict__ chunk_rows, int64_t cols, int32_t* count) {
    const int c = blockIdx.x;
    const int64_t b = ptr[chunk_rows[c]], e = ptr[chunk_rows[c + 1]];
    int32_t* cnt = count + static_cast<int64_t>(c) * cols;
    for (int64_t s = b + threadIdx.x; s < e; s += blockDim.x) atomicAdd(cnt + idx[s], 1);
}

// tot[col] = sum over chunks of count[c][col].
__global__ void transpose_totals_kernel(const int32_t* __restrict__ count, int nchunks, int64_t cols, int64_t* tot) {
    for (int64_t col = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; col < cols;
         col += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t s = 0;
        for (int c = 0; c < nchunks; ++c) s += count[static_cast<int64_t>(c) * cols + col];
        tot[col] = s;
    }
}

// cursor[c][col] = tptr[col] + entries of earlier chunks in col (int64 cursors).
__global__ void transpose_cursors_kernel(const int32_t* __restrict__ count, int nchunks, int64_t cols,
                                         const int64_t* __restrict__ tptr, int64_t* cursor) {
    for (int64_t col = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; col < cols;
         col += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t run = tptr[col];
        for (int c = 0; c < nchunks; ++c) {
            cursor[static_cast<int64_t>(c) * cols + col] = run;
            run += count[static_cast<int64_t>(c) * cols + col];
        }
    }
}

// One CTA per chunk walks its rows in order; the entries of one row have
// distinct columns, so each takes the next slot of its column: the output rows
// keep increasing input-row order.
template <typename VI, typename VO>
__global__ void transpose_scatter_kernel(const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                         const VI* __restrict__ val, const int64_t* __restrict__ chunk_rows,
                                         int64_t cols, int64_t* cursor, int32_t* __restrict__ tidx,
                                         VO* __restrict__ tval) {
    const int c = blockIdx.x;
    int64_t* cur = cursor + static_cast<int64_t>(c) * cols;
    for (int64_t r = chunk_rows[c]; r < chunk_rows[c + 1]; ++r) {
        const int64_t b = ptr[r], e = ptr[r + 1];
        for (int64_t s = b + threadIdx.x; s < e; s += blockDim.x) {
            const int64_t dst = atomicAdd(reinterpret_cast<unsigned long long*>(cur + idx[s]), 1ull);
            tidx[dst] = static_cast<int32_t>(r);
            tval[dst] = static_cast<VO>(val[s]);
        }
        __syncthreads();
    }
}

// ---- panel layout -------------------------------------------------------------
// cnt[p * rows + r] = entries of row r with column in panel p (rows sorted:
// lower bounds by binary search). One warp per row, lanes over panels.
__global__ void panel_count_kernel(int64_t rows, int32_t npanels, int64_t pw, const int64_t* __restrict__ ptr,
                                   const int32_t* __restrict__ idx, int64_t* cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r = gw; r < rows; r += nw) {
        const int64_t b = ptr[r], e = ptr[r + 1];
        for (int p = lane; p < npanels; p += 32) {
            auto lower = [&](int64_t key) {
                int64_t lo = b, hi = e;
                while (lo < hi) {
                    const int64_t mid = (lo + hi) >> 1;
                    if (idx[mid] < key) lo = mid + 1;
                    else hi = mid;
                }
                return lo;
            };
            const int64_t s0 = lower(p * pw), s1 = lower((p + 1) * pw);
            cnt[static_cast<int64_t>(p) * rows + r] = s1 - s0;
        }
    }
}

// Segment (p, r) = the contiguous run of row r in panel p, copied to segptr
// order with u16 panel offsets. One warp per segment.
template <typename VI, typename VO>
__global__ void panel_scatter_kernel(int64_t rows, int32_t npanels, int64_t pw, const int64_t* __restrict__ ptr,
                                     const int32_t* __restrict__ idx, const VI* __restrict__ val,
                                     const int64_t* __restrict__ segptr, uint16_t* __restrict__ idx16,
                                     VO* __restrict__ vout) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t nseg = static_cast<int64_t>(npanels) * rows;
    for (int64_t sg = gw; sg < nseg; sg += nw) {
        const int64_t p = sg / rows, r = sg % rows;
        const int64_t dst0 = segptr[sg], len = segptr[sg + 1] - dst0;
        if (len == 0) continue;
        // The run starts at the lower bound of p * pw in row r.
        int64_t lo = ptr[r], hi = ptr[r + 1];
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (idx[mid] < p * pw) lo = mid + 1;
            else hi = mid;
        }
        for (int64_t i = lane; i < len; i += 32) {
            idx16[dst0 + i] = static_cast<uint16_t>(idx[lo + i] - p * pw);
            vout[dst0 + i] = static_cast<VO>(val[lo + i]);
        }
    }
}

// One panel: u16 columns (staged) or int32 columns, values converted.
template <typename VI, typename VO>
__global__ void copy_entries_kernel(int64_t nnz, const int32_t* __restrict__ idx, const VI* __restrict__ val,
                                    uint16_t* __restrict__ idx16, int32_t* __restrict__ idx32, VO* __restrict__ vout) {
    for (int64_t s = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; s < nnz;
         s += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (idx16) idx16[s] = static_cast<uint16_t>(idx[s]);
        else idx32[s] = idx[s];
        vout[s] = static_cast<VO>(val[s]);
    }
}

// bseg[b] = first segment s with segptr[s] + cost * s >= total * b / nblocks.
__global__ void block_seg_kernel(const int64_t* __restrict__ segptr, int64_t nseg, int64_t cost, int64_t nblocks,
                                 int64_t* bseg) {
    const int64_t total = segptr[nseg] + cost * nseg;
    for (int64_t b = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; b <= nblocks;
         b += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (b == 0) {
            bseg[0] = 0;
            continue;
        }
        if (b == nblocks) {
            bseg[b] = nseg;
            continue;
        }
        const int64_t target = total * b / nblocks;
        int64_t lo = 0, hi = nseg;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (segptr[mid] + cost * mid < target) lo = mid + 1;
            else hi = mid;
        }
        bseg[b] = lo;
    }
}

template <typename F>
void with_value_types(bool in_f64, bool out_f64, F f) {
    if (in_f64) {
        if (out_f64) f(static_cast<double*>(nullptr), static_cast<double*>(nullptr));
        else f(static_cast<double*>(nullptr), static_cast<float*>(nullptr));
    } else {
        if (out_f64) f(static_cast<float*>(nullptr), static_cast<double*>(nullptr));
        else f(static_cast<float*>(nullptr), static_cast<float*>(nullptr));
    }
}

}  // namespace

void launch_validate(int64_t rows, int64_t cols, int64_t nnz, const int64_t* ptr, const int32_t* idx,
                     int32_t* flags, cudaStream_t s) {
    if (nnz == 0) return;
    validate_kernel<<<grid_of(nnz, 152 * 16), kT, 0, s>>>(rows, cols, nnz, ptr, idx, flags);
    count_launch();
}

size_t scan_scratch_elems(int64_t n) { return static_cast<size_t>((n + kScanBlock - 1) / kScanBlock) + 1; }

void launch_exclusive_scan(const int64_t* in, int64_t n, int64_t* out, int64_t* total, int64_t* scratch,
                           cudaStream_t s) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (n > 0) scan_block_sums_kernel<<<static_cast<unsigned>(nb), kT, 0, s>>>(in, n, scratch);
    scan_sums_kernel<<<1, kT, 0, s>>>(scratch, nb, total);
    if (n > 0) scan_apply_kernel<<<static_cast<unsigned>(nb), kT, 0, s>>>(in, n, scratch, out);
    count_launch(n > 0 ? 3 : 1);
}

void launch_transpose_count(const int64_t* ptr, const int32_t* idx, const int64_t* chunk_rows, int nchunks,
                            int64_t cols, int32_t* count, cudaStream_t s) {
    transpose_count_kernel<<<nchunks, 1024, 0, s>>>(ptr, idx, chunk_rows, cols, count);
    count_launch();
}

void launch_transpose_totals(const int32_t* count, int nchunks, int64_t cols, int64_t* tot, cudaStream_t s) {
    transpose_totals_kernel<<<grid_of(cols, 152 * 16), kT, 0, s>>>(count, nchunks, cols, tot);
    count_launch();
}

void launch_transpose_cursors(const int32_t* count, int nchunks, int64_t cols, const int64_t* tptr, int64_t* cursor,
                              cudaStream_t s) {
    transpose_cursors_kernel<<<grid_of(cols, 152 * 16), kT, 0, s>>>(count, nchunks, cols, tptr, cursor);
    count_launch();
}

void launch_transpose_scatter(const int64_t* ptr, const int32_t* idx, const void* val, bool in_f64,
                              const int64_t* chunk_rows, int nchunks, int64_t cols, int64_t* cursor, int32_t* tidx,
                              void* tval, bool out_f64, cudaStream_t s) {
    with_value_types(in_f64, out_f64, [&](auto vi, auto vo) {
        using VI = std::remove_pointer_t<decltype(vi)>;
        using VO = std::remove_pointer_t<decltype(vo)>;
        transpose_scatter_kernel<VI, VO><<<nchunks, 1024, 0, s>>>(ptr, idx, static_cast<const VI*>(val), chunk_rows,
                                                                cols, cursor, tidx, static_cast<VO*>(tval));
    });
    count_launch();
}

void launch_panel_count(int64_t rows, int32_t npanels, int64_t pw, const int64_t* ptr, const int32_t* idx,
                        int64_t* cnt, cudaStream_t s) {
    if (rows == 0) return;
    panel_count_kernel<<<grid_of(rows * 32, 152 * 16), kT, 0, s>>>(rows, npanels, pw, ptr, idx, cnt);
    count_launch();
}

void launch_panel_scatter(int64_t rows, int32_t npanels, int64_t pw, const int64_t* ptr, const int32_t* idx,
                          const void* val, bool in_f64, const int64_t* segptr, uint16_t* idx16, void* vout,
                          bool out_f64, cudaStream_t s) {
    if (rows == 0) return;
    with_value_types(in_f64, out_f64, [&](auto vi, auto vo) {
        using VI = std::remove_pointer_t<decltype(vi)>;
        using VO = std::remove_pointer_t<decltype(vo)>;
        panel_scatter_kernel<VI, VO><<<grid_of(static_cast<int64_t>(npanels) * rows * 32, 152 * 16), kT, 0, s>>>(
            rows, npanels, pw, ptr, idx, static_cast<const VI*>(val), segptr, idx16, static_cast<VO*>(vout));
    });
    count_launch();
}

void launch_copy_entries(int64_t nnz, const int32_t* idx, const void* val, bool in_f64, uint16_t* idx16,
                         int32_t* idx32, void* vout, bool out_f64, cudaStream_t s) {
    if (nnz == 0) return;
    with_value_types(in_f64, out_f64, [&](auto vi, auto vo) {
        using VI = std::remove_pointer_t<decltype(vi)>;
        using VO = std::remove_pointer_t<decltype(vo)>;
        copy_entries_kernel<VI, VO><<<grid_of(nnz, 152 * 16), kT, 0, s>>>(nnz, idx, static_cast<const VI*>(val),
                                                                        idx16, idx32, static_cast<VO*>(vout));
    });
    count_launch();
}

void launch_block_seg(const int64_t* segptr, int64_t nseg, int64_t cost, int64_t nblocks, int64_t* bseg,
                      cudaStream_t s) {
    block_seg_kernel<<<grid_of(nblocks + 1, 152), kT, 0, s>>>(segptr, nseg, cost, nblocks, bseg);
    count_launch();
}

// ---------------------------------------------------------------------------
// Value dictionary of an FP32 value array (dictionary-coded SpMV plans): an
// open-addressing hash set of the values' bit patterns (slot = 1 << 32 | bits,
// 0 empty; multiplicative hash, linear probing), the compaction of its
// occupied slots into codes, and the encoding of every entry.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ uint32_t dict_hash(uint32_t b, int log2h) {
    return (b * 0x9E3779B1u) >> (32 - log2h);
}

__global__ void dict_insert_kernel(const float* __restrict__ val, int64_t n, unsigned long long* slots, int log2h,
                                   uint32_t* count, int32_t* overflow, uint32_t maxd) {
    const uint32_t hmask = (1u << log2h) - 1;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint32_t b = __float_as_uint(val[i]);
        const unsigned long long key = (1ull << 32) | b;
        uint32_t h = dict_hash(b, log2h);
        bool placed = false;
        for (uint32_t probe = 0; probe <= hmask; ++probe) {
            const unsigned long long cur = __ldcg(slots + h);
            if (cur == key) {
                placed = true;
                break;
            }
            if (cur == 0ull) {
                const unsigned long long old = atomicCAS(slots + h, 0ull, key);
                if (old == 0ull) {
                    if (atomicAdd(count, 1u) >= maxd) atomicExch(overflow, 1);
                    placed = true;
                    break;
                }
                if (old == key) {
                    placed = true;
                    break;
                }
            }
            h = (h + 1) & hmask;
        }
        if (!placed) atomicExch(overflow, 1);
    }
}

// One warp: codes of the occupied slots in slot order, and the dictionary.
__global__ void dict_compact_kernel(const unsigned long long* __restrict__ slots, int log2h, uint16_t* slot_code,
                                    float* dict) {
    const int lane = threadIdx.x & 31;
    const uint32_t nh = 1u << log2h;
    uint32_t base = 0;
    for (uint32_t s0 = 0; s0 < nh; s0 += 32) {
        const unsigned long long v = slots[s0 + lane];
        const bool occ = v != 0ull;
        const uint32_t mask = __ballot_sync(0xffffffffu, occ);
        const uint32_t code = base + __popc(mask & ((1u << lane) - 1u));
        slot_code[s0 + lane] = static_cast<uint16_t>(occ ? code : 0u);
        if (occ) dict[code] = __uint_as_float(static_cast<uint32_t>(v));
        base += __popc(mask);
    }
}

// code[i] = the code of val[i]'s slot (every value is in the set); the slots
// and their codes are staged in shared memory.
__global__ void dict_encode_kernel(const float* __restrict__ val, int64_t n,
                                   const unsigned long long* __restrict__ slots,
                                   const uint16_t* __restrict__ slot_code, int log2h, uint16_t* __restrict__ code) {
    extern __shared__ __align__(16) unsigned char dsm[];
    const uint32_t nh = 1u << log2h, hmask = nh - 1;
    unsigned long long* ss = reinterpret_cast<unsigned long long*>(dsm);
    uint16_t* sc = reinterpret_cast<uint16_t*>(ss + nh);
    for (uint32_t i = threadIdx.x; i < nh; i += blockDim.x) {
        ss[i] = slots[i];
        sc[i] = slot_code[i];
    }
    __syncthreads();
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint32_t b = __float_as_uint(val[i]);
        const unsigned long long key = (1ull << 32) | b;
        uint32_t h = dict_hash(b, log2h);
        for (uint32_t probe = 0; probe <= hmask && ss[h] != key; ++probe) h = (h + 1) & hmask;
        code[i] = sc[h];
    }
}

}  // namespace

void launch_dict_insert(const float* val, int64_t n, unsigned long long* slots, int log2h, uint32_t* count,
                        int32_t* overflow, uint32_t maxd, cudaStream_t s) {
    if (n <= 0) return;
    dict_insert_kernel<<<grid_of(n, 152 * 16), kT, 0, s>>>(val, n, slots, log2h, count, overflow, maxd);
    count_launch();
}

void launch_dict_compact(const unsigned long long* slots, int log2h, uint16_t* slot_code, float* dict,
                         cudaStream_t s) {
    dict_compact_kernel<<<1, 32, 0, s>>>(slots, log2h, slot_code, dict);
    count_launch();
}

size_t dict_encode_smem(int log2h) { return (sizeof(unsigned long long) + sizeof(uint16_t)) << log2h; }

void launch_dict_encode(const float* val, int64_t n, const unsigned long long* slots, const uint16_t* slot_code,
                        int log2h, uint16_t* code, cudaStream_t s) {
    if (n <= 0) return;
    dict_encode_kernel<<<grid_of(n, 152 * 4), kT, dict_encode_smem(log2h), s>>>(val, n, slots, slot_code, log2h,
                                                                                 code);
    count_launch();
}

}  // namespace irlba_gb300
