// The restart rotation of the FP32 form, out[:, :k] = Q[:, :w] R[:w, :k]
// (compute.hpp:268-280: V <- V BV, W <- W BU), on the tcgen05 tensor cores.
//
// FP32 accuracy from BF16 operands by splitting every value into three BF16
// terms, x = a0 + a1 + a2 exactly (a0 = bf16(x), a1 = bf16(x - a0),
// a2 = x - a0 - a1: eight significant bits each), as in the error-free
// splitting of Ozaki, Ogita, Oishi and Rump ("Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication",
// Numerical Algorithms 59, 2012), here without exact accumulation: the
// products a_s b_t are exact in FP32 and the six pairs with s + t <= 2 are
// added into one FP32 accumulator (smallest pairs first), so the result has
// the rounding of an FP32 dot product (the dropped pairs weigh 2^-24 and
// less). R is rounded to FP32 first.
//
// One persistent CTA per SM walks 128-row tiles: eight producer warps (two
// groups of four, alternate tiles, one thread per row) copy their tile of Q
// into a shared-memory stage with cp.async one tile ahead (or load rows
// directly when Q is not 16-byte aligned), split it and write the three term
// slices in the no-swizzle K-major core-matrix layout; one thread issues the
// 24 MMAs of a tile (M = 128, N = 64, K = 16, kind::f16 with BF16 operands and
// FP32 accumulation) and commits them to an mbarrier; four epilogue warps read
// the accumulator of their 32 rows from TMEM (tcgen05.ld) and store the output
// rows. Two slice buffers and two TMEM accumulators let the loads and
// splitting of one tile overlap the MMAs and the epilogue of the previous one.
// Every wait is bounded: on expiry the CTA records an error, stops issuing work
// and frees its TMEM.
//
// The FP64 form's rotation (rotate_tc64_kernel, below) splits exactly: seven
// integer slices of eight bits taken from a fixed-point image of each FP64
// value, 28 slice pairs in exact accumulators, accurate to the FP64 rounding
// level.
//
// Shared-memory layout of a 128 x 64 (or 64 x 64) BF16 operand: core matrices
// of 8 rows x 16 bytes (eight K-consecutive elements), core (i, kc) at byte
// (8 i + kc) 128; so the leading byte offset (between K-adjacent cores) is 128
// and the stride byte offset (between row-adjacent cores) is 1024, and K-step
// kk of 16 starts 256 kk bytes in.

#include <cuda_bf16.h>

#include <cstdint>

#include "kernels.cuh"

namespace irlba_gb300 {

// Set by a rotation whose bounded waits expired (its output is then invalid);
// read and cleared by rotate_tc_take_error().
__device__ int32_t g_rotate_tc_error = 0;

namespace {

constexpr int kTcRows = 128;                                   // tile rows = MMA M
constexpr int kTcK = 64;                                       // padded w (4 K-steps)
constexpr int kTcN = 64;                                       // padded k = MMA N
constexpr int kTcSlices = 3;
constexpr uint32_t kTcSliceA = kTcRows * kTcK * 2;             // 16 KB
constexpr uint32_t kTcSliceB = kTcN * kTcK * 2;                // 8 KB
constexpr uint32_t kTcAccCols = 256;                           // TMEM columns per accumulator set (FP64 kernel)
constexpr uint32_t kTc32Cols = 64;                             // one FP32 accumulator
constexpr int kTcEpiWarps = 4, kTcProdWarps = 8;
constexpr int kTcThreads = 32 * (kTcEpiWarps + kTcProdWarps + 1);
constexpr long long kTcWaitCycles = 4000000000ll;              // bounded waits: about 2 s of SM clock

struct TcSmem {
    alignas(1024) unsigned char A[2][kTcSlices][kTcSliceA];
    alignas(1024) unsigned char B[kTcSlices][kTcSliceB];
    alignas(16) float stage[2][kTcK * kTcRows];   // Q tile per producer group, [column][row]
    alignas(8) unsigned long long full[2];
    alignas(8) unsigned long long tfull[2];
    alignas(8) unsigned long long tempty[2];
    uint32_t tmem;
    int err;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = static_cast<uint64_t>((addr & 0x3ffffu) >> 4);
    d |= static_cast<uint64_t>(128u >> 4) << 16;     // leading byte offset: K-adjacent cores
    d |= static_cast<uint64_t>(1024u >> 4) << 32;    // stride byte offset: row-adjacent cores
    d |= static_cast<uint64_t>(1) << 46;             // descriptor version
    return d;                                        // base offset 0, no swizzle
}

// Instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N, M.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kTcN >> 3) << 17) |
                              (static_cast<uint32_t>(kTcRows >> 4) << 24);

__device__ __forceinline__ int core_offset(int r, int k) {
    return ((r >> 3) * 8 + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ void mbar_init(unsigned long long* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_addr(b)) : "memory");
}
// Waits for the phase with the given parity; false once kTcWaitCycles SM
// cycles have passed without it.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, uint32_t parity) {
    uint32_t done = 0;
    const long long t0 = clock64();
    while (true) {
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(smem_addr(b)), "r"(parity) : "memory");
        if (done) return true;
        if (clock64() - t0 > kTcWaitCycles) return false;
    }
}

// 16-byte asynchronous copy global -> shared; bytes < 16 reads only that many
// and fills the rest with zeros.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// Barrier of the 128 threads of one producer group (named barrier id).
__device__ __forceinline__ void group_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
// The same barrier, returning whether v holds in every thread of the group.
__device__ __forceinline__ bool group_all(bool v, int id) {
    uint32_t r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, 128, p;\n"
                 " selp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(r) : "r"(static_cast<uint32_t>(v)), "r"(id) : "memory");
    return r != 0;
}

// Three-term BF16 split of two values, as packed BF16 pairs (first value in the
// low half): x = t0 + t1 + t2 exactly for normal x (each term the BF16
// rounding of the remainder, which is exact in FP32).
__device__ __forceinline__ void split3x2(float xa, float xb, uint32_t& t0, uint32_t& t1, uint32_t& t2) {
    __nv_bfloat162 h = __floats2bfloat162_rn(xa, xb);
    t0 = *reinterpret_cast<uint32_t*>(&h);
    const float ra = xa - __low2float(h), rb = xb - __high2float(h);
    h = __floats2bfloat162_rn(ra, rb);
    t1 = *reinterpret_cast<uint32_t*>(&h);
    h = __floats2bfloat162_rn(ra - __low2float(h), rb - __high2float(h));
    t2 = *reinterpret_cast<uint32_t*>(&h);
}

// STAGED: Q tiles are copied into shared memory by cp.async one tile ahead
// (needs a 16-byte aligned Q and ldq % 4 == 0); otherwise each producer
// thread loads its row directly.
template <bool STAGED>
__global__ void __launch_bounds__(kTcThreads, 1)
    rotate_tc32_kernel(const float* Q, int64_t L, int64_t ldq, int32_t w, const double* __restrict__ R, int32_t ldr,
                       int32_t k, float* out, int64_t ldo, const float* __restrict__ fcol, const double* fnorm,
                       const int32_t* abort, int32_t* error_flag) {
    extern __shared__ __align__(1024) unsigned char tc_raw[];
    // 1024-byte alignment of the operand buffers inside the dynamic window.
    TcSmem& S = *reinterpret_cast<TcSmem*>(tc_raw + ((1024 - (smem_addr(tc_raw) & 1023)) & 1023));
    if (abort && *abort) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (L + kTcRows - 1) / kTcRows;
    const int nk = (w + 15) / 16;   // K-steps with data

    // Setup: R's term slices (R rounded to FP32), spread over the whole CTA
    // with consecutive threads on consecutive rows of a column, two rows each.
    for (int e = tid; e < kTcN * kTcK / 2; e += blockDim.x) {
        const int c = (2 * e) / kTcK, j = (2 * e) % kTcK;
        const bool live = c < k;
        const float xa = (live && j < w) ? static_cast<float>(R[j + static_cast<int64_t>(c) * ldr]) : 0.0f;
        const float xb = (live && j + 1 < w) ? static_cast<float>(R[j + 1 + static_cast<int64_t>(c) * ldr]) : 0.0f;
        uint32_t t[kTcSlices];
        split3x2(xa, xb, t[0], t[1], t[2]);
        for (int q = 0; q < kTcSlices; ++q) *reinterpret_cast<uint32_t*>(S.B[q] + core_offset(c, j)) = t[q];
    }
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(&S.full[b], 32 * kTcProdWarps / 2);
            mbar_init(&S.tfull[b], 1);
            mbar_init(&S.tempty[b], 32 * kTcEpiWarps);
        }
        S.err = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem)),
                     "r"(2 * kTc32Cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = S.tmem;

    if (warp < kTcEpiWarps) {
        // Epilogue: rows 32 warp + lane of each tile (TMEM lanes of this warp).
        const float finv = fcol ? static_cast<float>(1.0 / *fnorm) : 0.0f;
        int64_t i = 0;
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            const int b = static_cast<int>(i & 1);
            // The warp leaves together (the TMEM loads below are warp-collective).
            bool ok = mbar_wait(&S.tfull[b], static_cast<uint32_t>((i >> 1) & 1));
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                atomicExch(&S.err, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int row = warp * 32 + lane;
            const int64_t r = tile * kTcRows + row;
            const uint32_t base = tmem + static_cast<uint32_t>(b) * kTc32Cols + (static_cast<uint32_t>(warp * 32) << 16);
            for (int c0 = 0; c0 < kTcN; c0 += 16) {
                uint32_t v[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(base + static_cast<uint32_t>(c0)));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (r < L) {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (c0 + j < k) out[r + static_cast<int64_t>(c0 + j) * ldo] = __uint_as_float(v[j]);
                }
            }
            if (fcol && r < L) out[r + static_cast<int64_t>(k) * ldo] = fcol[r] * finv;
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(&S.tempty[b]);
        }
    } else if (warp < kTcEpiWarps + kTcProdWarps) {
        // Producers: group g takes the CTA's tiles i = g, g + 2, ... into buffer g.
        const int pw = warp - kTcEpiWarps;
        const int g = pw / (kTcProdWarps / 2);
        const int row = (pw % (kTcProdWarps / 2)) * 32 + lane;   // also the thread's index in its group
        float* stg = S.stage[g];
        // Copies of tile `tile` into the group's stage: 2,048 16-byte chunks
        // (4 rows of one column each), 16 per thread, rows past L zero-filled.
        auto issue = [&](int64_t tile) {
            const int64_t r0 = tile * kTcRows;
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int q = row + 128 * u;
                const int j = q >> 5, r4 = (q & 31) * 4;
                if (j < w) {
                    const int64_t rem = L - (r0 + r4);
                    const uint32_t bytes = rem >= 4 ? 16u : (rem > 0 ? 4u * static_cast<uint32_t>(rem) : 0u);
                    const float* src = bytes ? Q + r0 + r4 + static_cast<int64_t>(j) * ldq : Q;
                    cp_async16(stg + j * kTcRows + r4, src, bytes);
                }
            }
            cp_async_commit();
        };
        int64_t i = g;
        int64_t tile = blockIdx.x + g * static_cast<int64_t>(gridDim.x);
        if (STAGED && tile < ntiles) issue(tile);
        for (; tile < ntiles; tile += 2 * static_cast<int64_t>(gridDim.x), i += 2) {
            const int64_t r = tile * kTcRows + row;
            float x[kTcK];
            if (STAGED) {
                cp_async_wait_all();
                group_sync(1 + g);          // the whole tile has landed
#pragma unroll
                for (int j = 0; j < kTcK; ++j) x[j] = j < w ? stg[j * kTcRows + row] : 0.0f;
                group_sync(1 + g);          // every thread has read its row
                const int64_t next = tile + 2 * static_cast<int64_t>(gridDim.x);
                if (next < ntiles) issue(next);
            }
            // Buffer g is free once the MMAs of tile i - 2 have completed (their
            // commit), independent of that tile's epilogue.
            bool ok = i < 2 || mbar_wait(&S.tfull[g], static_cast<uint32_t>(((i >> 1) - 1) & 1));
            ok = ok && !S.err;
            if (STAGED) ok = group_all(ok, 1 + g);   // the group leaves together
            if (!ok) {
                atomicExch(&S.err, 1);
                break;
            }
            if (!STAGED) {
#pragma unroll
                for (int j = 0; j < kTcK; ++j) x[j] = (j < w && r < L) ? Q[r + static_cast<int64_t>(j) * ldq] : 0.0f;
            }
#pragma unroll
            for (int j0 = 0; j0 < kTcK; j0 += 8) {
                uint32_t p[kTcSlices][4];
#pragma unroll
                for (int u = 0; u < 8; u += 2) split3x2(x[j0 + u], x[j0 + u + 1], p[0][u / 2], p[1][u / 2], p[2][u / 2]);
#pragma unroll
                for (int q = 0; q < kTcSlices; ++q)
                    *reinterpret_cast<uint4*>(S.A[g][q] + core_offset(row, j0)) =
                        make_uint4(p[q][0], p[q][1], p[q][2], p[q][3]);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&S.full[g]);
        }
        if (STAGED) cp_async_wait_all();   // no copies in flight at exit
    } else if (lane == 0) {
        // MMA issue: accumulator b collects the pairs s + t = d, d = 2, 1, 0
        // (smallest terms first), over the K-steps with data.
        int64_t i = 0;
        int64_t issued = -1;
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            const int b = static_cast<int>(i & 1);
            if (!mbar_wait(&S.full[b], static_cast<uint32_t>((i >> 1) & 1))) {
                atomicExch(&S.err, 1);
                break;
            }
            if (i >= 2 && !mbar_wait(&S.tempty[b], static_cast<uint32_t>(((i >> 1) - 1) & 1))) {
                atomicExch(&S.err, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t dcol = tmem + static_cast<uint32_t>(b) * kTc32Cols;
            int first = 1;
            for (int d = 2; d >= 0; --d) {
                for (int s = 0; s <= d; ++s) {
                    const int t = d - s;
                    for (int kk = 0; kk < nk; ++kk) {
                        const uint64_t ad = smem_desc(smem_addr(S.A[b][s]) + kk * 256);
                        const uint64_t bd = smem_desc(smem_addr(S.B[t]) + kk * 256);
                        const uint32_t acc = first ? 0u : 1u;
                        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                     " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol),
                                     "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc));
                        first = 0;
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&S.tfull[b]))
                         : "memory");
            issued = i;
        }
        // The last committed MMAs are complete before the TMEM is freed (the
        // epilogue may have stopped early on an error).
        if (issued >= 0 && !mbar_wait(&S.tfull[issued & 1], static_cast<uint32_t>((issued >> 1) & 1)))
            atomicExch(&S.err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kTc32Cols));
    }
    if (tid == 0 && S.err) atomicExch(error_flag ? error_flag : &g_rotate_tc_error, 1);
}

// ---------------------------------------------------------------------------
// FP64 form: out[:, :k] = Q[:, :w] R[:w, :k] in FP64, w, k <= 64.
//
// Each FP64 value x of row r becomes the integer X = round(x 2^(1077 - E_r)),
// E_r the largest biased exponent of the row, so |X| < 2^55, and X is cut into
// its seven two's-complement bytes X = sum_s a_s 2^(48 - 8 s) (a_0 signed in
// [-128, 127], a_1..a_6 in [0, 255]); R's columns likewise (exponent F_c,
// digits b_t). Every digit is exact in BF16 and every digit product in FP32
// (|a_0 b_t| <= 2^15, |a_s b_t| <= 2^16 otherwise). With
// acc_d = sum_{s + t = d} sum_j a_s b_t (d <= 6: 28 pairs, seven TMEM
// accumulators), acc_0..acc_4 stay within 2^24 in magnitude for K <= 64 (the
// five pairs of d = 4 hold two products of at most 2^15 and three of 2^16) and
// are exact; acc_5 and acc_6 weigh 2^-40 and 2^-48 relative to acc_0 and may
// round. The integer
//   T = 2^24 (acc_0 2^24 + acc_1 2^16 + acc_2 2^8 + acc_3) + acc_4 2^16 + acc_5 2^8 + acc_6
// is formed in 64-bit arithmetic (exactly, or, when |T| >= 2^62 - 2^41, with its
// low eight bits rounded off first) and rounded once to FP64:
//   sum_j x_rj R_jc = 2^(E_r + F_c - 2106) T.
// The parts dropped (pairs with s + t >= 7, bits below the 55th of the row's
// or column's largest entry) weigh about 2^-55 of |row max| |column max| per
// term, the level of FP64 rounding in a 57-term dot product.
//
// One persistent CTA per SM walks 128-row tiles. Eight producer warps (one
// thread per row and K-half) read their rows of Q twice: the high words for
// the row exponent, then the values, written as the seven digit slices in the
// core-matrix layout; one thread issues the 112 MMAs of a tile (28 pairs x 4
// K-steps of 16, M = 128, N = 64) and commits them; eight epilogue warps (TMEM
// lane quarter warp % 4, column half warp / 4) read the accumulators, form T
// in integers and store FP64 rows. The 112 KB of A slices and the 448 TMEM
// columns are single-buffered: the producers fill the next tile while the
// epilogue drains the current one.
// ---------------------------------------------------------------------------
constexpr int k64Slices = 7;
constexpr int k64Acc = 7;
constexpr int k64EpiWarps = 8, k64ProdWarps = 8;
constexpr int k64Threads = 32 * (k64EpiWarps + k64ProdWarps + 1);

struct Tc64Smem {
    alignas(1024) unsigned char A[k64Slices][kTcSliceA];   // 7 x 16 KB
    alignas(1024) unsigned char B[k64Slices][kTcSliceB];   // 7 x 8 KB
    int32_t rowexp[2][kTcRows];                             // E_r by tile parity
    int32_t colexp[kTcN];                                   // F_c
    alignas(8) unsigned long long full;        // producers -> MMA (A slices written)
    alignas(8) unsigned long long tfull;       // MMA commit -> epilogue, producers (A free)
    alignas(8) unsigned long long tempty;      // epilogue -> MMA (TMEM drained)
    alignas(8) unsigned long long rfull[2];    // producers -> epilogue (row exponents), by tile parity
    uint32_t tmem;
    int err;
};

// Biased exponent field of the double whose high word is hi (sign dropped).
__device__ __forceinline__ int32_t exp_field(uint32_t hi) { return static_cast<int32_t>((hi >> 20) & 0x7ffu); }

// X = round(x 2^(1077 - emax)) for a double x whose biased exponent is at most
// emax (so |X| < 2^55); zero and subnormal x give 0. Rounds half away from zero.
__device__ __forceinline__ long long fixed_point(double x, int32_t emax) {
    const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x));
    const int32_t e = static_cast<int32_t>((bits >> 52) & 0x7ffu);
    if (e == 0) return 0;
    const unsigned long long m = (bits & 0xfffffffffffffull) | (1ull << 52);
    const int32_t d = emax - e;   // >= 0
    unsigned long long u;
    if (d <= 2) {
        u = m << (2 - d);
    } else {
        const int32_t s = d - 2;
        u = s >= 54 ? 0ull : (m + (1ull << (s - 1))) >> s;
    }
    const long long v = static_cast<long long>(u);
    return (bits >> 63) ? -v : v;
}

// The seven digits of X as exact FP32 values (the low four bytes of the low
// word, the next two bytes and the signed top digit of the high word); the
// byte u becomes 2^23 + u - 2^23 without a conversion instruction.
__device__ __forceinline__ void digits7(long long X, float (&f)[k64Slices]) {
    const uint32_t lo = static_cast<uint32_t>(X);
    const int32_t hi = static_cast<int32_t>(X >> 32);
    const uint32_t hu = static_cast<uint32_t>(hi);
    f[6] = __int_as_float(0x4B000000 | (lo & 0xffu)) - 8388608.0f;
    f[5] = __int_as_float(0x4B000000 | ((lo >> 8) & 0xffu)) - 8388608.0f;
    f[4] = __int_as_float(0x4B000000 | ((lo >> 16) & 0xffu)) - 8388608.0f;
    f[3] = __int_as_float(0x4B000000 | (lo >> 24)) - 8388608.0f;
    f[2] = __int_as_float(0x4B000000 | (hu & 0xffu)) - 8388608.0f;
    f[1] = __int_as_float(0x4B000000 | ((hu >> 8) & 0xffu)) - 8388608.0f;
    f[0] = __int_as_float(0x4B000000 | static_cast<uint32_t>((hi >> 16) + 256)) - 8388864.0f;   // in [-128, 127]
}

// Packed BF16 pair of two exact small integers (first in the low half).
__device__ __forceinline__ uint32_t bf16_pair(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// 2^p T rounded to the nearest FP64 (ties to even), |T| < 2^63 exact.
__device__ __forceinline__ double scaled_int_to_double(long long T, int32_t p) {
    // The conversion rounds to nearest (ties to even); the power of two is
    // then added to the exponent field when the result stays normal.
    const double d = __ll2double_rn(T);
    if (T == 0) return 0.0;
    const long long bits = __double_as_longlong(d);
    const int32_t be = static_cast<int32_t>((bits >> 52) & 0x7ff) + p;
    if (be <= 0 || be >= 2047) return ldexp(d, p);   // outside the normal range
    return __longlong_as_double(bits + static_cast<long long>(p) * (1ll << 52));
}

// 2^p (hi 2^24 + lo) rounded to FP64, |hi| < 2^47, |lo| < 2^41: exact in
// 64 bits when |hi| < 2^38; otherwise |value| >= 2^62 - 2^41 and lo's low
// eight bits (at most 2^-55 of the value) are rounded off first.
__device__ __forceinline__ double combine_to_double(long long hi, long long lo, int32_t p) {
    if ((hi < 0 ? -hi : hi) < (1ll << 38)) return scaled_int_to_double(hi * (1ll << 24) + lo, p);
    return scaled_int_to_double(hi * (1ll << 16) + ((lo + 128) >> 8), p + 8);
}

__global__ void __launch_bounds__(k64Threads, 1)
    rotate_tc64_kernel(const double* Q, int64_t L, int64_t ldq, int32_t w, const double* __restrict__ R, int32_t ldr,
                       int32_t k, double* out, int64_t ldo, const double* __restrict__ fcol, const double* fnorm,
                       const int32_t* abort, int32_t* error_flag) {
    extern __shared__ __align__(1024) unsigned char tc_raw[];
    Tc64Smem& S = *reinterpret_cast<Tc64Smem*>(tc_raw + ((1024 - (smem_addr(tc_raw) & 1023)) & 1023));
    if (abort && *abort) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (L + kTcRows - 1) / kTcRows;
    const int nk = (w + 15) / 16;   // K-steps with data

    // Setup: R's column exponents (a shared maximum) and digit slices, spread
    // over the whole CTA with consecutive threads on consecutive rows of a column.
    if (tid < kTcN) S.colexp[tid] = 0;
    __syncthreads();
    for (int e = tid; e < kTcN * kTcK; e += blockDim.x) {
        const int c = e / kTcK, j = e % kTcK;
        if (c < k && j < w)
            atomicMax(&S.colexp[c], exp_field(reinterpret_cast<const uint32_t*>(R + j + static_cast<int64_t>(c) * ldr)[1]));
    }
    __syncthreads();
    for (int e = tid; e < kTcN * kTcK / 2; e += blockDim.x) {
        const int c = (2 * e) / kTcK, j = (2 * e) % kTcK;
        const bool live = c < k;
        const long long Xa = (live && j < w) ? fixed_point(R[j + static_cast<int64_t>(c) * ldr], S.colexp[c]) : 0;
        const long long Xb = (live && j + 1 < w) ? fixed_point(R[j + 1 + static_cast<int64_t>(c) * ldr], S.colexp[c]) : 0;
        float fa[k64Slices], fb[k64Slices];
        digits7(Xa, fa);
        digits7(Xb, fb);
        for (int t = 0; t < k64Slices; ++t)
            *reinterpret_cast<uint32_t*>(S.B[t] + core_offset(c, j)) = bf16_pair(fa[t], fb[t]);
    }
    if (tid == 0) {
        mbar_init(&S.full, 32 * k64ProdWarps);
        mbar_init(&S.tfull, 1);
        mbar_init(&S.tempty, 32 * k64EpiWarps);
        mbar_init(&S.rfull[0], 32 * k64ProdWarps / 2);
        mbar_init(&S.rfull[1], 32 * k64ProdWarps / 2);
        S.err = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem)),
                     "r"(2 * kTcAccCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = S.tmem;

    if (warp < k64EpiWarps) {
        // Epilogue: rows 32 (warp % 4) + lane, columns 32 (warp / 4) .. + 31.
        const int quarter = warp & 3, half = warp >> 2;
        const double finv = fcol ? 1.0 / *fnorm : 0.0;
        int64_t i = 0;
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            const uint32_t par = static_cast<uint32_t>(i & 1);
            bool ok = mbar_wait(&S.tfull, par) &&
                      mbar_wait(&S.rfull[i & 1], static_cast<uint32_t>((i >> 1) & 1));
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                atomicExch(&S.err, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int row = quarter * 32 + lane;
            const int64_t r = tile * kTcRows + row;
            const int32_t er = S.rowexp[i & 1][row];
            const uint32_t base = tmem + (static_cast<uint32_t>(quarter * 32) << 16);
            for (int c0 = half * 32; c0 < half * 32 + 32; c0 += 8) {
                uint32_t v[k64Acc][8];
#pragma unroll
                for (int d = 0; d < k64Acc; ++d) {
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                                 : "=r"(v[d][0]), "=r"(v[d][1]), "=r"(v[d][2]), "=r"(v[d][3]), "=r"(v[d][4]),
                                   "=r"(v[d][5]), "=r"(v[d][6]), "=r"(v[d][7])
                                 : "r"(base + static_cast<uint32_t>(d * kTcN + c0)));
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (r < L) {
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int c = c0 + j;
                        if (c < k) {
                            const int32_t fc = S.colexp[c];
                            double o;
                            if (er == 2047 || fc == 2047) {
                                o = __longlong_as_double(0x7ff8000000000000ll);   // non-finite input
                            } else {
                                int32_t a[k64Acc];
#pragma unroll
                                for (int d = 0; d < k64Acc; ++d) a[d] = __float2int_rn(__uint_as_float(v[d][j]));
                                const long long hi = static_cast<long long>(a[0]) * (1ll << 24) +
                                                     static_cast<long long>(a[1]) * (1ll << 16) +
                                                     static_cast<long long>(a[2]) * (1ll << 8) + a[3];
                                const long long lo = static_cast<long long>(a[4]) * (1ll << 16) +
                                                     static_cast<long long>(a[5]) * (1ll << 8) + a[6];
                                o = combine_to_double(hi, lo, er + fc - 2106);
                            }
                            out[r + static_cast<int64_t>(c) * ldo] = o;
                        }
                    }
                }
            }
            if (half == 0 && fcol && r < L) out[r + static_cast<int64_t>(k) * ldo] = fcol[r] * finv;
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(&S.tempty);
        }
    } else if (warp < k64EpiWarps + k64ProdWarps) {
        // Producers: row 32 (pw % 4) + lane, K-half pw / 4 (columns 32 kh .. + 31).
        const int pw = warp - k64EpiWarps;
        const int row = (pw & 3) * 32 + lane, kh = pw >> 2;
        int64_t i = 0;
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            // The MMAs of the previous tile have read the A slices.
            if (i >= 1 && !mbar_wait(&S.tfull, static_cast<uint32_t>((i - 1) & 1))) {
                atomicExch(&S.err, 1);
                break;
            }
            if (S.err) break;
            const int64_t r = tile * kTcRows + row;
            const bool live = r < L;
            // Row exponent from the high words, all loads issued before use.
            int32_t emax = 0;
#pragma unroll
            for (int j0 = 0; j0 < kTcK; j0 += 16) {
                uint32_t hw[16];
#pragma unroll
                for (int u = 0; u < 16; ++u)
                    hw[u] = (j0 + u < w && live) ? reinterpret_cast<const uint32_t*>(Q + r + static_cast<int64_t>(j0 + u) * ldq)[1]
                                                 : 0u;
#pragma unroll
                for (int u = 0; u < 16; ++u) emax = max(emax, exp_field(hw[u]));
            }
            if (kh == 0) S.rowexp[i & 1][row] = emax;
#pragma unroll 1
            for (int j1 = kh * 32; j1 < kh * 32 + 32; j1 += 16) {
                double x[16];   // sixteen loads in flight per thread
#pragma unroll
                for (int u = 0; u < 16; ++u) x[u] = (j1 + u < w && live) ? Q[r + static_cast<int64_t>(j1 + u) * ldq] : 0.0;
#pragma unroll
                for (int h = 0; h < 16; h += 8) {
                    uint32_t p[k64Slices][4];
#pragma unroll
                    for (int u = 0; u < 8; u += 2) {
                        float fa[k64Slices], fb[k64Slices];
                        digits7(fixed_point(x[h + u], emax), fa);
                        digits7(fixed_point(x[h + u + 1], emax), fb);
#pragma unroll
                        for (int s = 0; s < k64Slices; ++s) p[s][u / 2] = bf16_pair(fa[s], fb[s]);
                    }
#pragma unroll
                    for (int s = 0; s < k64Slices; ++s)
                        *reinterpret_cast<uint4*>(S.A[s] + core_offset(row, j1 + h)) =
                            make_uint4(p[s][0], p[s][1], p[s][2], p[s][3]);
                }
            }
            if (kh == 0) mbar_arrive(&S.rfull[i & 1]);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&S.full);
        }
    } else if (lane == 0) {
        // MMA issue: accumulator d collects the pairs s + t = d.
        int64_t i = 0;
        int64_t issued = -1;
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            if (!mbar_wait(&S.full, static_cast<uint32_t>(i & 1))) {
                atomicExch(&S.err, 1);
                break;
            }
            if (i >= 1 && !mbar_wait(&S.tempty, static_cast<uint32_t>((i - 1) & 1))) {
                atomicExch(&S.err, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int d = 0; d < k64Acc; ++d) {
                const uint32_t dcol = tmem + static_cast<uint32_t>(d * kTcN);
                int first = 1;
                for (int s = 0; s <= d; ++s) {
                    const int t = d - s;
                    for (int kk = 0; kk < nk; ++kk) {
                        const uint64_t ad = smem_desc(smem_addr(S.A[s]) + kk * 256);
                        const uint64_t bd = smem_desc(smem_addr(S.B[t]) + kk * 256);
                        const uint32_t acc = first ? 0u : 1u;
                        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                     " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol),
                                     "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc));
                        first = 0;
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&S.tfull))
                         : "memory");
            issued = i;
        }
        if (issued >= 0 && !mbar_wait(&S.tfull, static_cast<uint32_t>(issued & 1))) atomicExch(&S.err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kTcAccCols));
    }
    if (tid == 0 && S.err) atomicExch(error_flag ? error_flag : &g_rotate_tc_error, 1);
}

}  // namespace

size_t rotate_tc32_smem_bytes() { return sizeof(TcSmem) + 1024; }
size_t rotate_tc64_smem_bytes() { return sizeof(Tc64Smem) + 1024; }

static bool g_rotate_tc_ok = false;
static bool g_rotate_tc64_ok = false;
static int g_rotate_tc_sms = 0;
// 1: restart rotations of w, k <= 64 run on the tensor cores (default);
// 0: on the CUDA cores.
static int g_rotate_engine = 1;

cudaError_t rotate_tc_configure(size_t max_smem) {
    g_rotate_tc_ok = false;
    g_rotate_tc64_ok = false;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&g_rotate_tc_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaSuccess;
    if (max_smem >= rotate_tc32_smem_bytes()) {
        e = cudaFuncSetAttribute(rotate_tc32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(rotate_tc32_smem_bytes()));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(rotate_tc32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(rotate_tc32_smem_bytes()));
        g_rotate_tc_ok = e == cudaSuccess;
    }
    if (e == cudaSuccess && max_smem >= rotate_tc64_smem_bytes()) {
        e = cudaFuncSetAttribute(rotate_tc64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(rotate_tc64_smem_bytes()));
        g_rotate_tc64_ok = e == cudaSuccess;
    }
    return e;
}

bool rotate_tc32_available() { return g_rotate_tc_ok; }
bool rotate_tc64_available() { return g_rotate_tc64_ok; }
void set_rotate_engine(int engine) { g_rotate_engine = engine == 0 ? 0 : 1; }
int rotate_engine() { return g_rotate_engine; }

int rotate_tc_take_error() {
    int32_t v = 0;
    if (cudaMemcpyFromSymbol(&v, g_rotate_tc_error, sizeof(v)) != cudaSuccess) return -1;
    if (v) {
        const int32_t zero = 0;
        cudaMemcpyToSymbol(g_rotate_tc_error, &zero, sizeof(zero));
    }
    return v;
}

static int tc_grid(int64_t L, int sms) {
    if (sms <= 0) sms = g_rotate_tc_sms > 0 ? g_rotate_tc_sms : 1;
    const int64_t tiles = (L + kTcRows - 1) / kTcRows;
    return static_cast<int>(tiles < sms ? tiles : sms);
}

void launch_rotate_tc32(const float* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                        float* out, int64_t ldo, const float* fcol, const double* fnorm, const int32_t* abort,
                        int32_t* error_flag, int sms, cudaStream_t stream) {
    if (L <= 0) return;
    const bool staged = ldq % 4 == 0 && reinterpret_cast<uintptr_t>(Q) % 16 == 0;
    if (staged)
        rotate_tc32_kernel<true><<<tc_grid(L, sms), kTcThreads, rotate_tc32_smem_bytes(), stream>>>(
            Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort, error_flag);
    else
        rotate_tc32_kernel<false><<<tc_grid(L, sms), kTcThreads, rotate_tc32_smem_bytes(), stream>>>(
            Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort, error_flag);
    count_launch();
}

void launch_rotate_tc64(const double* Q, int64_t L, int64_t ldq, int32_t w, const double* R, int32_t ldr, int32_t k,
                        double* out, int64_t ldo, const double* fcol, const double* fnorm, const int32_t* abort,
                        int32_t* error_flag, int sms, cudaStream_t stream) {
    if (L <= 0) return;
    rotate_tc64_kernel<<<tc_grid(L, sms), k64Threads, rotate_tc64_smem_bytes(), stream>>>(
        Q, L, ldq, w, R, ldr, k, out, ldo, fcol, fnorm, abort, error_flag);
    count_launch();
}

}  // namespace irlba_gb300
