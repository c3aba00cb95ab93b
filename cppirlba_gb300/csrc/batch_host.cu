// Host side of the batched form: ingestion of many compressed matrices into
// pooled device arrays (both gather directions per matrix), the per-matrix
// workspace, the SpMV autotuner, the captured CUDA graph of the persistent
// launch, and the single-matrix re-solves. The C ABI is declared in
// include/irlba_gb300.h.
//
// HBM layout: one pool per array kind (values, u16 or int32 indices, row
// pointers) for each direction; matrix j's entries start at a multiple of four
// entries, so 16-byte vector loads of values and 8/16-byte loads of indices are
// aligned in every row. Workspaces (Lanczos bases, residuals, statistics,
// outputs) are pooled the same way with 32-element (128/256-byte) alignment.

#include <chrono>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>

#include "host.hpp"

namespace irlba_gb300 {

namespace {

constexpr int kCandidates[4] = {4, 8, 16, 32};
constexpr int kPrefetchCandidates[3] = {0, 1, 3};

// Lanes per row from the average number of 4-entry vectors per row (the
// schedule used before, or instead of, tuning).
int heuristic_group(int64_t nnz, int64_t rows) {
    const double vecs = rows > 0 ? static_cast<double>(nnz) / static_cast<double>(rows) / 4.0 : 0.0;
    if (vecs >= 96) return 32;
    if (vecs >= 24) return 16;
    if (vecs >= 6) return 8;
    return 4;
}

struct StreamScope {
    cudaStream_t s = nullptr;
    bool own = false;
    explicit StreamScope(void* user) {
        if (user) {
            s = static_cast<cudaStream_t>(user);
        } else {
            CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            own = true;
        }
    }
    ~StreamScope() {
        if (own) cudaStreamDestroy(s);
    }
};

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

}  // namespace irlba_gb300

using namespace irlba_gb300;

struct irlba_gb300_batch {
    int32_t count = 0;
    std::vector<int64_t> m, n, nnz;
    std::vector<int64_t> entry_off;              // first entry of matrix j in the value/index pools
    std::vector<int64_t> mul_ptr_off, adj_ptr_off;
    std::vector<uint8_t> mul_staged, adj_staged;
    int64_t total_nnz = 0, pool_entries = 0, max_staged = 0;
    DevBuf mul_ptr, adj_ptr, mul_val, adj_val, mul_idx16, adj_idx16, mul_idx32, adj_idx32;
    std::vector<int32_t> g_mul, g_adj, pf_mul, pf_adj;
    bool tuned = false, groups_fixed = false;

    // Workspace for one (work, number).
    int32_t ws_work = -1;
    int64_t ws_number = -1;
    DevBuf ws32, ws64;
    std::vector<BatchProblem> probs;
    DevBuf probs_dev, order_dev, results_dev, queue_dev, cycles_dev;
    std::vector<int32_t> order;
    std::vector<BatchResult> results;
    std::vector<irlba_gb300_batch_info> info;
    int64_t last_number = 0;
    int32_t last_center = 0, last_scale = 0;
    // Start vectors in the workspace: for which workspace and seed.
    uint64_t init_gen = ~0ull, init_seed = 0;
    bool init_random = false;
    bool have_results = false;

    // CTAs per team (0 = chosen per call from the cost estimate) and the number
    // of largest matrices a team solves jointly (-1 = from the cost estimate).
    int team_request = 0;
    int joint_request = -1;

    // Graph of [queue reset, persistent kernel] for one parameter set.
    cudaGraphExec_t exec = nullptr;
    BatchParams graph_prm;
    int graph_grid = 0, graph_count = 0, graph_team = 0, graph_joint = 0;
    size_t graph_smem = 0;
    uint64_t graph_gen = 0, ws_gen = 0;

    ~irlba_gb300_batch() {
        if (exec) cudaGraphExecDestroy(exec);
    }

    // ---- ingestion ----------------------------------------------------------
    void ingest(const int64_t* nrow, const int64_t* ncol, const void* const* values, bool f64,
                const int32_t* const* indices, const int64_t* const* pointers, bool column_major) {
        m.assign(nrow, nrow + count);
        n.assign(ncol, ncol + count);
        nnz.resize(count);
        entry_off.resize(count);
        mul_ptr_off.resize(count);
        adj_ptr_off.resize(count);
        mul_staged.resize(count);
        adj_staged.resize(count);
        const int64_t limit = batch_stage_limit();
        int64_t eo = 0, mo = 0, ao = 0;
        bool any16 = false, any32 = false;
        for (int j = 0; j < count; ++j) {
            if (m[j] < 0 || n[j] < 0) invalid("matrix " + std::to_string(j) + ": dimensions must be non-negative");
            const int64_t primary = column_major ? n[j] : m[j];
            if (!pointers[j]) invalid("matrix " + std::to_string(j) + ": pointers must not be NULL");
            if (pointers[j][0] != 0) invalid("matrix " + std::to_string(j) + ": pointers must start at zero");
            nnz[j] = pointers[j][primary];
            if (nnz[j] > 0 && (!values[j] || !indices[j]))
                invalid("matrix " + std::to_string(j) + ": values and indices must not be NULL");
            entry_off[j] = eo;
            eo += round_up(std::max<int64_t>(nnz[j], 1), 4);
            mul_ptr_off[j] = mo;
            mo += m[j] + 1;
            adj_ptr_off[j] = ao;
            ao += n[j] + 1;
            // The multiply gathers x (n entries), the adjoint y (m entries).
            mul_staged[j] = n[j] <= limit;
            adj_staged[j] = m[j] <= limit;
            if (mul_staged[j]) max_staged = std::max(max_staged, n[j]);
            if (adj_staged[j]) max_staged = std::max(max_staged, m[j]);
            any16 = any16 || mul_staged[j] || adj_staged[j];
            any32 = any32 || !mul_staged[j] || !adj_staged[j];
            total_nnz += nnz[j];
        }
        pool_entries = eo;

        std::vector<float> hv_mul(eo), hv_adj(eo);
        std::vector<uint16_t> hi16_mul(any16 ? eo : 0), hi16_adj(any16 ? eo : 0);
        std::vector<int32_t> hi32_mul(any32 ? eo : 0), hi32_adj(any32 ? eo : 0);
        std::vector<int64_t> hp_mul(mo), hp_adj(ao);

        // Matrices are independent: host threads take them largest first.
        std::vector<int32_t> by_size(count);
        for (int j = 0; j < count; ++j) by_size[j] = j;
        std::sort(by_size.begin(), by_size.end(), [&](int a, int b) { return nnz[a] > nnz[b]; });
        std::atomic<int> next{0};
        std::mutex err_mu;
        std::string err;
        auto worker = [&]() {
            std::vector<int64_t> cnt;
            while (true) {
                const int t = next.fetch_add(1);
                if (t >= count) break;
                const int j = by_size[t];
                const int64_t primary = column_major ? n[j] : m[j];
                const int64_t secondary = column_major ? m[j] : n[j];
                const int64_t* P = pointers[j];
                const int32_t* I = indices[j];
                bool ok = true;
                for (int64_t p = 0; p < primary && ok; ++p) ok = P[p + 1] >= P[p];
                for (int64_t s = 0; s < nnz[j] && ok; ++s) ok = I[s] >= 0 && I[s] < secondary;
                if (!ok) {
                    std::lock_guard<std::mutex> g(err_mu);
                    err = "matrix " + std::to_string(j) +
                          ": pointers must be non-decreasing and indices within the secondary dimension";
                    continue;
                }
                auto value = [&](int64_t s) -> float {
                    return f64 ? static_cast<float>(static_cast<const double*>(values[j])[s])
                               : static_cast<const float*>(values[j])[s];
                };
                // Native direction: rows = primary (adjoint when column-major).
                const bool native_is_mul = !column_major;
                int64_t* np_ = native_is_mul ? hp_mul.data() + mul_ptr_off[j] : hp_adj.data() + adj_ptr_off[j];
                int64_t* tp_ = native_is_mul ? hp_adj.data() + adj_ptr_off[j] : hp_mul.data() + mul_ptr_off[j];
                float* nv = (native_is_mul ? hv_mul.data() : hv_adj.data()) + entry_off[j];
                float* tv = (native_is_mul ? hv_adj.data() : hv_mul.data()) + entry_off[j];
                const bool n_staged = native_is_mul ? mul_staged[j] : adj_staged[j];
                const bool t_staged = native_is_mul ? adj_staged[j] : mul_staged[j];
                uint16_t* n16 = n_staged ? (native_is_mul ? hi16_mul.data() : hi16_adj.data()) + entry_off[j] : nullptr;
                int32_t* n32 = n_staged ? nullptr : (native_is_mul ? hi32_mul.data() : hi32_adj.data()) + entry_off[j];
                uint16_t* t16 = t_staged ? (native_is_mul ? hi16_adj.data() : hi16_mul.data()) + entry_off[j] : nullptr;
                int32_t* t32 = t_staged ? nullptr : (native_is_mul ? hi32_adj.data() : hi32_mul.data()) + entry_off[j];
                for (int64_t p = 0; p <= primary; ++p) np_[p] = P[p];
                for (int64_t s = 0; s < nnz[j]; ++s) {
                    nv[s] = value(s);
                    if (n16) n16[s] = static_cast<uint16_t>(I[s]);
                    else n32[s] = I[s];
                }
                // Transpose by counting sort (stable: rows stay sorted by primary).
                cnt.assign(secondary + 1, 0);
                for (int64_t s = 0; s < nnz[j]; ++s) ++cnt[I[s] + 1];
                for (int64_t r = 0; r < secondary; ++r) cnt[r + 1] += cnt[r];
                for (int64_t r = 0; r <= secondary; ++r) tp_[r] = cnt[r];
                for (int64_t p = 0; p < primary; ++p) {
                    for (int64_t s = P[p]; s < P[p + 1]; ++s) {
                        const int64_t d = cnt[I[s]]++;
                        tv[d] = value(s);
                        if (t16) t16[d] = static_cast<uint16_t>(p);
                        else t32[d] = static_cast<int32_t>(p);
                    }
                }
            }
        };
        const int nt = std::max(1, std::min(host_threads(), count));
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
        for (auto& th : pool) th.join();
        if (!err.empty()) invalid(err);

        device_info();
        // 64 bytes of padding: the kernels' 16-byte-rounded L2 prefetches of the
        // last rows stay inside the allocation.
        auto up = [](DevBuf& d, const void* h, size_t bytes) {
            d.alloc(bytes + 64);
            if (bytes) CUDA_TRY(h2d_sync(d.ptr, h, bytes));
        };
        up(mul_ptr, hp_mul.data(), sizeof(int64_t) * hp_mul.size());
        up(adj_ptr, hp_adj.data(), sizeof(int64_t) * hp_adj.size());
        up(mul_val, hv_mul.data(), sizeof(float) * hv_mul.size());
        up(adj_val, hv_adj.data(), sizeof(float) * hv_adj.size());
        if (any16) {
            up(mul_idx16, hi16_mul.data(), sizeof(uint16_t) * hi16_mul.size());
            up(adj_idx16, hi16_adj.data(), sizeof(uint16_t) * hi16_adj.size());
        }
        if (any32) {
            up(mul_idx32, hi32_mul.data(), sizeof(int32_t) * hi32_mul.size());
            up(adj_idx32, hi32_adj.data(), sizeof(int32_t) * hi32_adj.size());
        }
        g_mul.resize(count);
        g_adj.resize(count);
        pf_mul.assign(count, 1);
        pf_adj.assign(count, 1);
        for (int j = 0; j < count; ++j) {
            g_mul[j] = heuristic_group(nnz[j], m[j]);
            g_adj[j] = heuristic_group(nnz[j], n[j]);
        }
        queue_dev.alloc(sizeof(uint32_t));
        results_dev.alloc(sizeof(BatchResult) * std::max(count, 1));
        cycles_dev.alloc(sizeof(uint64_t) * std::max(count, 1));
        order_dev.alloc(sizeof(int32_t) * std::max(count, 1));
        probs_dev.alloc(sizeof(BatchProblem) * std::max(count, 1));
        results.resize(count);
        info.resize(count);
    }

    BatchDir dir(int j, bool adjoint) const {
        BatchDir d;
        d.rows = adjoint ? n[j] : m[j];
        d.cols = adjoint ? m[j] : n[j];
        d.ptr = (adjoint ? adj_ptr : mul_ptr).as<int64_t>() + (adjoint ? adj_ptr_off[j] : mul_ptr_off[j]);
        d.val = (adjoint ? adj_val : mul_val).as<float>() + entry_off[j];
        d.staged = adjoint ? adj_staged[j] : mul_staged[j];
        if (d.staged) d.idx = (adjoint ? adj_idx16 : mul_idx16).as<uint16_t>() + entry_off[j];
        else d.idx = (adjoint ? adj_idx32 : mul_idx32).as<int32_t>() + entry_off[j];
        d.group = adjoint ? g_adj[j] : g_mul[j];
        d.prefetch = adjoint ? pf_adj[j] : pf_mul[j];
        d.idx_bytes = d.staged ? 2 : 4;
        return d;
    }

    // ---- workspace ----------------------------------------------------------
    void workspace(int32_t work, int64_t number) {
        if (work == ws_work && number == ws_number) return;
        probs.assign(count, BatchProblem());
        int64_t o32 = 0, o64 = 0;
        std::vector<int64_t> off32(count), off64(count);
        for (int j = 0; j < count; ++j) {
            const int64_t ldv = round_up(std::max<int64_t>(n[j], 1), 32), ldw = round_up(std::max<int64_t>(m[j], 1), 32);
            off32[j] = o32;
            o32 += ldv * work + ldw * work + 4 * ldv + ldw;
            off64[j] = o64;
            o64 += 3 * ldv + round_up(m[j] * number, 32) + round_up(n[j] * number, 32) + round_up(number, 32);
        }
        ws32.alloc(sizeof(float) * std::max<int64_t>(o32, 32));
        ws64.alloc(sizeof(double) * std::max<int64_t>(o64, 32));
        for (int j = 0; j < count; ++j) {
            BatchProblem& P = probs[j];
            P.m = m[j];
            P.n = n[j];
            P.ldv = round_up(std::max<int64_t>(n[j], 1), 32);
            P.ldw = round_up(std::max<int64_t>(m[j], 1), 32);
            float* f = ws32.as<float>() + off32[j];
            P.V = f;
            f += P.ldv * work;
            P.W = f;
            f += P.ldw * work;
            P.F = f;
            f += P.ldv;
            P.xs = f;
            f += P.ldv;
            P.center = f;
            f += P.ldv;
            P.scale = f;
            f += P.ldv;
            P.Wn = f;
            double* d = ws64.as<double>() + off64[j];
            P.center64 = d;
            d += P.ldv;
            P.scale64 = d;
            d += P.ldv;
            P.init = d;
            d += P.ldv;
            P.scores = d;
            d += round_up(m[j] * number, 32);
            P.rotation = d;
            d += round_up(n[j] * number, 32);
            P.variances = d;
        }
        // Zeroed so that columns beyond the first Lanczos run read as zero.
        CUDA_TRY(cudaMemset(ws32.ptr, 0, ws32.bytes));
        CUDA_TRY(cudaMemset(ws64.ptr, 0, ws64.bytes));
        ws_work = work;
        ws_number = number;
        ++ws_gen;
    }

    // Descriptors on the device are rebuilt when the workspace or a schedule changes.
    uint64_t sched_version = 1, uploaded_ws_gen = ~0ull, uploaded_sched = 0;

    void upload_problems_if_changed(cudaStream_t s) {
        if (uploaded_ws_gen == ws_gen && uploaded_sched == sched_version) return;
        upload_problems(s);
        uploaded_ws_gen = ws_gen;
        uploaded_sched = sched_version;
    }

    void upload_problems(cudaStream_t s) {
        for (int j = 0; j < count; ++j) {
            probs[j].mul = dir(j, false);
            probs[j].adj = dir(j, true);
        }
        CUDA_TRY(h2d_async(probs_dev.ptr, probs.data(), sizeof(BatchProblem) * count, s));
        CUDA_TRY(cudaStreamSynchronize(s));
    }

    int grid_for(int32_t active) const {
        const DeviceInfo& di = device_info();
        return std::max(1, std::min<int>(active, di.sms));
    }

    // Team size and joint prefix for the active matrices (in cost order). A
    // matrix is solved by a whole team when its cost exceeds half of the
    // average per-CTA load; the rest run one per CTA. The candidate (1, 2, 4 or 8
    // CTAs per team) with the smallest estimated makespan
    //   max(largest cost / (team * eff), (joint cost / eff + solo cost) / CTAs)
    // wins; eff (1, 0.9, 0.8, 0.7) charges the team barriers.
    int choose_team(int32_t active, const std::vector<int64_t>& cost, size_t smem, int* teams_out,
                    int* joint_out) const {
        int best = 1, best_teams = 1, best_joint = 0;
        double best_est = 1e300;
        const int cands[4] = {1, 2, 4, 8};
        const double eff[4] = {1.0, 0.9, 0.8, 0.7};
        int64_t mx = 0, tot = 0;
        for (int i = 0; i < active; ++i) {
            mx = std::max(mx, cost[order[i]]);
            tot += cost[order[i]];
        }
        for (int c = 0; c < 4; ++c) {
            if (team_request && cands[c] != team_request) continue;
            const int resident = batch_max_teams(cands[c], smem);
            if (resident < 1) continue;
            const int teams = std::min(resident, std::max(active, 1));
            const double ctas = static_cast<double>(teams) * cands[c];
            int joint = 0;
            double joint_cost = 0, solo_cost = 0;
            for (int i = 0; i < active; ++i) {
                const double cj = static_cast<double>(cost[order[i]]);
                const bool take = joint_request >= 0 ? i < joint_request : cj > 0.5 * tot / ctas;
                if (cands[c] > 1 && joint == i && take) {
                    ++joint;
                    joint_cost += cj;
                } else {
                    solo_cost += cj;
                }
            }
            const double largest = joint > 0 ? mx / (cands[c] * eff[c]) : static_cast<double>(mx);
            const double est = std::max(largest, (joint_cost / eff[c] + solo_cost) / ctas);
            if (est < best_est) {
                best_est = est;
                best = cands[c];
                best_teams = teams;
                best_joint = joint;
            }
        }
        if (best_est == 1e300)
            throw Error(IRLBA_GB300_ERROR_CUDA, "no team size of the batched kernel can be resident on this device");
        *teams_out = best_teams;
        *joint_out = best > 1 ? best_joint : active;
        return best;
    }

    // ---- autotuner ----------------------------------------------------------
    // Every candidate schedule (lanes per row x L2 prefetch distance) runs as
    // one probe launch over all active matrices, so the probe sees the memory
    // contention of the solve; each matrix and direction keeps the schedule
    // with its shortest SpMV.
    double tune(int32_t repeats, int32_t active, cudaStream_t s) {
        const auto t0 = std::chrono::steady_clock::now();
        if (active == 0) return 0.0;
        const size_t smem = batch_smem_bytes(max_staged);
        const int grid = grid_for(active);
        std::vector<uint64_t> best_mul(count, ~0ull), best_adj(count, ~0ull), cyc(count);
        for (int adjoint = 0; adjoint < 2; ++adjoint) {
            for (int g : kCandidates) {
                for (int pf : kPrefetchCandidates) {
                    launch_batch_spmv_probe(probs_dev.as<BatchProblem>(), order_dev.as<int32_t>(), active, adjoint, g,
                                            pf, std::max(repeats, 1), cycles_dev.as<uint64_t>(), grid, smem, s);
                    CUDA_TRY(cudaGetLastError());
                    CUDA_TRY(d2h_async(cyc.data(), cycles_dev.ptr, sizeof(uint64_t) * count, s));
                    CUDA_TRY(cudaStreamSynchronize(s));
                    for (int i = 0; i < active; ++i) {
                        const int j = order[i];
                        auto& best = adjoint ? best_adj : best_mul;
                        if (cyc[j] < best[j]) {
                            best[j] = cyc[j];
                            (adjoint ? g_adj : g_mul)[j] = g;
                            (adjoint ? pf_adj : pf_mul)[j] = pf;
                        }
                    }
                }
            }
        }
        tuned = true;
        ++sched_version;
        return ms_since(t0);
    }
};

namespace irlba_gb300 {
namespace {

// pca() of matrix j through the single-matrix FP32 engine, outputs copied into
// the batch's device slots.
void solve_single(irlba_gb300_batch* b, int j, int32_t center, int32_t scale, int64_t number,
                  const irlba_gb300_options& opt, cudaStream_t s) {
    const int64_t m = b->m[j], n = b->n[j], nz = b->nnz[j];
    std::vector<int64_t> ptr(m + 1);
    std::vector<float> val(std::max<int64_t>(nz, 1));
    std::vector<int32_t> idx(std::max<int64_t>(nz, 1));
    const BatchDir d = b->dir(j, false);
    CUDA_TRY(d2h_async(ptr.data(), d.ptr, sizeof(int64_t) * (m + 1), s));
    if (nz) {
        CUDA_TRY(d2h_async(val.data(), d.val, sizeof(float) * nz, s));
        if (d.staged) {
            std::vector<uint16_t> i16(nz);
            CUDA_TRY(d2h_async(i16.data(), d.idx, sizeof(uint16_t) * nz, s));
            CUDA_TRY(cudaStreamSynchronize(s));
            for (int64_t e = 0; e < nz; ++e) idx[e] = i16[e];
        } else {
            CUDA_TRY(d2h_async(idx.data(), d.idx, sizeof(int32_t) * nz, s));
        }
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    irlba_gb300_matrix* mat = nullptr;
    irlba_gb300_status st = irlba_gb300_matrix_create_sparse(m, n, val.data(), IRLBA_GB300_VALUE_F32, idx.data(),
                                                             ptr.data(), 0, IRLBA_GB300_FORM_FP32_FP64STEPS, &mat);
    if (st != IRLBA_GB300_OK) throw Error(st, irlba_gb300_last_error());
    std::vector<double> sc(m * number), rot(n * number), var(number), cen(n), scl(n);
    int64_t out_number = 0;
    int32_t converged = 0, iterations = 0;
    irlba_gb300_stats stats;
    std::memset(&stats, 0, sizeof(stats));
    st = irlba_gb300_pca(mat, center, scale, number, &opt, sc.data(), rot.data(), var.data(), &out_number,
                         &converged, &iterations, center ? cen.data() : nullptr, scale ? scl.data() : nullptr,
                         &stats);
    const std::string msg = st == IRLBA_GB300_OK ? std::string() : std::string(irlba_gb300_last_error());
    irlba_gb300_matrix_destroy(mat);
    irlba_gb300_batch_info& inf = b->info[j];
    if (st != IRLBA_GB300_OK) {
        inf.status = IRLBA_GB300_BATCH_FAILED;
        inf.error = st;
        inf.converged = 0;
        return;
    }
    const BatchProblem& P = b->probs[j];
    const int64_t num = std::min(out_number, number);
    if (num * m > 0) CUDA_TRY(h2d_async(P.scores, sc.data(), sizeof(double) * m * num, s));
    if (num * n > 0) CUDA_TRY(h2d_async(P.rotation, rot.data(), sizeof(double) * n * num, s));
    if (num) CUDA_TRY(h2d_async(P.variances, var.data(), sizeof(double) * num, s));
    if (center && n) CUDA_TRY(h2d_async(P.center64, cen.data(), sizeof(double) * n, s));
    if (scale && n) CUDA_TRY(h2d_async(P.scale64, scl.data(), sizeof(double) * n, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    inf.status = IRLBA_GB300_BATCH_SINGLE;
    inf.error = 0;
    inf.converged = converged;
    inf.iterations = iterations;
    inf.lanczos_steps = stats.lanczos_steps;
    inf.svd_sweeps = stats.svd_sweeps;
    inf.ms = stats.device_ms;
}

bool requested_ge_half_b(int64_t requested, int64_t smaller) {
    const int64_t half = smaller / 2;
    if (requested == half) return smaller % 2 == 0;
    return requested > half;
}

}  // namespace
}  // namespace irlba_gb300

extern "C" {

irlba_gb300_status irlba_gb300_batch_create(int32_t count, const int64_t* nrow, const int64_t* ncol,
                                            const void* const* values, irlba_gb300_value_type value_type,
                                            const int32_t* const* indices, const int64_t* const* pointers,
                                            int32_t column_major, irlba_gb300_batch** out) {
    return guarded([&]() {
        if (!out) invalid("output handle pointer is NULL");
        *out = nullptr;
        if (count < 0) invalid("count must be non-negative");
        if (count > 0 && (!nrow || !ncol || !values || !indices || !pointers)) invalid("array arguments must not be NULL");
        if (value_type != IRLBA_GB300_VALUE_F32 && value_type != IRLBA_GB300_VALUE_F64) invalid("unknown value type");
        std::unique_ptr<irlba_gb300_batch> b(new irlba_gb300_batch());
        b->count = count;
        b->ingest(nrow, ncol, values, value_type == IRLBA_GB300_VALUE_F64, indices, pointers, column_major != 0);
        *out = b.release();
    });
}

irlba_gb300_status irlba_gb300_batch_destroy(irlba_gb300_batch* batch) {
    delete batch;
    return IRLBA_GB300_OK;
}

irlba_gb300_status irlba_gb300_batch_groups(const irlba_gb300_batch* batch, int32_t* group_mul, int32_t* group_adj) {
    return guarded([&]() {
        if (!batch) invalid("batch is NULL");
        if (group_mul) std::copy(batch->g_mul.begin(), batch->g_mul.end(), group_mul);
        if (group_adj) std::copy(batch->g_adj.begin(), batch->g_adj.end(), group_adj);
    });
}

irlba_gb300_status irlba_gb300_batch_set_groups(irlba_gb300_batch* batch, const int32_t* group_mul,
                                                const int32_t* group_adj) {
    return guarded([&]() {
        if (!batch) invalid("batch is NULL");
        auto check = [&](const int32_t* g) {
            if (!g) return;
            for (int j = 0; j < batch->count; ++j)
                if (g[j] != 4 && g[j] != 8 && g[j] != 16 && g[j] != 32) invalid("lanes per row must be 4, 8, 16 or 32");
        };
        check(group_mul);
        check(group_adj);
        if (group_mul) std::copy(group_mul, group_mul + batch->count, batch->g_mul.begin());
        if (group_adj) std::copy(group_adj, group_adj + batch->count, batch->g_adj.begin());
        ++batch->sched_version;
        batch->groups_fixed = true;
        batch->tuned = true;
    });
}

irlba_gb300_status irlba_gb300_batch_pca(irlba_gb300_batch* b, int32_t center, int32_t scale, int64_t number,
                                         const irlba_gb300_options* options, irlba_gb300_batch_stats* stats,
                                         void* stream) {
    return guarded([&]() {
        if (!b) invalid("batch is NULL");
        irlba_gb300_options opt;
        if (options) opt = *options;
        else irlba_gb300_default_options(&opt);
        if (number < 0) invalid("requested number of singular values must be non-negative");
        const auto t_call = std::chrono::steady_clock::now();
        const int64_t launches0 = irlba_gb300_launch_count();
        StreamScope ss(stream);
        const cudaStream_t s = ss.s;
        const int count = b->count;

        // Per-matrix argument checks (pca.hpp:76-83, compute.hpp:153-170) and
        // the choice between the batched kernel and the single-matrix engine.
        const int64_t work = number + opt.extra_work;
        std::vector<uint8_t> batched(count, 0);
        for (int j = 0; j < count; ++j) {
            const int64_t mj = b->m[j], nj = b->n[j];
            const std::string who = "matrix " + std::to_string(j) + ": ";
            if (scale && mj < 2) invalid(who + "cannot scale with fewer than two observations");
            if (center && mj < 1) invalid(who + "cannot center with no observations");
            const int64_t smaller = std::min(mj, nj);
            int64_t requested = number;
            if (requested > smaller) {
                if (!opt.cap_number)
                    invalid(who + "requested number of singular values cannot be greater than the smaller matrix dimension");
                requested = smaller;
            } else if (requested == smaller && !opt.exact_for_large_number) {
                invalid(who + "requested number of singular values must be less than the smaller matrix dimension for IRLBA iterations");
            }
            const bool exact = (opt.exact_for_small_matrix && smaller < 6) ||
                               (opt.exact_for_large_number && requested_ge_half_b(requested, smaller));
            const int64_t wj = requested + std::min<int64_t>(smaller - requested, opt.extra_work);
            batched[j] = !exact && number > 0 && requested == number && wj == work && work <= kBatchMaxWork;
            if (opt.initial && opt.initial_size != nj)
                invalid(who + "initialization vector does not have expected number of rows");
        }
        const int32_t w32 = static_cast<int32_t>(std::min<int64_t>(std::max<int64_t>(work, 1), kBatchMaxWork));
        b->workspace(w32, number);

        // Start vectors: the same options give every matrix the vector that a
        // separate pca() call would draw (compute.hpp:179-190). Uploaded when
        // the workspace, the seed or the caller's initial vector changes.
        if (opt.initial || b->init_gen != b->ws_gen || b->init_seed != opt.seed || !b->init_random) {
            std::map<int64_t, std::vector<double>> by_n;
            bool any = false;
            for (int j = 0; j < count; ++j) {
                if (!batched[j]) continue;
                any = true;
                auto it = by_n.find(b->n[j]);
                if (it == by_n.end()) {
                    std::vector<double> v(b->n[j]);
                    if (opt.initial) {
                        std::copy(opt.initial, opt.initial + b->n[j], v.begin());
                    } else {
                        std::mt19937_64 eng(opt.seed);
                        fill_normals(v, eng);
                    }
                    it = by_n.emplace(b->n[j], std::move(v)).first;
                }
                CUDA_TRY(h2d_async(const_cast<double*>(b->probs[j].init), it->second.data(),
                                   sizeof(double) * b->n[j], s));
            }
            if (any) CUDA_TRY(cudaStreamSynchronize(s));
            b->init_gen = b->ws_gen;
            b->init_seed = opt.seed;
            b->init_random = opt.initial == nullptr;
        }

        // Largest first (longest-processing-time order): cost ~ stored entries
        // of both directions plus the dense work on the bases.
        b->order.clear();
        for (int j = 0; j < count; ++j)
            if (batched[j]) b->order.push_back(j);
        std::vector<int64_t> costs(count);
        for (int j = 0; j < count; ++j) costs[j] = 2 * b->nnz[j] + (b->m[j] + b->n[j]) * static_cast<int64_t>(w32) * 4;
        std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return costs[x] > costs[y]; });
        const int32_t active = static_cast<int32_t>(b->order.size());
        if (active) CUDA_TRY(h2d_async(b->order_dev.ptr, b->order.data(), sizeof(int32_t) * active, s));
        b->upload_problems_if_changed(s);

        double tune_ms = 0;
        if (!b->tuned && active) {
            tune_ms = b->tune(3, active, s);
            b->upload_problems_if_changed(s);
        }

        BatchParams prm;
        prm.number = static_cast<int32_t>(number);
        prm.work = w32;
        prm.max_iter = opt.max_iterations;
        prm.center = center;
        prm.scale = scale;
        prm.tol = opt.convergence_tolerance;
        prm.svtol = opt.singular_value_ratio_tolerance >= 0 ? opt.singular_value_ratio_tolerance
                                                            : opt.convergence_tolerance;
        prm.eps = opt.invariant_subspace_tolerance < 0 ? std::pow(std::numeric_limits<double>::epsilon(), 0.8)
                                                       : opt.invariant_subspace_tolerance;
        const size_t smem = batch_smem_bytes(b->max_staged);
        int teams = 1, n_joint = 0;
        const int team = active ? b->choose_team(active, costs, smem, &teams, &n_joint) : 1;
        const int grid = teams * team;
        int captured = 0;
        float dev_ms = 0;
        if (active) {
            const bool same = b->exec && b->graph_gen == b->ws_gen && b->graph_grid == grid &&
                              b->graph_team == team && b->graph_joint == n_joint && b->graph_smem == smem &&
                              b->graph_count == active &&
                              std::memcmp(&b->graph_prm, &prm, sizeof(prm)) == 0;
            if (!same) {
                if (b->exec) cudaGraphExecDestroy(b->exec);
                b->exec = nullptr;
                cudaStream_t cs;
                CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
                cudaGraph_t graph = nullptr;
                cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    cudaMemsetAsync(b->queue_dev.ptr, 0, sizeof(uint32_t), cs);
                    launch_batch_pca(team, b->probs_dev.as<BatchProblem>(), b->order_dev.as<int32_t>(), active,
                                     n_joint, prm, b->results_dev.as<BatchResult>(), b->queue_dev.as<uint32_t>(),
                                     teams, smem, cs);
                    e = cudaStreamEndCapture(cs, &graph);
                }
                if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, graph, 0);
                if (graph) cudaGraphDestroy(graph);
                cudaStreamDestroy(cs);
                CUDA_TRY(e);
                b->graph_prm = prm;
                b->graph_grid = grid;
                b->graph_team = team;
                b->graph_joint = n_joint;
                b->graph_smem = smem;
                b->graph_count = active;
                b->graph_gen = b->ws_gen;
                captured = 1;
            }
            cudaEvent_t e0, e1;
            CUDA_TRY(cudaEventCreate(&e0));
            CUDA_TRY(cudaEventCreate(&e1));
            CUDA_TRY(cudaEventRecord(e0, s));
            CUDA_TRY(cudaGraphLaunch(b->exec, s));
            count_launch();
            CUDA_TRY(cudaEventRecord(e1, s));
            CUDA_TRY(cudaStreamSynchronize(s));
            CUDA_TRY(cudaGetLastError());
            cudaEventElapsedTime(&dev_ms, e0, e1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            CUDA_TRY(d2h_async(b->results.data(), b->results_dev.ptr, sizeof(BatchResult) * count, s));
            CUDA_TRY(cudaStreamSynchronize(s));
        }

        int single = 0;
        int64_t steps = 0;
        const auto t_single = std::chrono::steady_clock::now();
        for (int j = 0; j < count; ++j) {
            irlba_gb300_batch_info& inf = b->info[j];
            std::memset(&inf, 0, sizeof(inf));
            inf.group_mul = b->g_mul[j];
            inf.group_adj = b->g_adj[j];
            inf.prefetch_mul = b->pf_mul[j];
            inf.prefetch_adj = b->pf_adj[j];
            if (batched[j] && b->results[j].status == 0) {
                const BatchResult& r = b->results[j];
                inf.status = IRLBA_GB300_BATCH_OK;
                inf.converged = r.converged;
                inf.iterations = r.iterations;
                inf.lanczos_steps = r.steps;
                inf.svd_sweeps = r.svd_sweeps;
                inf.ms = static_cast<double>(r.t_end - r.t_start) * 1e-6;
                steps += r.steps;
            } else {
                solve_single(b, j, center, scale, number, opt, s);
                ++single;
            }
        }
        const double single_ms = single ? ms_since(t_single) : 0.0;
        b->last_number = number;
        b->last_center = center;
        b->last_scale = scale;
        b->have_results = true;
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->device_ms = dev_ms;
            stats->tune_ms = tune_ms;
            stats->single_ms = single_ms;
            stats->kernel_launches = irlba_gb300_launch_count() - launches0;
            stats->graph_captured = captured;
            stats->single = single;
            stats->ctas = active ? grid : 0;
            stats->team = active ? team : 0;
            stats->joint = active ? n_joint : 0;
            stats->nnz = b->total_nnz;
            stats->lanczos_steps = steps;
        }
        (void)t_call;
    });
}

irlba_gb300_status irlba_gb300_batch_set_team(irlba_gb300_batch* b, int32_t team, int32_t joint) {
    return guarded([&]() {
        if (!b) invalid("batch is NULL");
        if (team != 0 && team != 1 && team != 2 && team != 4 && team != 8)
            invalid("team must be 0 (automatic), 1, 2, 4 or 8");
        b->team_request = team;
        b->joint_request = joint < 0 ? -1 : joint;
    });
}

irlba_gb300_status irlba_gb300_batch_tune(irlba_gb300_batch* b, int32_t repeats, void* stream) {
    return guarded([&]() {
        if (!b) invalid("batch is NULL");
        if (b->ws_work < 0) invalid("tuning needs a workspace: call irlba_gb300_batch_pca first");
        StreamScope ss(stream);
        b->tuned = false;
        b->groups_fixed = false;
        b->upload_problems_if_changed(ss.s);
        b->tune(repeats, static_cast<int32_t>(b->order.size()), ss.s);
        b->upload_problems_if_changed(ss.s);
    });
}

irlba_gb300_status irlba_gb300_batch_result(const irlba_gb300_batch* b, int32_t index, double* scores,
                                            double* rotation, double* variances, double* center, double* scale,
                                            irlba_gb300_batch_info* info) {
    return guarded([&]() {
        if (!b) invalid("batch is NULL");
        if (index < 0 || index >= b->count) invalid("matrix index out of range");
        if (!b->have_results) invalid("no results: call irlba_gb300_batch_pca first");
        const BatchProblem& P = b->probs[index];
        const int64_t m = b->m[index], n = b->n[index], num = b->last_number;
        if (scores && m * num > 0) CUDA_TRY(d2h_sync(scores, P.scores, sizeof(double) * m * num));
        if (rotation && n * num > 0) CUDA_TRY(d2h_sync(rotation, P.rotation, sizeof(double) * n * num));
        if (variances && num) CUDA_TRY(d2h_sync(variances, P.variances, sizeof(double) * num));
        if (center && b->last_center && n) CUDA_TRY(d2h_sync(center, P.center64, sizeof(double) * n));
        if (scale && b->last_scale && n) CUDA_TRY(d2h_sync(scale, P.scale64, sizeof(double) * n));
        if (info) *info = b->info[index];
    });
}

irlba_gb300_status irlba_gb300_batch_result_device(const irlba_gb300_batch* b, int32_t index, const double** scores,
                                                   const double** rotation, const double** variances) {
    return guarded([&]() {
        if (!b) invalid("batch is NULL");
        if (index < 0 || index >= b->count) invalid("matrix index out of range");
        if (!b->have_results) invalid("no results: call irlba_gb300_batch_pca first");
        const BatchProblem& P = b->probs[index];
        if (scores) *scores = P.scores;
        if (rotation) *rotation = P.rotation;
        if (variances) *variances = P.variances;
    });
}

}  // extern "C"
