// Seeded synthetic single-cell-like count matrices (host C++, multithreaded).
//
// No public dataset is used by CppIrlba; these synthetic matrices stand in for
// the sparse log-count inputs that its ParallelSparseMatrix path is built for.
//
// Value model, per gene g of G genes and cell c of C cells:
//   mu_g  = exp(mu + sigma * z_g),  z_g ~ N(0, 1)            (per-gene mean)
//   entry (g, c) present with probability `density`, independently
//   X     ~ NegativeBinomial(mean mu_g, size 1/phi) conditioned on X >= 1
//   value = log1p(X)
// Conditioning on X >= 1 keeps the stated density exact in expectation while
// drawing the non-zero counts from the negative-binomial tail. X is drawn by
// inversion of the zero-truncated CDF (pmf recurrence
// p(x+1) = p(x) (x + r)/(x + 1) * mu/(mu + r), r = 1/phi).
// Present cells are drawn by geometric skipping (gap = floor(log u / log(1-p))).
//
// Random streams: std::mt19937_64, one engine per gene for positions and one for
// values, seeded from splitmix64(seed, gene, stream). Uniforms are 53-bit, in
// (0, 1]. Normals use Box-Muller. Output is gene-major CSR (genes x cells):
// ptr[G+1] (int64), idx (int32 cell), values (float32 or float64).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <thread>
#include <vector>
#include <algorithm>
#include <atomic>

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline uint64_t stream_seed(uint64_t seed, uint64_t gene, uint64_t stream) {
    return splitmix64(splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + gene);
}

inline double uniform01(std::mt19937_64& eng) {
    return (static_cast<double>(eng() >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

inline double normal(std::mt19937_64& eng) {
    const double u1 = uniform01(eng), u2 = uniform01(eng);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

struct Params {
    int64_t genes, cells;
    double density, mu, sigma, phi;
    uint64_t seed;
};

// Next present cell after `pos` (or -1 at start); returns >= cells when done.
inline int64_t next_present(std::mt19937_64& eng, int64_t pos, double log1mp, double density) {
    if (density >= 1.0) return pos + 1;
    const double u = uniform01(eng);
    const double gap = std::floor(std::log(u) / log1mp);
    if (gap > 9.0e15) return INT64_MAX / 2;
    return pos + 1 + static_cast<int64_t>(gap);
}

inline double truncated_nb(std::mt19937_64& eng, double mean, double size) {
    const double q = mean / (mean + size);
    double p = std::pow(size / (size + mean), size);  // P(X = 0)
    const double u = uniform01(eng);
    const double target = p + u * (1.0 - p);
    double cdf = p;
    double x = 0;
    for (int it = 0; it < 10000000; ++it) {
        p *= (x + size) / (x + 1.0) * q;
        x += 1.0;
        cdf += p;
        if (cdf >= target || p == 0.0) break;
    }
    return x < 1.0 ? 1.0 : x;
}

template <typename F>
void parallel_for(int64_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 2) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> pool;
    std::atomic<int64_t>* next = new std::atomic<int64_t>(0);
    for (int t = 0; t < nthreads; ++t) {
        pool.emplace_back([&, next]() {
            while (true) {
                const int64_t i = next->fetch_add(1);
                if (i >= n) break;
                f(i);
            }
        });
    }
    for (auto& th : pool) th.join();
    delete next;
}

}  // namespace

extern "C" {

// Per-gene means mu_g (length genes).
void irlba_gb300_datagen_gene_means(int64_t genes, double mu, double sigma, uint64_t seed, double* out) {
    std::mt19937_64 eng(stream_seed(seed, 0, 7));
    for (int64_t g = 0; g < genes; ++g) out[g] = std::exp(mu + sigma * normal(eng));
}

// Pass 1: number of present cells per gene (ptr must hold genes + 1 entries;
// ptr[0] = 0 and ptr[g + 1] = cumulative count). Returns total nnz.
int64_t irlba_gb300_datagen_counts(int64_t genes, int64_t cells, double density, uint64_t seed, int nthreads,
                                   int64_t* ptr) {
    const double log1mp = std::log1p(-std::min(density, 0.999999999));
    std::vector<int64_t> counts(genes, 0);
    parallel_for(genes, nthreads, [&](int64_t g) {
        std::mt19937_64 eng(stream_seed(seed, static_cast<uint64_t>(g), 1));
        int64_t n = 0;
        int64_t pos = next_present(eng, -1, log1mp, density);
        while (pos < cells) {
            ++n;
            pos = next_present(eng, pos, log1mp, density);
        }
        counts[g] = n;
    });
    ptr[0] = 0;
    for (int64_t g = 0; g < genes; ++g) ptr[g + 1] = ptr[g] + counts[g];
    return ptr[genes];
}

// Pass 2: fill indices and values (value_bytes 4 -> float32, 8 -> float64).
void irlba_gb300_datagen_fill(int64_t genes, int64_t cells, double density, double mu, double sigma, double phi,
                              uint64_t seed, int nthreads, const int64_t* ptr, int32_t* idx, void* values,
                              int value_bytes) {
    const double log1mp = std::log1p(-std::min(density, 0.999999999));
    std::vector<double> means(genes);
    irlba_gb300_datagen_gene_means(genes, mu, sigma, seed, means.data());
    const double size = 1.0 / phi;
    parallel_for(genes, nthreads, [&](int64_t g) {
        std::mt19937_64 epos(stream_seed(seed, static_cast<uint64_t>(g), 1));
        std::mt19937_64 eval(stream_seed(seed, static_cast<uint64_t>(g), 2));
        int64_t s = ptr[g];
        const int64_t end = ptr[g + 1];
        int64_t pos = next_present(epos, -1, log1mp, density);
        while (pos < cells && s < end) {
            const double x = truncated_nb(eval, means[g], size);
            const double v = std::log1p(x);
            idx[s] = static_cast<int32_t>(pos);
            if (value_bytes == 4) static_cast<float*>(values)[s] = static_cast<float>(v);
            else static_cast<double*>(values)[s] = v;
            ++s;
            pos = next_present(epos, pos, log1mp, density);
        }
    });
}

// Transpose a compressed matrix (primary x secondary) into (secondary x primary),
// keeping indices sorted within each output primary element. value_bytes 4 or 8.
void irlba_gb300_transpose_compressed(int64_t primary, int64_t secondary, const int64_t* ptr, const int32_t* idx,
                                      const void* values, int value_bytes, int64_t* tptr, int32_t* tidx,
                                      void* tvalues) {
    std::vector<int64_t> fill(secondary + 1, 0);
    const int64_t nnz = ptr[primary];
    for (int64_t s = 0; s < nnz; ++s) ++fill[idx[s] + 1];
    for (int64_t j = 0; j < secondary; ++j) fill[j + 1] += fill[j];
    std::memcpy(tptr, fill.data(), sizeof(int64_t) * (secondary + 1));
    for (int64_t p = 0; p < primary; ++p) {
        for (int64_t s = ptr[p]; s < ptr[p + 1]; ++s) {
            const int64_t dst = fill[idx[s]]++;
            tidx[dst] = static_cast<int32_t>(p);
            if (value_bytes == 4) static_cast<float*>(tvalues)[dst] = static_cast<const float*>(values)[s];
            else static_cast<double*>(tvalues)[dst] = static_cast<const double*>(values)[s];
        }
    }
}

}  // extern "C"
