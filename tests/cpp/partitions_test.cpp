// Host thread partitions that the drop-in ParallelSparseMatrix reports through
// get_primary_boundaries / get_secondary_boundaries /
// get_secondary_nonzero_boundaries (irlba::gpu::thread_partitions). Prints
// seeded sparse matrices and their partitions as JSON for
// tests/test_capi_cpu.py, which compares them with the oracle's.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "irlba_gb300/irlba.hpp"

static uint64_t state = 0x9E3779B97F4A7C15ull;
static double uniform() {
    state = state * 6364136223846793005ull + 1442695040888963407ull;
    return static_cast<double>(state >> 11) * (1.0 / 9007199254740992.0);
}

static void print_ints(const char* name, const std::vector<int64_t>& v) {
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%lld", i ? ", " : "", static_cast<long long>(v[i]));
    std::printf("]");
}

int main() {
    // (rows, cols, density, threads...): the drop-in GPU test's 120 x 70 shape
    // with 4 threads, uneven shapes, empty primary elements, more threads than
    // nonzeros.
    struct Case {
        int nr, nc;
        double density;
        std::vector<int> threads;
    };
    const std::vector<Case> cases = {{120, 70, 0.2, {2, 4}}, {37, 91, 0.15, {3, 7}}, {200, 5, 0.05, {4, 16}},
                                     {9, 8, 0.02, {5}}};
    std::printf("[\n");
    for (size_t ci = 0; ci < cases.size(); ++ci) {
        const Case& cs = cases[ci];
        // Column-major (CSC): primary = columns.
        std::vector<int64_t> ptr(1, 0), idx64;
        std::vector<int32_t> idx;
        for (int c = 0; c < cs.nc; ++c) {
            for (int r = 0; r < cs.nr; ++r)
                if (uniform() < cs.density) {
                    idx.push_back(r);
                    idx64.push_back(r);
                }
            ptr.push_back(static_cast<int64_t>(idx.size()));
        }
        std::printf("{\"nrow\": %d, \"ncol\": %d, ", cs.nr, cs.nc);
        print_ints("ptr", ptr);
        std::printf(", ");
        print_ints("idx", idx64);
        std::printf(", \"parts\": {");
        for (size_t ti = 0; ti < cs.threads.size(); ++ti) {
            const int nt = cs.threads[ti];
            const irlba::gpu::ThreadPartitions p = irlba::gpu::thread_partitions(cs.nc, cs.nr, ptr.data(), idx.data(), nt);
            std::vector<int64_t> prim(p.primary.begin(), p.primary.end()), sec(p.secondary.begin(), p.secondary.end()),
                snz;
            for (const auto& row : p.secondary_nonzero) snz.insert(snz.end(), row.begin(), row.end());
            std::printf("%s\"%d\": {", ti ? ", " : "", nt);
            print_ints("primary", prim);
            std::printf(", ");
            print_ints("secondary", sec);
            std::printf(", ");
            print_ints("secondary_nonzero", snz);
            std::printf("}");
        }
        std::printf("}}%s\n", ci + 1 < cases.size() ? "," : "");
    }
    std::printf("]\n");
    return 0;
}
