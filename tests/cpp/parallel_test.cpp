// irlba::parallelize and irlba::EigenThreadScope of the drop-in, reached
// through CppIrlba's own umbrella header name (include/irlba/irlba.hpp). Built
// twice by tests/test_capi_cpu.py: with the default worker threads, and with a
// caller-defined IRLBA_CUSTOM_PARALLEL (the reference's hook, parallel.hpp:32-40).
#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <vector>

#ifdef USE_CUSTOM_RUNNER
static std::atomic<int> custom_calls{0};
template <typename Task_, class Run_>
void custom_runner(Task_ n, Run_ f) {
    ++custom_calls;
    for (Task_ t = 0; t < n; ++t) f(t);
}
#define IRLBA_CUSTOM_PARALLEL(n, f) custom_runner(n, f)
#endif

#include "irlba/irlba.hpp"

int main() {
    std::vector<int> out(7, -1);
    irlba::parallelize(7, [&](int t) { out[t] = t * t; });
    for (int t = 0; t < 7; ++t)
        if (out[t] != t * t) return 1;
    irlba::parallelize(0, [&](int) { out[0] = -5; });
    if (out[0] != 0) return 2;
#ifdef USE_CUSTOM_RUNNER
    if (custom_calls.load() != 2) return 3;
#else
    bool threw = false;
    try {
        irlba::parallelize(3, [&](int t) {
            if (t == 2) throw std::runtime_error("task failed");
        });
    } catch (const std::runtime_error&) {
        threw = true;
    }
    if (!threw) return 4;
#endif
    {
        irlba::EigenThreadScope scope(4);
        irlba::EigenThreadScope other = 2;
        (void)scope;
        (void)other;
    }
    std::printf("ok\n");
    return 0;
}
