// host_threads.hpp -- a parallel loop over host threads for the set-up code (tree build,
// table conversions).  Outputs of each index have fixed places, so results do not depend on
// the number of threads.
#pragma once
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

namespace ifgf {

constexpr int kMaxThreads = 32;

// upper bound on the threads one set-up call uses (ifgf2d_set_host_threads); 0 = all cores.
// Callers that set up many contexts at once from their own threads set it to 1.
inline std::atomic<int>& host_thread_limit() {
    static std::atomic<int> n{0};
    return n;
}

// f(begin, end) over [0, n) in contiguous chunks of at least `grain` indices, on up to
// hardware_concurrency threads
template <class F>
void parallel_for(long long n, F&& f, long long grain = 1024) {
    unsigned hw = std::max(1u, std::min((unsigned)kMaxThreads, std::thread::hardware_concurrency()));
    const int lim = host_thread_limit().load(std::memory_order_relaxed);
    if (lim > 0) hw = std::min(hw, (unsigned)lim);
    const long long nt = std::min<long long>(hw, (n + grain - 1) / grain);
    if (nt <= 1) { f(0LL, n); return; }
    std::vector<std::thread> th;
    const long long chunk = (n + nt - 1) / nt;
    for (long long t = 0; t < nt; ++t) {
        const long long b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

}  // namespace ifgf
