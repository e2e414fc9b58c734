// host_threads.hpp -- a parallel loop over host threads for the set-up code (tree build,
// table conversions).  Outputs of each index have fixed places, so results do not depend on
// the number of threads.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <pthread.h>
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

// Worker threads kept for the life of the process: a set-up runs a hundred or more parallel
// loops, and creating and joining threads for each one cost tens of milliseconds in a process
// that holds a CUDA context.  One loop runs on the pool at a time; a loop that finds it busy
// (another caller's, or a loop nested in a worker) starts threads of its own instead.  Chunks
// are claimed from a ticket that carries the loop's generation, so a worker still finishing an
// earlier loop can never claim a chunk of the next one.
class HostPool {
public:
    static HostPool& get() {
        static HostPool* p = new HostPool;   // never destroyed: the workers wait until process exit
        return *p;
    }
    // false in a child process after fork(): the child has none of the workers, and a lock
    // that another thread held at the fork stays held, so the child starts threads per loop
    static bool usable() { return !forked().load(std::memory_order_relaxed); }
    // true on a thread that is running a chunk of a pool loop (a nested loop must not use the pool)
    static bool& inside() {
        static thread_local bool v = false;
        return v;
    }
    // f(begin, end) over nt chunks of `chunk` indices of [0, n); false when the pool is busy
    bool run(long long n, long long chunk, int nt, const std::function<void(long long, long long)>& f) {
        std::unique_lock<std::mutex> busy(run_mutex_, std::try_to_lock);
        if (!busy.owns_lock()) return false;
        grow(nt - 1);
        Job j{&f, n, chunk, nt};
        unsigned long long gen;
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = j;
            gen = ++gen_;
            left_ = nt;
            ticket_.store(gen << 32);
        }
        cv_.notify_all();
        work(gen, j);
        std::unique_lock<std::mutex> g(m_);
        done_cv_.wait(g, [&] { return left_ == 0; });
        return true;
    }

private:
    struct Job {
        const std::function<void(long long, long long)>* f;
        long long n, chunk;
        int nchunks;
    };
    HostPool() {
        static std::once_flag once;
        std::call_once(once, [] { pthread_atfork(nullptr, nullptr, [] { forked().store(true); }); });
    }
    static std::atomic<bool>& forked() {
        static std::atomic<bool> f{false};
        return f;
    }
    void grow(int want) {
        while ((int)workers_.size() < want) {
            workers_.emplace_back([this] { loop(); });
            workers_.back().detach();
        }
    }
    // claim chunks of loop `gen` until none is left; the last one done wakes the caller
    void work(unsigned long long gen, const Job& j) {
        for (;;) {
            unsigned long long v = ticket_.load();
            for (;;) {
                if ((v >> 32) != gen || (long long)(v & 0xffffffffull) >= j.nchunks) return;
                if (ticket_.compare_exchange_weak(v, v + 1)) break;
            }
            const long long c = (long long)(v & 0xffffffffull);
            const long long b = c * j.chunk, e = std::min(j.n, b + j.chunk);
            if (b < e) {
                inside() = true;
                (*j.f)(b, e);
                inside() = false;
            }
            std::lock_guard<std::mutex> g(m_);
            if (--left_ == 0) done_cv_.notify_one();
        }
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [&] { return gen_ != seen; });
                seen = gen_;
                j = job_;
            }
            work(seen, j);
        }
    }
    std::mutex run_mutex_, m_;
    std::condition_variable cv_, done_cv_;
    std::vector<std::thread> workers_;
    Job job_{nullptr, 0, 0, 0};
    unsigned long long gen_ = 0;
    int left_ = 0;
    std::atomic<unsigned long long> ticket_{0};
};

// f(begin, end) over [0, n) in contiguous chunks of at least `grain` indices, on up to
// hardware_concurrency threads
template <class F>
void parallel_for(long long n, F&& f, long long grain = 1024) {
    unsigned hw = std::max(1u, std::min((unsigned)kMaxThreads, std::thread::hardware_concurrency()));
    const int lim = host_thread_limit().load(std::memory_order_relaxed);
    if (lim > 0) hw = std::min(hw, (unsigned)lim);
    const long long nt = std::min<long long>(hw, (n + grain - 1) / grain);
    if (nt <= 1) { f(0LL, n); return; }
    const long long chunk = (n + nt - 1) / nt;
    const std::function<void(long long, long long)> job = [&f](long long b, long long e) { f(b, e); };
    if (!HostPool::inside() && HostPool::usable() && HostPool::get().run(n, chunk, (int)nt, job)) return;
    std::vector<std::thread> th;
    for (long long t = 0; t < nt; ++t) {
        const long long b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

}  // namespace ifgf
