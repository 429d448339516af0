// Host-side helpers shared by the library's translation units.
#pragma once

#include <algorithm>
#include <atomic>
#include <climits>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace bclbm {
namespace host {

// Persistent host worker threads for parallel_for: starting threads on every call
// cost as much as the loops it splits (about 1 ms for a 27 MB scan at 16 threads).
// One loop runs on the pool at a time; a loop started while it is busy (a nested
// loop, or another host thread's) runs on its caller's thread alone.  The workers
// sleep on a condition variable and are never joined, so no static destructor
// waits for them.
class Pool {
  public:
    static Pool& get() {
        static Pool* p = new Pool();
        return *p;
    }
    size_t workers() const { return nw_; }
    // fn(t) for t in [0, n) with the caller taking part; false when the pool is busy
    bool run(size_t n, const std::function<void(size_t)>& fn) {
        bool expected = false;
        if (!busy_.compare_exchange_strong(expected, true)) return false;
        Job j(&fn, n);
        {
            std::lock_guard<std::mutex> l(m_);
            job_ = &j;
            ++gen_;
        }
        wake_.notify_all();
        work(j);
        {
            std::unique_lock<std::mutex> l(m_);
            job_ = nullptr;  // a worker waking from now on finds no job
            done_.wait(l, [&] { return j.active == 0; });
        }
        busy_.store(false);
        return true;
    }

  private:
    struct Job {
        Job(const std::function<void(size_t)>* f, size_t count) : fn(f), n(count) {}
        const std::function<void(size_t)>* fn;
        size_t n;
        std::atomic<size_t> next{0};
        int active = 0;  // workers inside work(), counted under m_
    };
    Pool() {
        const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
        nw_ = hw - 1;
        for (unsigned i = 0; i < nw_; ++i) std::thread([this] { loop(); }).detach();
    }
    static void work(Job& j) {
        for (size_t t; (t = j.next.fetch_add(1)) < j.n;) (*j.fn)(t);
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            Job* j;
            {
                std::unique_lock<std::mutex> l(m_);
                wake_.wait(l, [&] { return gen_ != seen; });
                seen = gen_;
                j = job_;
                if (!j) continue;
                ++j->active;
            }
            work(*j);
            {
                std::lock_guard<std::mutex> l(m_);
                --j->active;
            }
            done_.notify_all();
        }
    }
    std::mutex m_;
    std::condition_variable wake_, done_;
    Job* job_ = nullptr;
    uint64_t gen_ = 0;
    std::atomic<bool> busy_{false};
    size_t nw_ = 0;
};

// fn(begin, end) over [0, n) on the host cores, in contiguous chunks of at
// least `grain` items
template <class F>
void parallel_for(size_t n, F&& fn, size_t grain = 32768) {
    Pool& pool = Pool::get();
    const size_t nt = std::min<size_t>(pool.workers() + 1, (n + grain - 1) / grain);
    if (nt <= 1) {
        fn(size_t(0), n);
        return;
    }
    const std::function<void(size_t)> task = [&fn, n, nt](size_t t) { fn(n * t / nt, n * (t + 1) / nt); };
    if (!pool.run(nt, task)) fn(size_t(0), n);
}

// smallest index at which a parallel check failed (INT64_MAX: none)
struct FirstBad {
    std::atomic<int64_t> v{INT64_MAX};
    void set(int64_t i) {
        int64_t cur = v.load();
        while (i < cur && !v.compare_exchange_weak(cur, i)) {
        }
    }
    bool any() const { return v.load() != INT64_MAX; }
    int64_t get() const { return v.load(); }
};

}  // namespace host
}  // namespace bclbm
