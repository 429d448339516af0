// Host-side helpers shared by the library's translation units.
#pragma once

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstddef>
#include <cstdint>
#include <thread>
#include <vector>

namespace bclbm {
namespace host {

// fn(begin, end) over [0, n) on the host cores, in contiguous chunks of at
// least `grain` items
template <class F>
void parallel_for(size_t n, F&& fn, size_t grain = 32768) {
    const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    const size_t nt = std::min<size_t>(hw, (n + grain - 1) / grain);
    if (nt <= 1) {
        fn(size_t(0), n);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(nt - 1);
    for (size_t t = 1; t < nt; ++t) th.emplace_back([&fn, n, t, nt] { fn(n * t / nt, n * (t + 1) / nt); });
    fn(size_t(0), n / nt);
    for (auto& x : th) x.join();
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
