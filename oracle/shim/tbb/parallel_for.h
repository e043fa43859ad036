#pragma once
#include "_shim_common.h"
#include "blocked_range.h"
namespace tbb {
class auto_partitioner {};
// Dynamic chunked parallel_for over shim::thread_count() threads. Each chunk
// is a sub-range of at most the grain size (or size/(4*threads) for the
// automatic partitioner); the body is copied per worker as TBB does.
template <typename Value, typename Body>
void _shim_parallel_for(const blocked_range<Value> &r, const Body &body, std::size_t grain) {
    const std::size_t n = r.size();
    if (n == 0) return;
    int nt = shim::thread_count();
    if (nt <= 1 || n <= grain) { Body b(body); b(r); return; }
    std::atomic<std::size_t> next(0);
    auto worker = [&]() {
        Body b(body);
        for (;;) {
            std::size_t s = next.fetch_add(grain);
            if (s >= n) break;
            std::size_t e = s + grain < n ? s + grain : n;
            b(blocked_range<Value>(r.begin() + (Value)s, r.begin() + (Value)e, grain));
        }
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
}
template <typename Value, typename Body>
void parallel_for(const blocked_range<Value> &r, const Body &body) {
    _shim_parallel_for(r, body, r.grainsize());
}
template <typename Value, typename Body>
void parallel_for(const blocked_range<Value> &r, const Body &body, const auto_partitioner &) {
    std::size_t nt = (std::size_t)shim::thread_count();
    std::size_t g = r.size() / (4 * nt);
    _shim_parallel_for(r, body, g ? g : 1);
}
}  // namespace tbb
