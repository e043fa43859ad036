#pragma once
#include "_shim_common.h"
namespace tbb {
class filter {
    bool serial_;
public:
    explicit filter(bool is_serial) : serial_(is_serial) {}
    virtual ~filter() {}
    bool is_serial() const { return serial_; }
    virtual void *operator()(void *item) = 0;
};
// Runs up to max_tokens items through the filter chain at once, one worker
// thread per token, each taking an item from the first filter and carrying
// it through the rest. Serial filters are guarded by a per-filter mutex.
class pipeline {
    std::vector<filter *> f_;
public:
    void add_filter(filter &f) { f_.push_back(&f); }
    void clear() { f_.clear(); }
    void run(std::size_t max_tokens) {
        if (f_.empty()) return;
        std::vector<std::mutex> locks(f_.size());
        std::mutex first_lock;
        auto worker = [&]() {
            for (;;) {
                void *item;
                {
                    std::lock_guard<std::mutex> l(first_lock);
                    item = (*f_[0])(nullptr);
                }
                if (!item) break;
                for (std::size_t i = 1; i < f_.size() && item; ++i) {
                    if (f_[i]->is_serial()) {
                        std::lock_guard<std::mutex> l(locks[i]);
                        item = (*f_[i])(item);
                    } else {
                        item = (*f_[i])(item);
                    }
                }
            }
        };
        std::size_t nt = max_tokens;
        std::size_t hw = (std::size_t)shim::thread_count();
        if (nt > hw) nt = hw;
        if (nt < 1) nt = 1;
        std::vector<std::thread> th;
        for (std::size_t i = 1; i < nt; ++i) th.emplace_back(worker);
        worker();
        for (auto &t : th) t.join();
    }
};
}  // namespace tbb
