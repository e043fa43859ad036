#pragma once
#include "_shim_common.h"
namespace tbb {
template <typename T>
class concurrent_bounded_queue {
    std::deque<T> q_;
    std::mutex m_;
    std::condition_variable cv_not_empty_, cv_not_full_;
    std::ptrdiff_t cap_;
public:
    concurrent_bounded_queue() : cap_(-1) {}
    void set_capacity(std::ptrdiff_t c) { std::lock_guard<std::mutex> l(m_); cap_ = c; }
    void push(const T &v) {
        std::unique_lock<std::mutex> l(m_);
        cv_not_full_.wait(l, [&] { return cap_ < 0 || (std::ptrdiff_t)q_.size() < cap_; });
        q_.push_back(v);
        cv_not_empty_.notify_one();
    }
    void pop(T &v) {
        std::unique_lock<std::mutex> l(m_);
        cv_not_empty_.wait(l, [&] { return !q_.empty(); });
        v = q_.front();
        q_.pop_front();
        cv_not_full_.notify_one();
    }
    bool try_pop(T &v) {
        std::lock_guard<std::mutex> l(m_);
        if (q_.empty()) return false;
        v = q_.front();
        q_.pop_front();
        cv_not_full_.notify_one();
        return true;
    }
    bool pop_if_present(T &v) { return try_pop(v); }
    std::ptrdiff_t size() { std::lock_guard<std::mutex> l(m_); return (std::ptrdiff_t)q_.size(); }
    bool empty() { return size() == 0; }
    void clear() { std::lock_guard<std::mutex> l(m_); q_.clear(); }
};
}  // namespace tbb
