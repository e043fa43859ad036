#pragma once
#include "_shim_common.h"
namespace tbb {
class spin_mutex {
    std::mutex m_;
public:
    class scoped_lock {
        spin_mutex *m_;
    public:
        scoped_lock() : m_(nullptr) {}
        explicit scoped_lock(spin_mutex &m) : m_(&m) { m_->m_.lock(); }
        void acquire(spin_mutex &m) { m_ = &m; m_->m_.lock(); }
        void release() { if (m_) { m_->m_.unlock(); m_ = nullptr; } }
        ~scoped_lock() { release(); }
    };
};
}  // namespace tbb
