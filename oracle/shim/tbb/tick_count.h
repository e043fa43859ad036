#pragma once
#include "_shim_common.h"
namespace tbb {
class tick_count {
    double t_;
public:
    class interval_t {
        double d_;
    public:
        explicit interval_t(double d = 0) : d_(d) {}
        double seconds() const { return d_; }
        interval_t &operator+=(const interval_t &o) { d_ += o.d_; return *this; }
    };
    tick_count() : t_(0) {}
    static tick_count now() {
        tick_count c;
        c.t_ = std::chrono::duration<double>(
                   std::chrono::steady_clock::now().time_since_epoch()).count();
        return c;
    }
    friend interval_t operator-(const tick_count &a, const tick_count &b) {
        return interval_t(a.t_ - b.t_);
    }
};
}  // namespace tbb
