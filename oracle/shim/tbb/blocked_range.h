#pragma once
#include "_shim_common.h"
namespace tbb {
template <typename Value>
class blocked_range {
    Value b_, e_;
    std::size_t g_;
public:
    typedef Value const_iterator;
    blocked_range(Value b, Value e, std::size_t g = 1) : b_(b), e_(e), g_(g ? g : 1) {}
    Value begin() const { return b_; }
    Value end() const { return e_; }
    std::size_t size() const { return std::size_t(e_ - b_); }
    std::size_t grainsize() const { return g_; }
    bool empty() const { return !(b_ < e_); }
};
}  // namespace tbb
