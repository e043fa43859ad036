#pragma once
#include "_shim_common.h"
namespace tbb {
class task_scheduler_init {
public:
    static const int automatic = -1;
    explicit task_scheduler_init(int n = automatic) {
        if (n <= 0) n = (int)std::thread::hardware_concurrency();
        if (n <= 0) n = 1;
        shim::thread_count() = n;
    }
    ~task_scheduler_init() {}
};
}  // namespace tbb
