// Minimal stand-in for the legacy Intel TBB API used by MRAG (TBB is not
// installed here). Test infrastructure for the CPU oracle only: threads are
// plain std::thread, queues are mutex-protected.
#pragma once
// MRAGCommon.h defines function-like min/max macros before it includes TBB;
// hide them while the standard headers are read.
#pragma push_macro("min")
#pragma push_macro("max")
#undef min
#undef max
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <cstdlib>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>
#include <memory>
#include <utility>
#pragma pop_macro("max")
#pragma pop_macro("min")

namespace tbb {
namespace shim {
inline int &thread_count() {
    static int n = 1;
    return n;
}
}  // namespace shim
}  // namespace tbb
