// Process-wide count of kernel launches issued by the library (reported by
// lshg_launch_count so benchmarks can state how many of their kernels ran).
#pragma once
#include <atomic>
#include <stdint.h>

namespace lshg {
std::atomic<int64_t>& launch_counter();
inline void count_launch(int64_t n = 1) { launch_counter().fetch_add(n, std::memory_order_relaxed); }
}  // namespace lshg
