// Optional per-kernel timing with CUDA events recorded on the launching stream around
// each launch (off by default; enabled by lshg_profile_enable for benchmarks).  Never
// enable it while a stream is being captured into a graph.
#pragma once
#include <cuda_runtime.h>

namespace lshg {

bool profiling_on();
void profile_push(const char* name, cudaEvent_t a, cudaEvent_t b);

struct ProfScope {
  const char* name;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(const char* n, cudaStream_t st) : name(n), s(st) {
    if (profiling_on()) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEventRecord(b, s);
      profile_push(name, a, b);
    }
  }
};

}  // namespace lshg
