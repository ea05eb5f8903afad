// Per-kernel event timing (see profile.h) and its C entry points.
#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "profile.h"

namespace lshg {

namespace {
std::atomic<bool> g_on{false};
std::mutex g_mu;
struct Rec {
  std::string name;
  cudaEvent_t a, b;
};
std::vector<Rec> g_recs;
}  // namespace

bool profiling_on() { return g_on.load(std::memory_order_relaxed); }

void profile_push(const char* name, cudaEvent_t a, cudaEvent_t b) {
  std::lock_guard<std::mutex> g(g_mu);
  g_recs.push_back({name, a, b});
}

}  // namespace lshg

using namespace lshg;

extern "C" {

int lshg_profile_enable(int on) {
  g_on.store(on != 0);
  return LSHG_OK;
}

// Writes "name launches total_ms\n" lines (summed over all recorded launches since the
// last report) into buf; waits for the recorded events.  Returns the bytes needed.
int lshg_profile_report(char* buf, int cap) {
  std::vector<Rec> recs;
  {
    std::lock_guard<std::mutex> g(g_mu);
    recs.swap(g_recs);
  }
  std::map<std::string, std::pair<int64_t, double>> agg;
  for (auto& r : recs) {
    cudaEventSynchronize(r.b);
    float ms = 0;
    cudaEventElapsedTime(&ms, r.a, r.b);
    auto& e = agg[r.name];
    e.first += 1;
    e.second += ms;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  std::string out;
  char line[256];
  for (auto& kv : agg) {
    snprintf(line, sizeof line, "%s %lld %.6f\n", kv.first.c_str(), (long long)kv.second.first, kv.second.second);
    out += line;
  }
  if (buf && cap > 0) {
    size_t n = std::min((size_t)cap - 1, out.size());
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  return (int)out.size() + 1;
}

}  // extern "C"
