// CPU brute force of GoldStandard/goldstandard.cpp -- TEST / BASELINE INFRASTRUCTURE ONLY.
//
// Restates computeGoldStandard (goldstandard.cpp:136-173): for every query, the
// "innerProduct" distance -cos to every base point (goldstandard.cpp:112-121: float
// magnitudes accumulated in float, dot product accumulated in double from float
// products, everything else single precision), then std::sort of all N points by
// distance and the first k written.  The reference keeps each point as a struct with a
// std::vector and copies it for every distance; this port keeps the arithmetic and the
// full sort but stores rows flat.  Queries are split across `threads` host threads
// (the reference is single-threaded); the return value is the wall time of the compute
// in seconds, measured with steady_clock.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

float magnitude(const float* x, int d) {
  // accumulate(..., 0.0, [](float state, float xi){ return state + xi*xi; })
  float state = 0.0f;
  for (int j = 0; j < d; ++j) {
    float sq = x[j] * x[j];
    state = state + sq;
  }
  return (float)std::sqrt((double)state);
}

float inner_product_dist(const float* q, const float* x, int d, float qm, float xm) {
  double acc = 0.0;  // inner_product(..., 0.0)
  for (int j = 0; j < d; ++j) {
    float prod = q[j] * x[j];
    acc = acc + (double)prod;
  }
  float dot = (float)acc;
  float denom = qm * xm;
  float sim = dot / denom;
  return -sim;
}

struct Entry {
  float dist;
  int id;
};

}  // namespace

extern "C" double or_goldstandard(const float* x, int64_t n, const float* q, int64_t nq, int d, int k, int threads,
                                  int32_t* ids, float* dists) {
  auto t0 = std::chrono::steady_clock::now();
  std::vector<float> xm(n);
  for (int64_t i = 0; i < n; ++i) xm[i] = magnitude(x + i * d, d);
  if (threads < 1) threads = 1;
  auto work = [&](int tid) {
    std::vector<Entry> all(n);
    for (int64_t qi = tid; qi < nq; qi += threads) {
      const float* qr = q + qi * d;
      float qm = magnitude(qr, d);
      for (int64_t i = 0; i < n; ++i) all[i] = {inner_product_dist(qr, x + i * d, d, qm, xm[i]), (int)i};
      std::sort(all.begin(), all.end(), [](const Entry& a, const Entry& b) { return a.dist < b.dist; });
      for (int j = 0; j < k; ++j) {
        ids[qi * k + j] = j < n ? all[j].id : -1;
        dists[qi * k + j] = j < n ? all[j].dist : 0.0f;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
