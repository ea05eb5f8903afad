// Host random generators with the reference's streams.
//
// The reference draws its projections on the host with a default-constructed
// std::default_random_engine (libstdc++: minstd_rand0, seed 1) and
// std::normal_distribution<double> / std::uniform_int_distribution<int>
// (randomVectorGenerator.cpp:5-87, weightedMinHash.cuh:231-250).  Those libstdc++
// algorithms (GCC 13 <bits/random.tcc>) are restated here so the engine produces the
// same numbers on any host compiler, with every floating-point step rounded separately
// (the x86-64 build of the reference has no FMA contraction):
//   minstd_rand0          x <- 16807 x mod (2^31 - 1), outputs in [1, 2^31 - 2]
//   generate_canonical    two draws: (g1 - 1) + (g2 - 1) * R, divided by R^2,
//                         R = 2^31 - 2; clamped below 1
//   normal (polar)        x = 2u - 1, y = 2u - 1 until 0 < x^2 + y^2 <= 1;
//                         m = sqrt(-2 ln r2 / r2); returns y*m, caches x*m
//   uniform_int(a, b)     rejection with scaling = (2^31 - 3) / (b - a + 1)
#include <cmath>
#include <cstdint>

#include "host_rng.h"

namespace lshg {

namespace {

struct MinStdRand0 {
  uint64_t x = 1;
  uint64_t operator()() {
    x = (x * 16807ull) % 2147483647ull;
    return x;
  }
};

constexpr uint64_t kMin = 1, kMax = 2147483646;

double canonical(MinStdRand0& g) {
  const double r = (double)(kMax - kMin + 1);  // 2147483646
  volatile double sum = 0.0;
  volatile double tmp = 1.0;
  for (int k = 0; k < 2; ++k) {
    double prod = (double)(g() - kMin) * tmp;
    sum = sum + prod;
    tmp = tmp * r;
  }
  double ret = sum / tmp;
  if (ret >= 1.0) ret = std::nextafter(1.0, 0.0);
  return ret;
}

struct Normal {
  bool saved_available = false;
  double saved = 0.0;
  double operator()(MinStdRand0& g, double mean, double stddev) {
    double ret;
    if (saved_available) {
      saved_available = false;
      ret = saved;
    } else {
      volatile double x, y, r2;
      do {
        double u1 = canonical(g);
        x = 2.0 * u1 - 1.0;
        double u2 = canonical(g);
        y = 2.0 * u2 - 1.0;
        double xx = x * x;
        double yy = y * y;
        r2 = xx + yy;
      } while (r2 > 1.0 || r2 == 0.0);
      volatile double lg = std::log((double)r2);
      volatile double num = -2.0 * lg;
      volatile double q = num / r2;
      const double mult = std::sqrt((double)q);
      saved = x * mult;
      saved_available = true;
      ret = y * mult;
    }
    volatile double scaled = ret * stddev;
    return scaled + mean;
  }
};

int uniform_int(MinStdRand0& g, int a, int b) {
  const uint64_t urngrange = kMax - kMin;                 // 2147483645
  const uint64_t urange = (uint64_t)((int64_t)b - (int64_t)a);
  const uint64_t uerange = urange + 1;
  const uint64_t scaling = urngrange / uerange;
  const uint64_t past = uerange * scaling;
  uint64_t ret;
  do {
    ret = g() - kMin;
  } while (ret >= past);
  ret /= scaling;
  return (int)(ret + (uint64_t)a);
}

}  // namespace

void random_normals(int64_t count, double stddev, float* out) {
  MinStdRand0 g;
  Normal nd;
  for (int64_t i = 0; i < count; ++i) out[i] = (float)nd(g, 0.0, stddev);
}

void random_plus_minus(int64_t count, int32_t* out) {
  MinStdRand0 g;
  for (int64_t i = 0; i < count; ++i) out[i] = uniform_int(g, 0, 2) == 0 ? -1 : 1;
}

void random_bools(int64_t count, uint8_t* out) {
  MinStdRand0 g;
  for (int64_t i = 0; i < count; ++i) out[i] = uniform_int(g, 0, 1) != 0 ? 1 : 0;
}

}  // namespace lshg
