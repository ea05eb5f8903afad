// Host random generators reproducing the reference's libstdc++ streams (see host_rng.cpp).
#pragma once
#include <stdint.h>

namespace lshg {
void random_normals(int64_t count, double stddev, float* out);
void random_plus_minus(int64_t count, int32_t* out);
void random_bools(int64_t count, uint8_t* out);
}  // namespace lshg
