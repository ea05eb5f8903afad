// Exact distances with the reference's single-precision arithmetic, one thread per
// (query, candidate): angular 1 - dot/(|q||x|) with a sequential FMA dot product
// (distanceFunctions.cuh:23-40), generalized Jaccard 1 - sum(min)/sum(max)
// (distanceFunctions.cuh:10-21), Euclidean / squared Euclidean on float rows.
#pragma once
#include "common.cuh"
#include "kernels.h"

namespace lshg {

template <int DIST>
__device__ __forceinline__ float exact_distance(const float* __restrict__ xr, const float* qr, int d, float qn,
                                                float xn) {
  if (DIST == DIST_ANGULAR) {
    float dot = 0.0f;
    for (int j = 0; j < d; ++j) dot = __fmaf_rn(qr[j], xr[j], dot);
    return __fsub_rn(1.0f, __fdiv_rn(dot, __fmul_rn(qn, xn)));
  } else if (DIST == DIST_JACCARD) {
    float mn = 0.0f, mx = 0.0f;
    for (int j = 0; j < d; ++j) {
      float a = xr[j], b = qr[j];
      mn = __fadd_rn(mn, fminf(a, b));
      mx = __fadd_rn(mx, fmaxf(a, b));
    }
    return __fsub_rn(1.0f, __fdiv_rn(mn, mx));
  } else {
    float acc = 0.0f;
    for (int j = 0; j < d; ++j) {
      float df = __fsub_rn(qr[j], xr[j]);
      acc = __fmaf_rn(df, df, acc);
    }
    return DIST == DIST_EUCLID ? __fsqrt_rn(acc) : acc;
  }
}

}  // namespace lshg
