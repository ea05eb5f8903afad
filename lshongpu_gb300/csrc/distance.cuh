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

constexpr int kVecRowBatch = 8;  // float4 row loads in flight per thread (direct path)

// Shared-memory slot of one staged row of d floats (d % 4 == 0): an odd number of 16-byte
// units, so the float4 reads of 8 consecutive lanes -- each walking its own row -- fall in
// 8 different bank groups.
__host__ __device__ inline uint32_t stage_slot_bytes(int d) { return ((((uint32_t)d * 4u) / 16u) | 1u) * 16u; }

// Non-coherent 16-byte load, issued where written.
__device__ __forceinline__ float4 ldg_nc_f4(const float4* p) {
  float4 v;
  asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}

// Exact distance of a 16-byte-aligned row held as d4 float4s: the same operations in the
// same order as exact_distance, with the row fetched kVecRowBatch float4s at a time (all
// loads of a batch issued before its first use).  kShared: the row was staged in shared
// memory.
template <int DIST, bool kShared = false>
__device__ __forceinline__ float exact_distance_v4(const float4* __restrict__ xr, const float4* qr, int d4, float qn,
                                                   float xn) {
  float acc = 0.0f, mx = 0.0f;
  for (int j0 = 0; j0 < d4; j0 += kVecRowBatch) {
    float4 xv[kVecRowBatch];
#pragma unroll
    for (int u = 0; u < kVecRowBatch; ++u)
      xv[u] = j0 + u < d4 ? (kShared ? xr[j0 + u] : ldg_nc_f4(xr + j0 + u)) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kVecRowBatch; ++u) {
      if (j0 + u >= d4) break;
      const float4 qv = qr[j0 + u];
      const float xs[4] = {xv[u].x, xv[u].y, xv[u].z, xv[u].w};
      const float qs[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (DIST == DIST_ANGULAR) {
          acc = __fmaf_rn(qs[e], xs[e], acc);
        } else if (DIST == DIST_JACCARD) {
          acc = __fadd_rn(acc, fminf(xs[e], qs[e]));
          mx = __fadd_rn(mx, fmaxf(xs[e], qs[e]));
        } else {
          const float df = __fsub_rn(qs[e], xs[e]);
          acc = __fmaf_rn(df, df, acc);
        }
      }
    }
  }
  if (DIST == DIST_ANGULAR) return __fsub_rn(1.0f, __fdiv_rn(acc, __fmul_rn(qn, xn)));
  if (DIST == DIST_JACCARD) return __fsub_rn(1.0f, __fdiv_rn(acc, mx));
  return DIST == DIST_EUCLID ? __fsqrt_rn(acc) : acc;
}

}  // namespace lshg
