// Cross-polytope LSH keys (crossPolyTope.cuh:25-85).
//
// Per point and table: zero-pad to P = next power of two >= d, then `rounds` times
// {multiply by a +-1 diagonal; unnormalised Walsh-Hadamard butterflies for offsets
// P/2 .. 1, where the lower index of a pair gets a+b and the upper gets b-a}; the hash
// is the first index of the largest |y| (strict >, dimension order), coded as the index
// when y < 0 and index + P otherwise.  Additions are exact-order identical to the
// reference, so keys are bit-identical.
//
// GB300 form: one warp per point holds the padded vector in registers (P/32 values per
// lane); in-lane butterflies for small offsets, warp shuffles for the rest, and a
// shuffle arg-max.  The reference instead keeps two P-float scratch rows per thread in
// global memory (crossPolyTope.cuh:120-124).  `hashes` > 1 concatenates independent
// rotations into one key (key = h0 * 2P + h1 ...), which the reference does not have.
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"

namespace lshg {

namespace {

template <int E>
__global__ void __launch_bounds__(256) crosspoly_kernel(const float* __restrict__ x, int64_t n, int d, int P,
                                                        int tables, int hashes, int rounds,
                                                        const int* __restrict__ diag, uint16_t* __restrict__ keys) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = warp; p < n; p += nwarps) {
    float xin[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      int i = lane * E + e;
      xin[e] = (i < d) ? x[p * d + i] : 0.0f;
    }
    for (int t = 0; t < tables; ++t) {
      uint32_t key = 0;
      for (int h = 0; h < hashes; ++h) {
        float v[E];
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = xin[e];
        for (int r = 0; r < rounds; ++r) {
          const int* dg = diag + ((((int64_t)t * hashes + h) * rounds + r) * P);
#pragma unroll
          for (int e = 0; e < E; ++e) {
            int i = lane * E + e;
            if (i < P) v[e] = __fmul_rn(v[e], (float)dg[i]);
          }
          for (int o = P >> 1; o > 0; o >>= 1) {
            if (o < E) {
#pragma unroll
              for (int e = 0; e < E; ++e) {
                if ((e & o) == 0) {
                  float a = v[e], b = v[e | o];
                  v[e] = __fadd_rn(a, b);
                  v[e | o] = __fsub_rn(a, b);  // upper index: partner - self
                }
              }
            } else {
              int lo = o / E;
              bool lower = (lane & lo) == 0;
#pragma unroll
              for (int e = 0; e < E; ++e) {
                float other = __shfl_xor_sync(0xffffffffu, v[e], lo);
                v[e] = lower ? __fadd_rn(v[e], other) : __fsub_rn(other, v[e]);
              }
            }
          }
        }
        // first maximum of |v| in dimension order
        float best = -1.0f;
        int bi = 0x7fffffff;
        bool bneg = false;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          int i = lane * E + e;
          float a = fabsf(v[e]);
          if (i < P && a > best) { best = a; bi = i; bneg = v[e] < 0.0f; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          float ob = __shfl_xor_sync(0xffffffffu, best, off);
          int oi = __shfl_xor_sync(0xffffffffu, bi, off);
          bool on = __shfl_xor_sync(0xffffffffu, (int)bneg, off) != 0;
          if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; bneg = on; }
        }
        uint32_t code = (bi == 0x7fffffff) ? 0u : (bneg ? (uint32_t)bi : (uint32_t)(bi + P));
        key = key * (uint32_t)(2 * P) + code;
      }
      if (lane == 0) keys[p * tables + t] = (uint16_t)key;
    }
  }
}

}  // namespace

void launch_crosspoly(const float* x, int64_t n, int d, int P, int tables, int hashes, int rounds,
                      const int* diag, uint16_t* keys, cudaStream_t s) {
  if (n <= 0) return;
  LSHG_REQUIRE(P >= d && (P & (P - 1)) == 0 && P <= 1024, "cross-polytope: P must be a power of two >= d, <= 1024");
  int E = P >= 32 ? P / 32 : 1;
  int64_t warps = n;
  int blocks = (int)std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)num_sms() * 16);
  switch (E) {
#define LSHG_CP(EV) \
  case EV: crosspoly_kernel<EV><<<blocks, 256, 0, s>>>(x, n, d, P, tables, hashes, rounds, diag, keys); break;
    LSHG_CP(1) LSHG_CP(2) LSHG_CP(4) LSHG_CP(8) LSHG_CP(16) LSHG_CP(32)
#undef LSHG_CP
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "cross-polytope: unsupported P");
  }
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace lshg
