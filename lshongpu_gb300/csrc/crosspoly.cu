// Cross-polytope LSH keys (crossPolyTope.cuh:25-85).
//
// Per point and table: zero-pad to P = next power of two >= d, then `rounds` times
// {multiply by a +-1 diagonal; unnormalised Walsh-Hadamard butterflies for offsets
// P/2 .. 1, where the lower index of a pair gets a+b and the upper gets b-a}; the hash
// is the first index of the largest |y| (strict >, dimension order), coded as the index
// when y < 0 and index + P otherwise.  Additions are exact-order identical to the
// reference, so keys are bit-identical.
//
// GB300 form: a (point, table) unit's padded vector spread over P/32 lanes, 32 values a
// lane in 4-float chunks dealt round-robin (a warp works on 32/(P/32) units at once, and
// a group's 16-byte loads read contiguous runs); butterflies of the chunk bits and of the
// two lowest bits run inside a lane, those of the lane bits are shuffles, and the arg-max
// ends in shuffles.  The reference instead keeps two P-float scratch rows per thread in
// global memory (crossPolyTope.cuh:120-124).  `hashes` > 1 concatenates independent
// rotations into one key (key = h0 * 2P + h1 ...), which the reference does not have.
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"

namespace lshg {

namespace {

// v * g for a diagonal entry g = +1 or -1: the product is exact, so it is v with its sign
// bit flipped when g < 0 (no int-to-float conversion and no multiply)
__device__ __forceinline__ float times_sign(float v, int g) {
  return __int_as_float(__float_as_int(v) ^ (g & (int)0x80000000u));
}

// One (point, table) unit per group of G = P / 32 lanes (P >= 32; a warp holds 32 / G
// units), or per lane for P < 32.  The padded vector is cut into 4-float chunks dealt
// round-robin over the group: lane j holds chunks j, j + G, j + 2G, ..., so register
// e = 4c + r of lane j is element i = 4(Gc + j) + r.  A group's 16-byte loads then read
// contiguous runs of the row and of the diagonal.  Butterfly offsets 1 and 2 (bits of r)
// and offsets 4G and up (bits of c) pair registers inside a lane; offsets 4 .. 2G (bits of
// j) pair lanes of the group (shuffles).  Units are numbered table-major, so the groups of
// a warp usually share a table and its diagonals.
// vec: d % 4 == 0 and 16-byte aligned rows -- chunks are read as 16-byte loads.
template <int W>  // values a lane holds: 32 (P >= 32) or P
__global__ void __launch_bounds__(256, W == 32 ? 3 : 1) crosspoly_kernel(const float* __restrict__ x, int64_t n, int d, int P,
                                                        int tables, int hashes, int rounds,
                                                        const int* __restrict__ diag, uint16_t* __restrict__ keys,
                                                        bool vec) {
  constexpr int R = W < 4 ? W : 4;  // values a chunk
  constexpr int NC = W / R;         // chunks a lane
  const int lane = threadIdx.x & 31;
  const int G = P >= 32 ? P / 32 : 1;  // lanes a unit
  const int V = 32 / G;                // units a warp step
  const int j = lane % G, grp = lane / G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t units = n * tables;
  for (int64_t u0 = warp * V; u0 < units; u0 += nwarps * V) {  // warp-uniform
    const int64_t u = u0 + grp;
    const bool live = u < units;
    const int t = live ? (int)(u / n) : 0;
    const int64_t p = live ? u - (int64_t)t * n : 0;
    uint32_t key = 0;
    for (int h = 0; h < hashes; ++h) {
      float v[W];
      if (W == 32 && vec) {
        const float4* xr = reinterpret_cast<const float4*>(x + p * d);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const int ch = G * c + j;
          const float4 f = (live && 4 * ch < d) ? __ldg(xr + ch) : make_float4(0.f, 0.f, 0.f, 0.f);
          v[4 * c] = f.x; v[4 * c + 1] = f.y; v[4 * c + 2] = f.z; v[4 * c + 3] = f.w;
        }
      } else {
#pragma unroll
        for (int e = 0; e < W; ++e) {
          const int i = R * (G * (e / R) + j) + e % R;
          v[e] = (live && i < d) ? x[p * d + i] : 0.0f;
        }
      }
      for (int r = 0; r < rounds; ++r) {
        const int* dg = diag + ((((int64_t)t * hashes + h) * rounds + r) * P);
        if (W == 32) {  // P >= 32: all 32 of the lane's elements are inside P
          const int4* dg4 = reinterpret_cast<const int4*>(dg);
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            const int4 g = __ldg(dg4 + G * c + j);
            v[4 * c] = times_sign(v[4 * c], g.x);
            v[4 * c + 1] = times_sign(v[4 * c + 1], g.y);
            v[4 * c + 2] = times_sign(v[4 * c + 2], g.z);
            v[4 * c + 3] = times_sign(v[4 * c + 3], g.w);
          }
        } else {  // P < 32: G = 1, register e is element e
#pragma unroll
          for (int e = 0; e < W; ++e) v[e] = times_sign(v[e], dg[e]);
        }
        // offsets P/2 .. 4G: chunk bits, pairs of registers R*o/(4G) apart in a lane
#pragma unroll
        for (int oc = NC >> 1; oc > 0; oc >>= 1) {
#pragma unroll
          for (int e = 0; e < W; ++e) {
            if ((e & (R * oc)) == 0) {
              const float a = v[e], b = v[e | (R * oc)];
              v[e] = __fadd_rn(a, b);
              v[e | (R * oc)] = __fsub_rn(a, b);  // upper index: lower - upper
            }
          }
        }
        // offsets 2G .. 4: lane bits, partner lane j ^ o/4 of the group.  The lower lane
        // keeps other + v and the upper one other - v, both as fma(v, +-1, other): v * +-1
        // is exact and the fma rounds once, so the result is the rounded sum other + (+-v)
        // -- IEEE addition commutes and subtraction is addition of the negation, so it is
        // the reference's a + b or a - b bit for bit.
        for (int lo = G >> 1; lo > 0; lo >>= 1) {
          const float sgn = (j & lo) ? -1.0f : 1.0f;
#pragma unroll
          for (int e = 0; e < W; ++e) {
            const float other = __shfl_xor_sync(0xffffffffu, v[e], lo);
            v[e] = __fmaf_rn(v[e], sgn, other);
          }
        }
        // offsets 2, 1: bits of r, inside a chunk
#pragma unroll
        for (int o = R >> 1; o > 0; o >>= 1) {
#pragma unroll
          for (int e = 0; e < W; ++e) {
            if ((e & o) == 0) {
              const float a = v[e], b = v[e | o];
              v[e] = __fadd_rn(a, b);
              v[e | o] = __fsub_rn(a, b);
            }
          }
        }
      }
      // first maximum of |v| in dimension order (a lane's element index grows with e)
      float best = -1.0f;
      int bi = 0x7fffffff;
      bool bneg = false;
#pragma unroll
      for (int e = 0; e < W; ++e) {
        const int i = R * (G * (e / R) + j) + e % R;
        const float a = fabsf(v[e]);
        if (i < P && a > best) { best = a; bi = i; bneg = v[e] < 0.0f; }
      }
      for (int off = G >> 1; off > 0; off >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        const bool on = __shfl_xor_sync(0xffffffffu, (int)bneg, off) != 0;
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; bneg = on; }
      }
      const uint32_t code = (bi == 0x7fffffff) ? 0u : (bneg ? (uint32_t)bi : (uint32_t)(bi + P));
      key = key * (uint32_t)(2 * P) + code;
    }
    if (live && j == 0) keys[p * tables + t] = (uint16_t)key;
  }
}

}  // namespace

void launch_crosspoly(const float* x, int64_t n, int d, int P, int tables, int hashes, int rounds,
                      const int* diag, uint16_t* keys, cudaStream_t s) {
  if (n <= 0) return;
  LSHG_REQUIRE(P >= d && (P & (P - 1)) == 0 && P <= 1024, "cross-polytope: P must be a power of two >= d, <= 1024");
  const int W = P >= 32 ? 32 : P;                  // values a lane holds
  const bool vec = d % 4 == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(diag) & 15) == 0;
  const int V = P >= 32 ? 32 / (P / 32) : 32;     // units a warp step
  const int64_t warps = (n * tables + V - 1) / V;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)num_sms() * 16));
  switch (W) {
#define LSHG_CP(WV) \
  case WV: crosspoly_kernel<WV><<<blocks, 256, 0, s>>>(x, n, d, P, tables, hashes, rounds, diag, keys, vec); break;
    LSHG_CP(1) LSHG_CP(2) LSHG_CP(4) LSHG_CP(8) LSHG_CP(16) LSHG_CP(32)
#undef LSHG_CP
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "cross-polytope: unsupported P");
  }
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace lshg
