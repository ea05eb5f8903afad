// Random projections: SimHash sign bits (simHash.cu:22-47, simHash.cuh:20-46) and JL
// float sketches (simHashJL.cuh:34-51).
//
// Each output is the reference's dot product: a single-precision fused multiply-add
// chain over the dimensions in order (nvcc contracts `dot += x[j]*r[j]`), so sign bits
// and JL floats are bit-identical to the reference's per-thread loops.  The GB300 form
// tiles 64 points x 64 planes per CTA through shared memory (each thread owns a 4x4
// register micro-tile), instead of one thread walking every plane of one point.
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "profile.h"

namespace lshg {

namespace {

constexpr int kTP = 64;      // points per CTA
constexpr int kTL = 64;      // planes per CTA
constexpr int kPitch = 68;   // shared row pitch (floats), keeps float4 alignment

__global__ void __launch_bounds__(256) project_kernel(const float* __restrict__ x, int64_t n, int d,
                                                      const float* __restrict__ planes, int nplanes,
                                                      int mode, int bits, int words,
                                                      uint32_t* __restrict__ out32, float* __restrict__ outf,
                                                      const int* __restrict__ gate) {
  if (gate && *gate == 0) return;  // block-uniform
  extern __shared__ __align__(16) float sm[];
  float* xs = sm;                 // [d][kPitch]
  float* rs = sm + d * kPitch;    // [d][kPitch]
  const int64_t p0 = (int64_t)blockIdx.x * kTP;
  const int l0 = blockIdx.y * kTL;
  const int np = (int)imin<int64_t>(kTP, n - p0);
  const int nl = min(kTL, nplanes - l0);

  for (int i = threadIdx.x; i < kTP * d; i += blockDim.x) {
    int p = i / d, j = i - p * d;
    xs[j * kPitch + p] = (p < np) ? x[(p0 + p) * d + j] : 0.0f;
  }
  for (int i = threadIdx.x; i < kTL * d; i += blockDim.x) {
    int l = i / d, j = i - l * d;
    rs[j * kPitch + l] = (l < nl) ? planes[(int64_t)(l0 + l) * d + j] : 0.0f;
  }
  __syncthreads();

  const int tl = threadIdx.x & 15;  // planes 4*tl .. 4*tl+3
  const int tp = threadIdx.x >> 4;  // points 4*tp .. 4*tp+3
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;

  for (int j = 0; j < d; ++j) {
    float4 xv = *reinterpret_cast<const float4*>(&xs[j * kPitch + 4 * tp]);
    float4 rv = *reinterpret_cast<const float4*>(&rs[j * kPitch + 4 * tl]);
    float xa[4] = {xv.x, xv.y, xv.z, xv.w};
    float rb[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = __fmaf_rn(xa[a], rb[b], acc[a][b]);
  }

  if (mode == 1) {
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      int p = 4 * tp + a;
      if (p >= np) continue;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        int l = 4 * tl + b;
        if (l < nl) outf[(p0 + p) * nplanes + l0 + l] = acc[a][b];
      }
    }
    return;
  }

  // Sign bits: the 8 lanes sharing (tp, plane group) hold 4 bits each of one 32-plane mask.
  const int g = tl >> 3;
  const int pb = l0 + 32 * g;  // first plane of this 32-plane group
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    uint32_t m = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) m |= (acc[a][b] >= 0.0f ? 1u : 0u) << ((tl & 7) * 4 + b);
    m |= __shfl_xor_sync(0xffffffffu, m, 1);
    m |= __shfl_xor_sync(0xffffffffu, m, 2);
    m |= __shfl_xor_sync(0xffffffffu, m, 4);
    int p = 4 * tp + a;
    if ((tl & 7) != 0 || p >= np || pb >= nplanes) continue;
    int valid = min(32, nplanes - pb);
    if (valid < 32) m &= (1u << valid) - 1u;
    uint32_t* row = out32 + (p0 + p) * words;
    if (bits == 32) {
      row[pb >> 5] = m;
    } else {
      int qq = pb;
      while (qq < pb + valid) {
        int w = qq / bits, b = qq - w * bits;
        int run = min(bits - b, pb + valid - qq);
        uint32_t chunk = (m >> (qq - pb)) & (run == 32 ? 0xffffffffu : ((1u << run) - 1u));
        if (chunk) atomicOr(&row[w], chunk << b);
        qq += run;
      }
    }
  }
}

}  // namespace

void launch_project(const float* x, int64_t n, int d, const float* planes, int nplanes, int mode, int bits,
                    int words, uint32_t* out32, float* out_f, cudaStream_t s) {
  if (n <= 0 || nplanes <= 0) return;
  LSHG_REQUIRE(mode == 1 || (bits >= 1 && bits <= 32 && words * bits == nplanes), "bad projection shape");
  size_t smem = (size_t)2 * d * kPitch * sizeof(float);
  LSHG_REQUIRE(smem <= 220 * 1024, "dimension too large for projection");
  ProfScope _ps(mode == 1 ? "project_jl" : "project_simhash", s);
  LSHG_CUDA(cudaFuncSetAttribute(project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(ceil_div(n, kTP), ceil_div(nplanes, kTL));
  project_kernel<<<grid, 256, smem, s>>>(x, n, d, planes, nplanes, mode, bits, words, out32, out_f, nullptr);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_project_gated(const float* x, int64_t n, int d, const float* planes, int nplanes, int words,
                          uint32_t* out32, const int* gate, cudaStream_t s) {
  if (n <= 0 || nplanes <= 0) return;
  size_t smem = (size_t)2 * d * kPitch * sizeof(float);
  LSHG_REQUIRE(smem <= 220 * 1024 && nplanes == 32 * words, "bad projection shape");
  LSHG_CUDA(cudaFuncSetAttribute(project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(ceil_div(n, kTP), ceil_div(nplanes, kTL));
  project_kernel<<<grid, 256, smem, s>>>(x, n, d, planes, nplanes, 0, 32, words, out32, nullptr, gate);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace lshg
