// Weighted MinHash by rejection sampling (weightedMinHash.cuh:92-166).
//
// The reference draws, for every (point, hash), from an XORWOW stream seeded only by
// the hash: curand_init(seed_h, 0, 10000) then r = M * curand_uniform(), and counts
// the red draws before the first green one (green: r <= start[c] + x[c] with
// c = map[(int)r]).  Because the stream does not depend on the point, this engine
// draws each hash's stream once into a table (launch_wmh_tables) and every point walks
// the shared table; past the table it continues the saved XORWOW state.  cuRAND's
// device API (CUDA 13.0 curand_kernel.h) is called, not re-derived.
//
// Defined behaviour where the reference reads out of bounds:
//  * (int)r == M (curand_uniform returned 1.0f): the reference reads map[M]; here the
//    draw counts as red.
//  * one-bit variant with counter >= bitmapLen (255 in the reference): the reference
//    reads randomBitMap[counter] past its 255 entries (weightedMinHash.cuh:132); here
//    the bit is 0.
// The sampler stops after kMaxDraws draws and raises an error flag (the reference loops
// forever, e.g. on a zero vector whose normalisation produced NaNs).
#include <curand_kernel.h>

#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"

namespace lshg {

namespace {

constexpr int kMaxDraws = 1 << 20;

__global__ void wmh_tables_kernel(const int* __restrict__ seeds, int H, int T, int M, float* __restrict__ r,
                                  curandStateXORWOW_t* __restrict__ states) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= H) return;
  curandStateXORWOW_t st;
  curand_init((unsigned long long)(long long)seeds[h], 0ull, 10000ull, &st);
  const float Mf = (float)M;
  for (int j = 0; j < T; ++j) r[(int64_t)j * H + h] = __fmul_rn(Mf, curand_uniform(&st));
  states[h] = st;
}

// One warp per (point, group of up to 32 hashes).  Byte variant: a group is 32
// consecutive hashes.  One-bit variant: a group is one output word (hashBits seeds).
__global__ void __launch_bounds__(256) wmh_sketch_kernel(
    const float* __restrict__ x, int64_t n, int d, const int* __restrict__ start_g, const int* __restrict__ map_g,
    int M, const float* __restrict__ rtab, const curandStateXORWOW_t* __restrict__ states, int H, int T,
    int onebit, int words, int hashBits, const uint8_t* __restrict__ bitmap, int bitmapLen,
    uint8_t* __restrict__ out8, uint32_t* __restrict__ out32, int* err) {
  extern __shared__ int smi[];
  int* start = smi;       // [d]
  int* map = smi + d;     // [M]
  for (int i = threadIdx.x; i < d; i += blockDim.x) start[i] = start_g[i];
  for (int i = threadIdx.x; i < M; i += blockDim.x) map[i] = map_g[i];
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int groups = onebit ? words : (H + 31) / 32;
  const int64_t items = n * groups;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const float Mf = (float)M;
  for (int64_t it = warp0; it < items; it += nw) {
    const int64_t i = it / groups;
    const int grp = (int)(it - i * groups);
    int h;
    bool active;
    if (onebit) {
      h = grp * hashBits + lane;
      active = lane < hashBits;
    } else {
      h = grp * 32 + lane;
      active = h < H;
    }
    const float* xi = x + i * d;
    int cnt = 0;
    if (active) {
      curandStateXORWOW_t st;
      bool live = false;
      while (true) {
        float r;
        if (cnt < T) {
          r = rtab[(int64_t)cnt * H + h];
        } else {
          if (!live) { st = states[h]; live = true; }
          r = __fmul_rn(Mf, curand_uniform(&st));
        }
        int ri = (int)r;
        if (ri < M) {
          int c = map[ri];
          if (r <= __fadd_rn((float)start[c], xi[c])) break;  // green
        }
        if (++cnt >= kMaxDraws) { atomicExch(err, 1); break; }
      }
    }
    if (onebit) {
      uint32_t bit = (active && cnt < bitmapLen) ? (bitmap[cnt] ? 1u : 0u) : 0u;
      uint32_t word = __ballot_sync(0xffffffffu, bit != 0);
      if (lane == 0) out32[i * words + grp] = word;
    } else if (active) {
      out8[i * H + h] = (uint8_t)(cnt & 255);
    }
  }
}

}  // namespace

void launch_wmh_tables(const int* seeds, int H, int T, int M, float* r, void* states, cudaStream_t s) {
  if (H <= 0) return;
  wmh_tables_kernel<<<(H + 127) / 128, 128, 0, s>>>(seeds, H, T, M, r, (curandStateXORWOW_t*)states);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

size_t wmh_state_bytes() { return sizeof(curandStateXORWOW_t); }

void launch_wmh_sketch(const float* x, int64_t n, int d, const int* start, const int* map, int M, const float* r,
                       const void* states, int H, int T, int onebit, int words, int hashBits, const uint8_t* bitmap,
                       int bitmapLen, uint8_t* out8, uint32_t* out32, int* err, cudaStream_t s) {
  if (n <= 0) return;
  LSHG_REQUIRE(M >= 1, "weighted MinHash: index map is empty (all-zero data?)");
  LSHG_REQUIRE(!onebit || (hashBits >= 1 && hashBits <= 32 && words * hashBits == H), "one-bit WMH: bad shape");
  size_t smem = (size_t)(d + M) * sizeof(int);
  LSHG_REQUIRE(smem <= 200 * 1024, "weighted MinHash: index map too large");
  LSHG_CUDA(cudaFuncSetAttribute(wmh_sketch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int groups = onebit ? words : (H + 31) / 32;
  int64_t warps = n * groups;
  int blocks = (int)std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)num_sms() * 16);
  wmh_sketch_kernel<<<blocks, 256, smem, s>>>(x, n, d, start, map, M, r, (const curandStateXORWOW_t*)states, H, T,
                                              onebit, words, hashBits, bitmap, bitmapLen, out8, out32, err);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace lshg
