// Preprocessing kernels: magnitudes, in-place normalisation, point-tile transpose, the
// generalized-Jaccard min shift and the weighted-MinHash bounds.
//
// Magnitudes use the reference's arithmetic bit for bit: a sequential single-precision
// sum of squares in dimension order, each step a fused multiply-add (nvcc contracts
// `m += x*x`), then an IEEE square root, then an IEEE division for normalisation
// (processingUtils.cuh:48-67, distanceFunctions.cuh:23-40).  Rows are staged through
// shared memory so global reads stay coalesced while each thread walks its own row.
#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"

namespace lshg {

namespace {

constexpr int kRowsPerBlock = 32;  // small blocks: a 10k-row query batch spreads over every SM

// Stage kRowsPerBlock rows into shared memory with an odd row pitch (conflict-free
// column walks), then let thread t own row t.
template <bool kNormalize>
__global__ void row_norm_kernel(float* __restrict__ x, int64_t n, int d, float* __restrict__ norms) {
  extern __shared__ float sm[];
  const int pitch = d | 1;
  const int64_t row0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int rows = (int)imin<int64_t>(kRowsPerBlock, n - row0);
  const float* src = x + row0 * d;
  for (int i = threadIdx.x; i < rows * d; i += blockDim.x) {
    int r = i / d, c = i - r * d;
    sm[r * pitch + c] = src[i];
  }
  __syncthreads();
  __shared__ float mags[kRowsPerBlock];
  if (threadIdx.x < rows) {
    const float* row = sm + threadIdx.x * pitch;
    float m = 0.0f;
    for (int j = 0; j < d; ++j) m = __fmaf_rn(row[j], row[j], m);
    m = __fsqrt_rn(m);
    if (kNormalize) mags[threadIdx.x] = m;
    else norms[row0 + threadIdx.x] = m;
  }
  if (kNormalize) {  // the divides are independent: every thread takes a share
    __syncthreads();
    for (int i = threadIdx.x; i < rows * d; i += blockDim.x) {
      const int r = i / d, c = i - r * d;
      sm[r * pitch + c] = __fdiv_rn(sm[r * pitch + c], mags[r]);
    }
    __syncthreads();
    float* dst = x + row0 * d;
    for (int i = threadIdx.x; i < rows * d; i += blockDim.x) {
      int r = i / d, c = i - r * d;
      dst[i] = sm[r * pitch + c];
    }
  }
}

// xt[tile][j][128] <- x[tile*128 + p][j]; rows past n are zero.
__global__ void tile_transpose_kernel(const float* __restrict__ x, int64_t n, int d, float* __restrict__ xt) {
  extern __shared__ float sm[];
  const int pitch = d | 1;
  const int64_t row0 = (int64_t)blockIdx.x * 128;
  const int rows = (int)imin<int64_t>(128, n - row0);
  const float* src = x + row0 * d;
  for (int i = threadIdx.x; i < rows * d; i += blockDim.x) {
    int r = i / d, c = i - r * d;
    sm[r * pitch + c] = src[i];
  }
  __syncthreads();
  float* dst = xt + (int64_t)blockIdx.x * 128 * d;
  for (int i = threadIdx.x; i < 128 * d; i += blockDim.x) {
    int j = i >> 7, p = i & 127;
    dst[i] = (p < rows) ? sm[p * pitch + j] : 0.0f;
  }
}

// Per-dimension atomicMin of (int)floor(x) (processingUtils.cuh:20-31).
__global__ void min_floor_kernel(const float* __restrict__ x, int64_t n, int d, int* minv) {
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    int m = INT_MAX;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) m = min(m, (int)floorf(x[i * d + j]));
    if (m != INT_MAX) atomicMin(&minv[j], m);
  }
}

// x += abs(minv[dim]) (processingUtils.cuh:33-45): float + (float)int.
__global__ void shift_abs_kernel(float* __restrict__ x, int64_t n, int d, const int* __restrict__ minv) {
  int64_t total = n * d;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int j = (int)(i % d);
    x[i] = __fadd_rn(x[i], (float)abs(minv[j]));
  }
}

// Per-dimension atomicMax of (int)ceil(x) (weightedMinHash.cuh:47-57).
__global__ void max_ceil_kernel(const float* __restrict__ x, int64_t n, int d, int* maxv) {
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    int m = INT_MIN;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) m = max(m, (int)ceilf(x[i * d + j]));
    if (m != INT_MIN) atomicMax(&maxv[j], m);
  }
}

__global__ void fill_u32_kernel(uint32_t* p, int64_t n, uint32_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

__global__ void u32_to_u16_kernel(const uint32_t* in, int64_t n, uint16_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint16_t)in[i];
}

__global__ void u32_to_u8_kernel(const uint32_t* in, int64_t n, uint8_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint8_t)in[i];
}

__global__ void pad_words_kernel(const uint32_t* in, int64_t n, int words, uint32_t* out, int wp, uint32_t pad) {
  int64_t total = n * wp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / wp;
    int c = (int)(i - r * wp);
    out[i] = c < words ? in[r * words + c] : pad;
  }
}

// Pack byte rows (sbytes per row) into rows of wp 32-bit words, little-endian, padding
// the tail bytes with `pad`.
__global__ void pack_bytes_kernel(const uint8_t* in, int64_t n, int sbytes, uint32_t* out, int wp, uint8_t pad) {
  int64_t total = n * wp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / wp;
    int c = (int)(i - r * wp);
    uint32_t w = 0;
    for (int b = 0; b < 4; ++b) {
      int byte = c * 4 + b;
      uint32_t v = byte < sbytes ? in[r * sbytes + byte] : pad;
      w |= v << (8 * b);
    }
    out[i] = w;
  }
}

int grid_for(int64_t total, int threads) {
  int64_t g = (total + threads - 1) / threads;
  int cap = num_sms() * 16;
  return (int)imax<int64_t>(1, imin<int64_t>(g, cap));
}

size_t staged_smem(int rows, int d) { return (size_t)rows * (size_t)(d | 1) * sizeof(float); }

}  // namespace

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

// Query batches allocate their temporaries (hundreds of MB for large batches) with
// cudaMallocAsync.  The default pool returns unused memory to the driver at every
// synchronisation, so each batch would map its temporaries again; keeping what the
// process has reserved (release threshold = max) makes those allocations free after the
// first batch.  The pool is per process: nothing outlives it.
void keep_pool_memory() {
  static std::mutex mu;
  static bool done[128] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return;
  std::lock_guard<std::mutex> g(mu);
  if (done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = true;
}

void launch_row_norms(const float* x, int64_t n, int d, float* norms, cudaStream_t s) {
  if (n <= 0) return;
  size_t smem = staged_smem(kRowsPerBlock, d);
  LSHG_REQUIRE(smem <= 200 * 1024, "dimension too large for row_norms");
  LSHG_CUDA(cudaFuncSetAttribute(row_norm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  row_norm_kernel<false><<<ceil_div(n, kRowsPerBlock), 128, smem, s>>>(const_cast<float*>(x), n, d, norms);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_normalize(float* x, int64_t n, int d, cudaStream_t s) {
  if (n <= 0) return;
  size_t smem = staged_smem(kRowsPerBlock, d);
  LSHG_REQUIRE(smem <= 200 * 1024, "dimension too large for normalize");
  LSHG_CUDA(cudaFuncSetAttribute(row_norm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  row_norm_kernel<true><<<ceil_div(n, kRowsPerBlock), 128, smem, s>>>(x, n, d, nullptr);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_tile_transpose(const float* x, int64_t n, int d, float* xt, cudaStream_t s) {
  if (n <= 0) return;
  size_t smem = staged_smem(128, d);
  LSHG_REQUIRE(smem <= 220 * 1024, "dimension too large for the tiled layout");
  LSHG_CUDA(cudaFuncSetAttribute(tile_transpose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tile_transpose_kernel<<<ceil_div(n, 128), 256, smem, s>>>(x, n, d, xt);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_min_floor(const float* x, int64_t n, int d, int* minv, cudaStream_t s) {
  if (n <= 0) return;
  int grid = (int)imin<int64_t>(n, num_sms() * 8);
  min_floor_kernel<<<grid, 128, 0, s>>>(x, n, d, minv);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_shift_abs(float* x, int64_t n, int d, const int* minv, cudaStream_t s) {
  if (n <= 0) return;
  shift_abs_kernel<<<grid_for(n * d, 256), 256, 0, s>>>(x, n, d, minv);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_max_ceil(const float* x, int64_t n, int d, int* maxv, cudaStream_t s) {
  if (n <= 0) return;
  int grid = (int)imin<int64_t>(n, num_sms() * 8);
  max_ceil_kernel<<<grid, 128, 0, s>>>(x, n, d, maxv);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_fill_u32(uint32_t* p, int64_t n, uint32_t v, cudaStream_t s) {
  if (n <= 0) return;
  fill_u32_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, n, v);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_u32_to_u16(const uint32_t* in, int64_t n, uint16_t* out, cudaStream_t s) {
  if (n <= 0) return;
  u32_to_u16_kernel<<<grid_for(n, 256), 256, 0, s>>>(in, n, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_u32_to_u8(const uint32_t* in, int64_t n, uint8_t* out, cudaStream_t s) {
  if (n <= 0) return;
  u32_to_u8_kernel<<<grid_for(n, 256), 256, 0, s>>>(in, n, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_pad_words(const uint32_t* in, int64_t n, int words, uint32_t* out, int wp, uint32_t pad,
                      cudaStream_t s) {
  if (n <= 0) return;
  pad_words_kernel<<<grid_for(n * wp, 256), 256, 0, s>>>(in, n, words, out, wp, pad);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_pack_bytes(const uint8_t* in, int64_t n, int sbytes, uint32_t* out, int wp, uint8_t pad, cudaStream_t s) {
  if (n <= 0) return;
  pack_bytes_kernel<<<grid_for(n * wp, 256), 256, 0, s>>>(in, n, sbytes, out, wp, pad);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace lshg
