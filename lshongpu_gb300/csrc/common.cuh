// Shared device/host utilities for the lshg engine: status handling, stream-ordered
// device buffers, and the 64-bit ordering key used by every top-k selection.
//
// Ordering key: (order-preserving float bits << 32) | id.  Sorting keys ascending sorts
// candidates by (distance ascending, id ascending), i.e. ties are broken by the lower
// index.  The reference compares distances with |a-b| < 1e-6 meaning "equal, keep the
// incumbent" (LinearScan/pointExtensions.cuh:8-33); the key order is the deterministic
// total order that agrees with it everywhere except inside such near-ties.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <stdexcept>
#include <cstdio>
#include <cstring>
#include <climits>

#include "lshg.h"

namespace lshg {

// ---------------------------------------------------------------------------------
// Errors.  The reference exits the process on any CUDA error (cudaHelpers.cuh:8-15);
// this library turns every failure into an exception that the C ABI maps to a status.
// ---------------------------------------------------------------------------------
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define LSHG_CUDA(call)                                                                  \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess) {                                                             \
      throw ::lshg::Error(_e == cudaErrorMemoryAllocation ? LSHG_ERR_OUT_OF_MEMORY      \
                                                          : LSHG_ERR_CUDA,              \
                          std::string(#call) + ": " + cudaGetErrorString(_e) + " at " + \
                              __FILE__ + ":" + std::to_string(__LINE__));                \
    }                                                                                    \
  } while (0)

#define LSHG_CHECK_LAUNCH() LSHG_CUDA(cudaGetLastError())

#define LSHG_REQUIRE(cond, msg)                                     \
  do {                                                              \
    if (!(cond)) throw ::lshg::Error(LSHG_ERR_INVALID_ARGUMENT, msg); \
  } while (0)

// ---------------------------------------------------------------------------------
// Stream-ordered device buffer (cudaMallocAsync / cudaFreeAsync on the owning stream).
// ---------------------------------------------------------------------------------
template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t n = 0;
  cudaStream_t stream = nullptr;
  DevBuf() = default;
  DevBuf(size_t count, cudaStream_t s) { alloc(count, s); }
  void alloc(size_t count, cudaStream_t s) {
    release();
    stream = s;
    n = count;
    if (count) LSHG_CUDA(cudaMallocAsync((void**)&ptr, count * sizeof(T), s));
  }
  void release() {
    if (ptr) cudaFreeAsync(ptr, stream);
    ptr = nullptr;
    n = 0;
  }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), n(o.n), stream(o.stream) { o.ptr = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); ptr = o.ptr; n = o.n; stream = o.stream; o.ptr = nullptr; o.n = 0; }
    return *this;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// ---------------------------------------------------------------------------------
// Keys.
// ---------------------------------------------------------------------------------
constexpr uint64_t kEmptyKey = ~0ull;

__host__ __device__ __forceinline__ uint32_t float_to_ordered(float f) {
  if (f == 0.0f) f = 0.0f;  // -0 and +0 compare equal in the reference; give them one key
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__host__ __device__ __forceinline__ float ordered_to_float(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

__host__ __device__ __forceinline__ uint64_t make_key(float dist, int id) {
  return ((uint64_t)float_to_ordered(dist) << 32) | (uint32_t)id;
}
__host__ __device__ __forceinline__ int key_id(uint64_t k) { return (int)(uint32_t)(k & 0xffffffffu); }
__host__ __device__ __forceinline__ float key_dist(uint64_t k) { return ordered_to_float((uint32_t)(k >> 32)); }

// Distance written for empty result slots: the reference stores (float)INT_MAX for
// queue entries with ID < 0 (candidateSetScanner.cuh:23) and initialises queues with it.
constexpr float kEmptyDistance = 2147483648.0f;

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

int num_sms();
void keep_pool_memory();  // keep the default mempool's reserve between query batches

template <typename T>
__host__ __device__ __forceinline__ T imin(T a, T b) { return a < b ? a : b; }
template <typename T>
__host__ __device__ __forceinline__ T imax(T a, T b) { return a > b ? a : b; }

}  // namespace lshg
