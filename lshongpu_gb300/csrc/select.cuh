// Top-C selection primitives on 64-bit ordering keys (see common.cuh).
//
// This replaces the reference's per-lane thread queues + lane-stride bitonic sort
// (LinearScan/sortingFramework.cuh:163-254) and its buffered insert rule
// (sketchedDistanceScanners.cuh:68-80).  Design:
//   * each query owns, in shared memory, a sorted "kept" list of its C best keys and an
//     unsorted append buffer;
//   * producers push a key only if it beats the query's current threshold (the C-th
//     kept key, a monotonically tightening upper bound), appending with a shared-memory
//     atomic;
//   * when a buffer might overflow, one warp sorts it (bitonic, in shared memory) and
//     folds it into the kept list with a single bitonic "min + merge" pass.
// All orderings are on (distance, id) so results do not depend on thread timing.
#pragma once

#include "common.cuh"

namespace lshg {

__device__ __forceinline__ int next_pow2_dev(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Warp-cooperative ascending bitonic sort of n (power of two) keys in shared memory.
__device__ __forceinline__ void warp_bitonic_sort(uint64_t* a, int n) {
  const int lane = threadIdx.x & 31;
  for (int size = 2; size <= n; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < (n >> 1); t += 32) {
        int i = 2 * t - (t & (stride - 1));
        int j = i + stride;
        bool up = ((i & size) == 0);
        uint64_t x = a[i], y = a[j];
        if ((x > y) == up) { a[i] = y; a[j] = x; }
      }
      __syncwarp();
    }
  }
}

// Warp-cooperative ascending sort of a bitonic sequence of n (power of two) keys.
__device__ __forceinline__ void warp_bitonic_merge(uint64_t* a, int n) {
  const int lane = threadIdx.x & 31;
  for (int stride = n >> 1; stride > 0; stride >>= 1) {
    for (int t = lane; t < (n >> 1); t += 32) {
      int i = 2 * t - (t & (stride - 1));
      int j = i + stride;
      uint64_t x = a[i], y = a[j];
      if (x > y) { a[i] = y; a[j] = x; }
    }
    __syncwarp();
  }
}

// One compare-exchange stage of a bitonic network on the 32 keys of a warp's registers
// (lane l holds element c*32 + l): partners are lanes l and l ^ s (s < 32); `up` (from the
// element index and the block size being sorted) says whether the lower index keeps the
// smaller key.  Same result as the shared-memory stage below.
__device__ __forceinline__ uint64_t bitonic_lane_stage(uint64_t x, int s, bool up, int lane) {
  const uint64_t y = __shfl_xor_sync(0xffffffffu, x, s);
  const bool keep_min = ((lane & s) == 0) == up;
  return keep_min ? (x < y ? x : y) : (x < y ? y : x);
}

// Block-cooperative ascending bitonic sort of n (power of two) keys in shared memory;
// every thread of the block (a whole number of warps) must call it.  Stages with stride >= 32 run in shared memory (a warp's pairs are 32 consecutive keys:
// no bank conflicts); each size's stages with stride < 32 run in registers on 32-key
// chunks, one chunk a warp, with shuffles -- one load, up to five exchanges and one store
// instead of five shared-memory passes with 2-way conflicts and a barrier each.
__device__ __forceinline__ void block_bitonic_sort(uint64_t* a, int n) {
  if (n < 64) {  // small lists: the plain network
    for (int size = 2; size <= n; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
          int i = 2 * t - (t & (stride - 1));
          int j = i + stride;
          bool up = ((i & size) == 0);
          uint64_t x = a[i], y = a[j];
          if ((x > y) == up) { a[i] = y; a[j] = x; }
        }
        __syncthreads();
      }
    }
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int c = warp; c < (n >> 5); c += nw) {  // sizes 2 .. 32: all inside a 32-key chunk
    const int i = c * 32 + lane;
    uint64_t x = a[i];
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1)
#pragma unroll
      for (int s = size >> 1; s > 0; s >>= 1) x = bitonic_lane_stage(x, s, (i & size) == 0, lane);
    a[i] = x;
  }
  __syncthreads();
  for (int size = 64; size <= n; size <<= 1) {
    for (int stride = size >> 1; stride >= 32; stride >>= 1) {
      for (int t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
        int i = 2 * t - (t & (stride - 1));
        int j = i + stride;
        bool up = ((i & size) == 0);
        uint64_t x = a[i], y = a[j];
        if ((x > y) == up) { a[i] = y; a[j] = x; }
      }
      __syncthreads();
    }
    for (int c = warp; c < (n >> 5); c += nw) {  // strides 16 .. 1 of this size
      const int i = c * 32 + lane;
      const bool up = (i & size) == 0;  // the same for the whole chunk (size >= 64)
      uint64_t x = a[i];
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) x = bitonic_lane_stage(x, s, up, lane);
      a[i] = x;
    }
    __syncthreads();
  }
}

// Block-cooperative ascending sort of a bitonic sequence of n (power of two) keys; strides
// below 32 in registers as in block_bitonic_sort.
__device__ __forceinline__ void block_bitonic_merge(uint64_t* a, int n) {
  const int reg_below = n >= 64 ? 32 : 0;
  for (int stride = n >> 1; stride > 0 && stride >= reg_below; stride >>= 1) {
    for (int t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
      int i = 2 * t - (t & (stride - 1));
      int j = i + stride;
      uint64_t x = a[i], y = a[j];
      if (x > y) { a[i] = y; a[j] = x; }
    }
    __syncthreads();
  }
  if (reg_below == 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int c = warp; c < (n >> 5); c += nw) {
    const int i = c * 32 + lane;
    uint64_t x = a[i];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) x = bitonic_lane_stage(x, s, true, lane);
    a[i] = x;
  }
  __syncthreads();
}

// Fold an unsorted buffer of `cnt` keys into the sorted kept list of C keys (C a power
// of two); afterwards kept holds the C smallest keys of the union, ascending.  `buf`
// must have room for next_pow2(cnt) entries.  Executed by one full warp.
__device__ __forceinline__ void warp_fold_buffer(uint64_t* kept, int C, uint64_t* buf, int cnt) {
  const int lane = threadIdx.x & 31;
  if (cnt <= 0) return;
  int nb = next_pow2_dev(cnt < 2 ? 2 : cnt);
  for (int i = cnt + lane; i < nb; i += 32) buf[i] = kEmptyKey;
  __syncwarp();
  warp_bitonic_sort(buf, nb);
  // kept ascending, buffer ascending: min(kept[i], buf[C-1-i]) is bitonic and holds the
  // C smallest keys of the union.
  for (int i = lane; i < C; i += 32) {
    int j = C - 1 - i;
    uint64_t b = (j < nb) ? buf[j] : kEmptyKey;
    if (b < kept[i]) kept[i] = b;
  }
  __syncwarp();
  warp_bitonic_merge(kept, C);
}

template <int E>
__device__ __forceinline__ void warp_bitonic(uint64_t (&x)[E], int lane, bool merge_only);

template <int E>
__device__ __forceinline__ void warp_sort_buffer_regs(uint64_t* buf, int cnt, int nb) {
  const int lane = threadIdx.x & 31;
  uint64_t x[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int i = e * 32 + lane;
    x[e] = i < cnt ? buf[i] : kEmptyKey;
  }
  warp_bitonic<E>(x, lane, false);
  __syncwarp();
#pragma unroll
  for (int e = 0; e < E; ++e)
    if (e * 32 + lane < nb) buf[e * 32 + lane] = x[e];
  __syncwarp();
}

// warp_fold_buffer with buffers of up to 256 keys sorted in registers (a shuffle
// network: no chain of dependent shared-memory round trips); larger ones as before.
// Same result, same room requirement.
static __device__ __noinline__ void warp_fold_buffer_regs(uint64_t* kept, int C, uint64_t* buf, int cnt) {
  const int lane = threadIdx.x & 31;
  if (cnt <= 0) return;
  const int nb = next_pow2_dev(cnt < 2 ? 2 : cnt);
  if (nb > 256) {
    warp_fold_buffer(kept, C, buf, cnt);
    return;
  }
  if (nb <= 32) warp_sort_buffer_regs<1>(buf, cnt, nb);
  else if (nb <= 64) warp_sort_buffer_regs<2>(buf, cnt, nb);
  else if (nb <= 128) warp_sort_buffer_regs<4>(buf, cnt, nb);
  else warp_sort_buffer_regs<8>(buf, cnt, nb);
  for (int i = lane; i < C; i += 32) {
    const int j = C - 1 - i;
    const uint64_t b = (j < nb) ? buf[j] : kEmptyKey;
    if (b < kept[i]) kept[i] = b;
  }
  __syncwarp();
  warp_bitonic_merge(kept, C);
}

// Per-query selection state in shared memory, laid out by the kernel:
//   kept[q*C .. q*C+C)   sorted ascending
//   buf [q*B .. q*B+B)   append buffer
//   cnt[q], thr[q]
struct TopCShared {
  uint64_t* kept;
  uint64_t* buf;
  int* cnt;
  uint64_t* thr;
  int C;
  int B;
};

__device__ __forceinline__ void topc_init(TopCShared s, int nq) {
  for (int i = threadIdx.x; i < nq * s.C; i += blockDim.x) s.kept[i] = kEmptyKey;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    s.cnt[q] = 0;
    s.thr[q] = kEmptyKey;
  }
}

// Append `key` for query q if it beats the threshold snapshot `thr`.
__device__ __forceinline__ void topc_push(TopCShared s, int q, uint64_t key, uint64_t thr) {
  if (key < thr) {
    int p = atomicAdd(&s.cnt[q], 1);
    s.buf[(size_t)q * s.B + p] = key;
  }
}

// Merge the buffers of every query whose fill exceeds `limit` (or all non-empty buffers
// when limit < 0).  Block-wide: all threads call it; warps take queries round-robin.
// Returns after a __syncthreads so new thresholds are visible.
// kRegSort: fold with warp_fold_buffer_regs.
// Block-cooperative warp_fold_buffer: every thread of the block takes part (same result).
__device__ __forceinline__ void block_fold_buffer(uint64_t* kept, int C, uint64_t* buf, int cnt) {
  const int nb = next_pow2_dev(cnt < 2 ? 2 : cnt);
  for (int i = cnt + threadIdx.x; i < nb; i += blockDim.x) buf[i] = kEmptyKey;
  __syncthreads();
  block_bitonic_sort(buf, nb);
  for (int i = threadIdx.x; i < C; i += blockDim.x) {
    const int j = C - 1 - i;
    const uint64_t b = (j < nb) ? buf[j] : kEmptyKey;
    if (b < kept[i]) kept[i] = b;
  }
  __syncthreads();
  block_bitonic_merge(kept, C);
}

template <bool kRegSort = false>
__device__ __forceinline__ void topc_flush(TopCShared s, int nq, int limit) {
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  if (s.C >= 512 && nq * 4 <= nwarps) {
    // long lists and few queries a block: one warp per query would leave most of the
    // block waiting on a C-key merge, so the whole block folds each query in turn
    for (int q = 0; q < nq; ++q) {
      const int c = s.cnt[q];  // read by every thread before the fold's first barrier
      if (c > limit && c > 0) {
        block_fold_buffer(s.kept + (size_t)q * s.C, s.C, s.buf + (size_t)q * s.B, c);
        if (threadIdx.x == 0) {
          s.cnt[q] = 0;
          s.thr[q] = s.kept[(size_t)q * s.C + s.C - 1];
        }
      }
    }
    __syncthreads();
    return;
  }
  for (int q = warp; q < nq; q += nwarps) {
    int c = s.cnt[q];
    if (c > limit && c > 0) {
      if (kRegSort) warp_fold_buffer_regs(s.kept + (size_t)q * s.C, s.C, s.buf + (size_t)q * s.B, c);
      else warp_fold_buffer(s.kept + (size_t)q * s.C, s.C, s.buf + (size_t)q * s.B, c);
      if ((threadIdx.x & 31) == 0) {
        s.cnt[q] = 0;
        s.thr[q] = s.kept[(size_t)q * s.C + s.C - 1];
      }
      __syncwarp();
    }
  }
  __syncthreads();
}

// Warp-wide bitonic network on 32*E 64-bit keys held as x[e] of lane l = element e*32+l.
// Sorts ascending when `merge_only` is false; with `merge_only` the input must already
// be bitonic and one merge pass sorts it.
template <int E>
__device__ __forceinline__ void warp_bitonic(uint64_t (&x)[E], int lane, bool merge_only) {
  constexpr int N = 32 * E;
#pragma unroll
  for (int k = 2; k <= N; k <<= 1) {
    if (merge_only && k != N) continue;
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int i = e * 32 + lane;
        const bool up = (i & k) == 0 || merge_only;
        if (j >= 32) {
          const int f = e ^ (j >> 5);
          if (f > e) {  // both elements live in this lane
            const uint64_t lo = x[e] < x[f] ? x[e] : x[f];
            const uint64_t hi = x[e] < x[f] ? x[f] : x[e];
            x[e] = up ? lo : hi;
            x[f] = up ? hi : lo;
          }
        } else {
          const uint64_t o = __shfl_xor_sync(0xffffffffu, x[e], j);
          const bool lower = (lane & j) == 0;
          x[e] = (lower == up) ? (x[e] < o ? x[e] : o) : (x[e] < o ? o : x[e]);
        }
      }
    }
  }
}

}  // namespace lshg
