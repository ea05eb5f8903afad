// Split merge, exact re-rank of candidate sets and result write-out.
//
// The re-rank restates candidateSetScan (candidateSetScanner.cuh:10-32): every
// candidate's exact distance is recomputed with the reference's arithmetic (one thread
// walks one candidate row in dimension order), then the candidates are sorted by
// (distance, id) and the first k written in ascending order -- the order the reference
// produces by writing its sorted warp queue back to front (sketchedDistanceScanners.cuh:
// 84-99).  Empty candidates (no point) become (-1, INT_MAX) as in the reference.
//
// FP64 re-check (optional, on by default for the tensor-core scans): after the FP32 sort,
// the candidates whose FP32 distance lies within the FP32 error bound of the k-th one --
// the only ones that FP32 may put on the wrong side of the k-th place -- are re-scored in
// double precision and reordered by (FP64 distance, id), so the top-k set is that of the
// exact distances.  Returned distances stay the FP32 values of the reference's formula.
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "select.cuh"
#include "distance.cuh"
#include "profile.h"
#include "tc_ptx.cuh"

namespace lshg {

namespace {

constexpr int kBandMax = 128;  // entries a query's FP64 re-check covers at most
constexpr uint64_t kPartitionBytes = 32ull << 20;  // base rows above this: gather in base order

// Double-precision closeness of a float row to the query as a ratio a / b (larger =
// closer, b > 0), computed by a whole warp: lane l sums the terms of dimensions l, l + 32,
// ... in order (products of floats are exact in double), then the 32 partial sums are added
// in a fixed tree to lane 0 and broadcast.  The GPU's FP64 pipe is narrow, and a warp
// instruction costs the same with one active lane as with 32, so one lane walking a whole
// row would cost 32 times as much.
//   angular   a = q.x, b = |x|      (1 - a / (|q| b) orders as -a / b; |q| is common)
//   Jaccard   a = sum min, b = sum max
//   Euclidean a = -sum (q - x)^2, b = 1
// Two candidates are then ordered by comparing a_i b_j with a_j b_i in double: no division
// or square root per candidate.  xn: the row's norm in double when the index keeps them.
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  return __shfl_sync(0xffffffffu, v, 0);
}

template <int DIST>
__device__ double2 fp64_closeness_warp(const float* __restrict__ xr, const float* qr, int d, double xn, int lane) {
  if (DIST == DIST_ANGULAR) {
    double dot = 0.0, xx = 0.0;
    if (xn > 0.0) {
      for (int j = lane; j < d; j += 32) dot = __dadd_rn(dot, __dmul_rn((double)qr[j], (double)xr[j]));
    } else {
      for (int j = lane; j < d; j += 32) {
        const double a = qr[j], b = xr[j];
        dot = __dadd_rn(dot, __dmul_rn(a, b));
        xx = __dadd_rn(xx, __dmul_rn(b, b));
      }
      xn = __dsqrt_rn(warp_sum_d(xx));
    }
    return make_double2(warp_sum_d(dot), xn);
  } else if (DIST == DIST_JACCARD) {
    double mn = 0.0, mx = 0.0;
    for (int j = lane; j < d; j += 32) {
      const double a = xr[j], b = qr[j];
      mn = __dadd_rn(mn, fmin(a, b));
      mx = __dadd_rn(mx, fmax(a, b));
    }
    return make_double2(warp_sum_d(mn), warp_sum_d(mx));
  } else {
    double acc = 0.0;
    for (int j = lane; j < d; j += 32) {
      const double df = __dadd_rn((double)qr[j], -(double)xr[j]);
      acc = __dadd_rn(acc, __dmul_rn(df, df));
    }
    return make_double2(-warp_sum_d(acc), 1.0);
  }
}

// FP64 re-check at the k-th place.  After the FP32 sort, the run of entries around entry
// k - 1 whose consecutive FP32 distances differ by at most the band (twice the FP32 error
// bound, band_abs + band_rel * |distance|) holds every candidate whose order against the
// k-th could differ in exact arithmetic: outside it the FP32 order is the exact order.  A
// run of two or more entries is re-scored in double precision and sorted by (FP64
// closeness, id), so the top-k set -- and its order around the k-th place -- is that of
// the exact distances.  The run is searched among the first kBandMax entries.  Called by
// every thread of the block after the sort; qr is the query row.
template <int DIST>
__device__ void fp64_boundary(uint64_t* keys, int C, int k, const float* __restrict__ x,
                              const double* __restrict__ xn64, int d, const float* qr, float band_abs,
                              float band_rel) {
  __shared__ double2 s_ab[kBandMax];  // closeness a / b in double
  __shared__ uint64_t s_key[kBandMax];
  __shared__ int s_lo, s_hi;
  const int L = imin(C, kBandMax);
  const int kk = imin(k, L) - 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (kk < 0) return;
  __syncthreads();  // a previous call's readers of s_lo / s_hi are done before they change
  if (threadIdx.x == 0) {
    auto joined = [&](int i) {  // entries i - 1 and i are within the band
      const uint64_t a = keys[i - 1], b = keys[i];
      if (a == kEmptyKey || b == kEmptyKey) return false;
      const float da = key_dist(a), db = key_dist(b);
      return fabsf(db - da) <= band_abs + band_rel * fmaxf(fabsf(da), fabsf(db));
    };
    int lo = kk, hi = kk;
    while (lo > 0 && joined(lo)) --lo;
    while (hi + 1 < L && joined(hi + 1)) ++hi;
    s_lo = lo;
    s_hi = hi;
  }
  __syncthreads();
  const int lo = s_lo, m = s_hi - s_lo + 1;
  if (m < 2) return;  // block-uniform
  for (int t = threadIdx.x; t < m; t += blockDim.x) s_key[t] = keys[lo + t];
  __syncthreads();
  for (int t = warp; t < m; t += nwarps) {  // a warp a candidate
    const int id = key_id(s_key[t]);
    const double2 ab = fp64_closeness_warp<DIST>(x + (int64_t)id * d, qr, d, xn64 ? xn64[id] : 0.0, lane);
    if (lane == 0) s_ab[t] = ab;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const double2 pi = s_ab[t];
    const uint32_t ii = (uint32_t)key_id(s_key[t]);
    int r = 0;
    for (int j = 0; j < m; ++j) {
      const double2 pj = s_ab[j];
      const double lj = __dmul_rn(pj.x, pi.y), li = __dmul_rn(pi.x, pj.y);  // j closer: a_j b_i > a_i b_j
      const uint32_t ij = (uint32_t)key_id(s_key[j]);
      r += (lj > li) || (lj == li && (ij < ii || (ij == ii && j < t)));
    }
    keys[lo + r] = s_key[t];
  }
  __syncthreads();
}

// One block per query: fold S sorted lists of C keys into one.
__global__ void merge_splits_kernel(const uint64_t* __restrict__ in, int nq, int splits, int C,
                                    uint64_t* __restrict__ out) {
  extern __shared__ uint64_t ms[];
  const int q = blockIdx.x;
  const uint64_t* src = in + (int64_t)q * splits * C;
  for (int i = threadIdx.x; i < C; i += blockDim.x) ms[i] = src[i];
  __syncthreads();
  for (int s = 1; s < splits; ++s) {
    const uint64_t* lst = src + (int64_t)s * C;
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
      uint64_t b = lst[C - 1 - i];
      if (b < ms[i]) ms[i] = b;
    }
    __syncthreads();
    block_bitonic_merge(ms, C);
  }
  for (int i = threadIdx.x; i < C; i += blockDim.x) out[(int64_t)q * C + i] = ms[i];
}

template <int DIST>
__global__ void rerank_kernel(const uint64_t* __restrict__ cand, int nq, int C, const float* __restrict__ x,
                              int64_t n, int d, const float* __restrict__ xnorm, const float* __restrict__ q,
                              const float* __restrict__ qnorm, int k, lshg_point* __restrict__ out, float band_abs,
                              float band_rel, const double* __restrict__ xn64, const RerankBounds* __restrict__ kx) {
  extern __shared__ __align__(16) unsigned char rsm[];
  uint64_t* keys = reinterpret_cast<uint64_t*>(rsm);
  float* qr = reinterpret_cast<float*>(rsm + (size_t)C * 8);
  const int qi = blockIdx.x;
  for (int j = threadIdx.x; j < d; j += blockDim.x) qr[j] = q[(int64_t)qi * d + j];
  __syncthreads();
  const float qn = (DIST == DIST_ANGULAR) ? qnorm[qi] : 1.0f;
  for (int i = threadIdx.x; i < C; i += blockDim.x) {
    uint64_t kin = cand[(int64_t)qi * C + i];
    uint64_t ko = kEmptyKey;
    if (kin != kEmptyKey) {
      int id = key_id(kin);
      if (id >= 0 && id < n) {
        float xn = (DIST == DIST_ANGULAR) ? xnorm[id] : 1.0f;
        ko = make_key(exact_distance<DIST>(x + (int64_t)id * d, qr, d, qn, xn), id);
      }
    }
    keys[i] = ko;
  }
  __syncthreads();
  block_bitonic_sort(keys, C);
  if (band_abs >= 0.0f) {
    fp64_boundary<DIST>(keys, C, k, x, xn64, d, qr, band_abs, band_rel);
    const int nx = kx ? imin(kx->n, 4) : 0;
    for (int b = 0; b < nx; ++b) {
      const int kb = kx->k[b];
      if (kb >= 1 && kb < k) fp64_boundary<DIST>(keys, C, kb, x, xn64, d, qr, band_abs, band_rel);
    }
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    uint64_t kk = i < C ? keys[i] : kEmptyKey;
    lshg_point pt;
    if (kk == kEmptyKey) { pt.ID = -1; pt.distance = kEmptyDistance; }
    else { pt.ID = key_id(kk); pt.distance = key_dist(kk); }
    out[(int64_t)qi * k + i] = pt;
  }
}

// The same re-rank with the candidate rows staged in shared memory by bulk copies, one
// row per thread and blockDim rows per chunk (per-thread 4- or 16-byte loads of scattered
// rows top out near 2 TB/s; bulk copies keep several hundred rows in flight per SM).
// Needs d % 4 == 0 and 16-byte aligned rows.  A copy wait that times out raises error 3
// on `err` and the rows are read directly from then on (results are unchanged).
template <int DIST>
__global__ void rerank_staged_kernel(const uint64_t* __restrict__ cand, int nq, int C, const float* __restrict__ x,
                                     int64_t n, int d, const float* __restrict__ xnorm, const float* __restrict__ q,
                                     const float* __restrict__ qnorm, int k, lshg_point* __restrict__ out, int* err,
                                     float band_abs, float band_rel, const double* __restrict__ xn64, int test_stall,
                                     const RerankBounds* __restrict__ kx) {
  extern __shared__ __align__(128) unsigned char rsm[];
  const int CH = blockDim.x;
  const uint32_t slot = stage_slot_bytes(d), rowb = (uint32_t)d * 4u;
  unsigned char* stage = rsm;
  uint64_t* keys = reinterpret_cast<uint64_t*>(rsm + (size_t)CH * slot);
  float* qr = reinterpret_cast<float*>(keys + C);
  __shared__ __align__(8) uint64_t bar, never;
  const int qi = blockIdx.x, tid = threadIdx.x;
  const uint32_t bar_a = tc::smem_u32(&bar);
  // test_stall: the first wait is made on `never`, a barrier nothing arrives on, with a
  // 1 ms limit -- the give-up path (error 3, rows read directly, the copy drained at exit)
  // runs without any fault
  const uint32_t never_a = tc::smem_u32(&never);
  if (tid == 0) {
    tc::mbar_init(bar_a, 1);
    tc::mbar_init(never_a, 1);
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const float qn = (DIST == DIST_ANGULAR) ? qnorm[qi] : 1.0f;
  unsigned char* dst = stage + (size_t)tid * slot;
  uint32_t phase = 0, pending = 0;
  bool ok = true;  // block-uniform
  for (int c0 = 0; c0 < C; c0 += CH) {
    const int i = c0 + tid;
    int id = -1;
    if (i < C) {
      const uint64_t kin = cand[(int64_t)qi * C + i];
      if (kin != kEmptyKey) {
        id = key_id(kin);
        if (id < 0 || id >= n) id = -1;
      }
    }
    const float xn = (DIST == DIST_ANGULAR && id >= 0) ? xnorm[id] : 1.0f;
    const int nv = __syncthreads_count(id >= 0);
    if (ok && nv > 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // this thread's earlier slot reads first
      if (tid == 0) tc::mbar_expect_tx(bar_a, (uint32_t)nv * rowb);
      __syncthreads();
      if (id >= 0) tc::bulk_load(tc::smem_u32(dst), x + (int64_t)id * d, rowb, bar_a);
    }
    // the query row while the first chunk's rows are in flight; published by the barrier
    // that ends this chunk's wait (or the next chunk's count when this one has no rows)
    if (c0 == 0)
      for (int j = tid; j < d; j += CH) qr[j] = q[(int64_t)qi * d + j];
    if (ok && nv > 0) {
      const bool stall = test_stall && c0 == 0;
      const uint32_t wbar = stall ? never_a : bar_a;
      const uint64_t limit = stall ? 1000000ull : tc::kWaitNs;
      bool got = tc::mbar_try(wbar, phase);
      if (!got) {
        const uint64_t t0 = tc::global_ns();
        while (!(got = tc::mbar_try_sleep(wbar, phase, 20000u)))
          if (tc::global_ns() - t0 > limit) break;
      }
      ok = __syncthreads_and(got);
      if (!ok) {
        pending = phase;
        if (tid == 0 && err) atomicExch(err, 3);
      }
      phase ^= 1u;
    }
    if (i < C) {
      uint64_t ko = kEmptyKey;
      if (id >= 0) {
        const float dist =
            ok ? exact_distance_v4<DIST, true>(reinterpret_cast<const float4*>(dst), reinterpret_cast<const float4*>(qr),
                                               d >> 2, qn, xn)
               : exact_distance<DIST>(x + (int64_t)id * d, qr, d, qn, xn);
        ko = make_key(dist, id);
      }
      keys[i] = ko;
    }
  }
  __syncthreads();
  block_bitonic_sort(keys, C);
  if (band_abs >= 0.0f) {
    fp64_boundary<DIST>(keys, C, k, x, xn64, d, qr, band_abs, band_rel);
    const int nx = kx ? imin(kx->n, 4) : 0;
    for (int b = 0; b < nx; ++b) {
      const int kb = kx->k[b];
      if (kb >= 1 && kb < k) fp64_boundary<DIST>(keys, C, kb, x, xn64, d, qr, band_abs, band_rel);
    }
  }
  for (int i = tid; i < k; i += CH) {
    const uint64_t kk = i < C ? keys[i] : kEmptyKey;
    lshg_point pt;
    if (kk == kEmptyKey) { pt.ID = -1; pt.distance = kEmptyDistance; }
    else { pt.ID = key_id(kk); pt.distance = key_dist(kk); }
    out[(int64_t)qi * k + i] = pt;
  }
  if (!ok) {  // a timed-out copy may still land: wait for it (bounded) before the block exits
    const uint64_t t0 = tc::global_ns();
    while (!tc::mbar_try_sleep(bar_a, pending, 20000u))
      if (tc::global_ns() - t0 > tc::kWaitNs) break;
  }
}

// Candidate lists in base order, for the gather below: each query's C keys are
// partitioned into B = C / 128 ranges of ids (range = id * B / n), empty and out-of-range
// entries last.  The gather's grid runs chunk-major (every query's first chunk of 128,
// then every query's second, ...), so the CTAs in flight at one time read rows from about
// one range, 1 / B of the base; that range stays in L2 while every query's candidates in
// it are scored, and a base larger than L2 is read from DRAM about once a batch instead of
// once a candidate.  The order inside a range is the order of shared-memory atomics; the
// re-rank's result does not depend on it (its keys are ordered by (distance, id)).
constexpr int kPartPer = 8;  // keys a thread; C <= 512 * kPartPer
__global__ void __launch_bounds__(512) cand_partition_kernel(const uint64_t* __restrict__ cand, int C, int64_t n,
                                                             uint64_t* __restrict__ out) {
  __shared__ int cnt[4096 / 128 + 1];
  const int B = C / 128, qi = blockIdx.x;
  for (int b = threadIdx.x; b <= B; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  uint64_t v[kPartPer];
  int at[kPartPer];  // range << 16 | place in the range
#pragma unroll
  for (int e = 0; e < kPartPer; ++e) {
    const int i = e * blockDim.x + threadIdx.x;
    at[e] = -1;
    if (i < C) {
      v[e] = cand[(int64_t)qi * C + i];
      const int id = key_id(v[e]);
      const int r = (v[e] != kEmptyKey && id >= 0 && id < n) ? (int)(((int64_t)id * B) / n) : B;
      at[e] = (r << 16) | atomicAdd(&cnt[r], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = 0; b <= B; ++b) {
      const int c = cnt[b];
      cnt[b] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int e = 0; e < kPartPer; ++e)
    if (at[e] >= 0) out[(int64_t)qi * C + cnt[at[e] >> 16] + (at[e] & 0xffff)] = v[e];
}

// Long candidate lists (C >= 1024) in two kernels: the gather kernel scores one chunk of
// blockDim candidates of one query a CTA (rows staged by bulk copies as above) and writes
// their keys; small CTAs with nothing but the gather keep several chunks in flight an SM,
// where one CTA a query walking all its chunks in turn waited on each.  The grid is
// (query, chunk) with the query fastest, so with lists in base order (above) the CTAs in
// flight share one range of the base.  cand and keys_out may be the same buffer: each
// thread reads its entry before it writes it.  The select kernel then sorts each query's
// keys, applies the FP64 re-check and writes the first k.
template <int DIST>
__global__ void rerank_gather_kernel(const uint64_t* cand, int C, const float* __restrict__ x, int64_t n,
                                     int d, const float* __restrict__ xnorm, const float* __restrict__ q,
                                     const float* __restrict__ qnorm, uint64_t* keys_out, int* err) {
  extern __shared__ __align__(128) unsigned char rsm[];
  const int CH = blockDim.x;
  const uint32_t slot = stage_slot_bytes(d), rowb = (uint32_t)d * 4u;
  float* qr = reinterpret_cast<float*>(rsm + (size_t)CH * slot);
  __shared__ __align__(8) uint64_t bar;
  const int qi = blockIdx.x, tid = threadIdx.x, i = blockIdx.y * CH + tid;
  const uint32_t bar_a = tc::smem_u32(&bar);
  if (tid == 0) tc::mbar_init(bar_a, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  int id = -1;
  if (i < C) {
    const uint64_t kin = cand[(int64_t)qi * C + i];
    if (kin != kEmptyKey) {
      id = key_id(kin);
      if (id < 0 || id >= n) id = -1;
    }
  }
  const float qn = (DIST == DIST_ANGULAR) ? qnorm[qi] : 1.0f;
  const float xn = (DIST == DIST_ANGULAR && id >= 0) ? xnorm[id] : 1.0f;
  unsigned char* dst = rsm + (size_t)tid * slot;
  const int nv = __syncthreads_count(id >= 0);
  bool ok = false;
  if (nv > 0) {
    if (tid == 0) tc::mbar_expect_tx(bar_a, (uint32_t)nv * rowb);
    __syncthreads();
    if (id >= 0) tc::bulk_load(tc::smem_u32(dst), x + (int64_t)id * d, rowb, bar_a);
    // the query row while the candidate rows are in flight (published by the barrier below)
    for (int j = tid; j < d; j += CH) qr[j] = q[(int64_t)qi * d + j];
    bool got = tc::mbar_try(bar_a, 0);
    if (!got) {
      const uint64_t t0 = tc::global_ns();
      while (!(got = tc::mbar_try_sleep(bar_a, 0, 20000u)))
        if (tc::global_ns() - t0 > tc::kWaitNs) break;
    }
    ok = __syncthreads_and(got);
    if (!ok && tid == 0 && err) atomicExch(err, 3);
  }
  if (i < C) {
    uint64_t ko = kEmptyKey;
    if (id >= 0) {
      const float dist =
          ok ? exact_distance_v4<DIST, true>(reinterpret_cast<const float4*>(dst), reinterpret_cast<const float4*>(qr),
                                             d >> 2, qn, xn)
             : exact_distance<DIST>(x + (int64_t)id * d, qr, d, qn, xn);
      ko = make_key(dist, id);
    }
    keys_out[(int64_t)qi * C + i] = ko;
  }
  if (nv > 0 && !ok) {  // a timed-out copy may still land: wait for it (bounded) before the block exits
    const uint64_t t0 = tc::global_ns();
    while (!tc::mbar_try_sleep(bar_a, 0, 20000u))
      if (tc::global_ns() - t0 > tc::kWaitNs) break;
  }
}

template <int DIST>
__global__ void rerank_select_kernel(const uint64_t* __restrict__ keys_in, int C, const float* __restrict__ x, int d,
                                     const float* __restrict__ q, int k, lshg_point* __restrict__ out, float band_abs,
                                     float band_rel, const double* __restrict__ xn64, const RerankBounds* __restrict__ kx) {
  extern __shared__ __align__(16) unsigned char rsm[];
  uint64_t* keys = reinterpret_cast<uint64_t*>(rsm);
  float* qr = reinterpret_cast<float*>(rsm + (size_t)C * 8);
  const int qi = blockIdx.x;
  for (int j = threadIdx.x; j < d; j += blockDim.x) qr[j] = q[(int64_t)qi * d + j];
  for (int i = threadIdx.x; i < C; i += blockDim.x) keys[i] = keys_in[(int64_t)qi * C + i];
  __syncthreads();
  block_bitonic_sort(keys, C);
  if (band_abs >= 0.0f) {
    fp64_boundary<DIST>(keys, C, k, x, xn64, d, qr, band_abs, band_rel);
    const int nx = kx ? imin(kx->n, 4) : 0;
    for (int b = 0; b < nx; ++b) {
      const int kb = kx->k[b];
      if (kb >= 1 && kb < k) fp64_boundary<DIST>(keys, C, kb, x, xn64, d, qr, band_abs, band_rel);
    }
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const uint64_t kk = i < C ? keys[i] : kEmptyKey;
    lshg_point pt;
    if (kk == kEmptyKey) { pt.ID = -1; pt.distance = kEmptyDistance; }
    else { pt.ID = key_id(kk); pt.distance = key_dist(kk); }
    out[(int64_t)qi * k + i] = pt;
  }
}

// The same select when only the first 128 places matter (k <= 128: the output and the
// FP64 re-check, which never looks past place 128): each of the 16 warps sorts its 32 E
// keys in registers and keeps the first 128, and four rounds of "min against the reversed
// partner list, then one bitonic merge" fold the 16 lists into the 128 smallest, sorted --
// the same 128 keys in the same order as sorting all C, without a block-wide sort.
template <int DIST, int E>
__global__ void __launch_bounds__(512) rerank_top_kernel(const uint64_t* __restrict__ keys_in, int C,
                                                         const float* __restrict__ x, int d,
                                                         const float* __restrict__ q, int k,
                                                         lshg_point* __restrict__ out, float band_abs, float band_rel,
                                                         const double* __restrict__ xn64,
                                                         const RerankBounds* __restrict__ kx) {
  constexpr int P = 128, EP = P / 32;
  __shared__ uint64_t lists[16][P];
  extern __shared__ __align__(16) unsigned char rsm[];
  float* qr = reinterpret_cast<float*>(rsm);
  const int qi = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = threadIdx.x; j < d; j += blockDim.x) qr[j] = q[(int64_t)qi * d + j];
  const uint64_t* src = keys_in + (int64_t)qi * C + warp * (32 * E);
  uint64_t v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = src[e * 32 + lane];
  warp_bitonic<E>(v, lane, false);
#pragma unroll
  for (int e = 0; e < EP; ++e) lists[warp][e * 32 + lane] = e < E ? v[e] : kEmptyKey;
  __syncthreads();
#pragma unroll
  for (int half = 8; half >= 1; half >>= 1) {
    if (warp < half) {
      // a ascending, b ascending: min(a[i], b[P - 1 - i]) is bitonic and holds the P smallest
      uint64_t a[EP];
#pragma unroll
      for (int e = 0; e < EP; ++e) {
        const uint64_t av = lists[warp][e * 32 + lane];
        const uint64_t bv = lists[warp + half][(EP - 1 - e) * 32 + (31 - lane)];
        a[e] = av < bv ? av : bv;
      }
      warp_bitonic<EP>(a, lane, true);
#pragma unroll
      for (int e = 0; e < EP; ++e) lists[warp][e * 32 + lane] = a[e];
    }
    __syncthreads();
  }
  uint64_t* keys = lists[0];
  if (band_abs >= 0.0f) {
    fp64_boundary<DIST>(keys, P, k, x, xn64, d, qr, band_abs, band_rel);
    const int nx = kx ? imin(kx->n, 4) : 0;
    for (int b = 0; b < nx; ++b) {
      const int kb = kx->k[b];
      if (kb >= 1 && kb < k) fp64_boundary<DIST>(keys, P, kb, x, xn64, d, qr, band_abs, band_rel);
    }
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const uint64_t kk = keys[i];
    lshg_point pt;
    if (kk == kEmptyKey) { pt.ID = -1; pt.distance = kEmptyDistance; }
    else { pt.ID = key_id(kk); pt.distance = key_dist(kk); }
    out[(int64_t)qi * k + i] = pt;
  }
}

__global__ void keys_to_points_kernel(const uint64_t* __restrict__ keys, int nq, int C, int k,
                                      lshg_point* __restrict__ out) {
  int64_t total = (int64_t)nq * k;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t qi = t / k;
    int i = (int)(t - qi * k);
    uint64_t kk = i < C ? keys[qi * C + i] : kEmptyKey;
    lshg_point pt;
    if (kk == kEmptyKey) { pt.ID = -1; pt.distance = kEmptyDistance; }
    else { pt.ID = key_id(kk); pt.distance = key_dist(kk); }
    out[t] = pt;
  }
}

}  // namespace

void launch_merge_splits(const uint64_t* in, int nq, int splits, int C, uint64_t* out, cudaStream_t s) {
  if (nq <= 0) return;
  ProfScope _ps("merge_splits", s);
  size_t smem = (size_t)C * 8;
  LSHG_CUDA(cudaFuncSetAttribute(merge_splits_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  merge_splits_kernel<<<nq, 128, smem, s>>>(in, nq, splits, C, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void fp64_band(int dist, int d, float* band_abs, float* band_rel) {
  // Twice the bound E on |FP32 distance - exact distance| (u = 2^-24, d-term sequential
  // sums: relative error <= d*u each): a candidate outside [kth - 2E, kth + 2E] is on the
  // same side of the k-th in FP32 and in exact arithmetic.  Angular: the dot within d*u of
  // |q||x|, each norm within (d/2 + 1)*u, product and quotient 2u, the subtraction u:
  // E <= (2d + 7)u.  Jaccard: two sums within d*u, quotient and subtraction: E <= (2d + 3)u.
  // Euclidean: relative, E <= (d + 3)u |distance|.
  const double u = 1.0 / 16777216.0;
  *band_abs = 0.0f;
  *band_rel = 0.0f;
  if (dist == DIST_ANGULAR) *band_abs = (float)(2.0 * (2.0 * d + 7.0) * u);
  else if (dist == DIST_JACCARD) *band_abs = (float)(2.0 * (2.0 * d + 3.0) * u);
  else *band_rel = (float)(2.0 * (d + 3.0) * u);
}

void launch_rerank(const uint64_t* cand, int nq, int C, const float* x, int64_t n, int d, const float* xnorm,
                   const float* q, const float* qnorm, int dist, int k, lshg_point* out, cudaStream_t s, int* err,
                   bool fp64_recheck, const double* xn64, const RerankBounds* extra_dev) {
  if (nq <= 0) return;
  float band_abs = -1.0f, band_rel = 0.0f;
  if (fp64_recheck) fp64_band(dist, d, &band_abs, &band_rel);
  const RerankBounds* kb = extra_dev;  // further places of the FP64 re-check (device memory)
  // test hook: LSHG_TEST_ROW_WAIT_STALL=1 makes the first row-copy wait of the staged
  // re-rank run out (see rerank_staged_kernel)
  const char* stall_env = getenv("LSHG_TEST_ROW_WAIT_STALL");
  const int test_stall = (stall_env && stall_env[0] == '1') ? 1 : 0;
  LSHG_REQUIRE((C & (C - 1)) == 0 && C >= 2, "re-rank: candidate count must be a power of two");
  ProfScope _ps("rerank", s);
  // staged: rows of d % 4 == 0 floats, 16-byte aligned, up to 128 a chunk
  const int CH = std::min(C, 128);
  const size_t staged_smem = (size_t)CH * stage_slot_bytes(d) + (size_t)C * 8 + (size_t)d * 4 + 16;
  const bool stageable = d % 4 == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
  const size_t gather_smem = (size_t)128 * stage_slot_bytes(d) + (size_t)d * 4 + 16;
  const size_t select_smem = (size_t)C * 8 + (size_t)d * 4 + 16;
  if (stageable && C >= 1024 && !test_stall && gather_smem <= 96 * 1024 && select_smem <= 200 * 1024) {
    DevBuf<uint64_t> gk((size_t)nq * C, s);
    // lists in base order when the rows do not fit in a quarter of L2 (the gather then
    // reads them in place)
    const uint64_t* gin = cand;
    if (C <= 512 * kPartPer && (uint64_t)n * (uint64_t)d * 4u > kPartitionBytes) {
      cand_partition_kernel<<<nq, 512, 0, s>>>(cand, C, n, gk.ptr);
      count_launch();
      LSHG_CHECK_LAUNCH();
      gin = gk.ptr;
    }
#define LSHG_RR2(DV)                                                                                            \
  do {                                                                                                          \
    LSHG_CUDA(cudaFuncSetAttribute(rerank_gather_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                   (int)gather_smem));                                                          \
    rerank_gather_kernel<DV><<<dim3(nq, C / 128), 128, gather_smem, s>>>(gin, C, x, n, d, xnorm, q, qnorm,      \
                                                                         gk.ptr, err);                          \
    count_launch();                                                                                             \
    LSHG_CHECK_LAUNCH();                                                                                        \
    if (k <= 128 && C == 4096)                                                                                  \
      rerank_top_kernel<DV, 8><<<nq, 512, (size_t)d * 4, s>>>(gk.ptr, C, x, d, q, k, out, band_abs, band_rel,   \
                                                              xn64, kb);                                        \
    else if (k <= 128 && C == 2048)                                                                             \
      rerank_top_kernel<DV, 4><<<nq, 512, (size_t)d * 4, s>>>(gk.ptr, C, x, d, q, k, out, band_abs, band_rel,   \
                                                              xn64, kb);                                        \
    else if (k <= 128 && C == 1024)                                                                             \
      rerank_top_kernel<DV, 2><<<nq, 512, (size_t)d * 4, s>>>(gk.ptr, C, x, d, q, k, out, band_abs, band_rel,   \
                                                              xn64, kb);                                        \
    else {                                                                                                      \
      LSHG_CUDA(cudaFuncSetAttribute(rerank_select_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                     (int)select_smem));                                                        \
      rerank_select_kernel<DV><<<nq, 512, select_smem, s>>>(gk.ptr, C, x, d, q, k, out, band_abs, band_rel,     \
                                                            xn64, kb);                                          \
    }                                                                                                           \
  } while (0)
    switch (dist) {
      case DIST_ANGULAR: LSHG_RR2(DIST_ANGULAR); break;
      case DIST_JACCARD: LSHG_RR2(DIST_JACCARD); break;
      case DIST_EUCLID: LSHG_RR2(DIST_EUCLID); break;
      case DIST_SQEUCLID: LSHG_RR2(DIST_SQEUCLID); break;
      default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "re-rank: invalid distance function");
    }
#undef LSHG_RR2
    count_launch();
    LSHG_CHECK_LAUNCH();
    return;
  }
  if (stageable && staged_smem <= 96 * 1024) {
#define LSHG_RRS(DV)                                                                                           \
  do {                                                                                                         \
    LSHG_CUDA(cudaFuncSetAttribute(rerank_staged_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                   (int)staged_smem));                                                         \
    rerank_staged_kernel<DV><<<nq, CH, staged_smem, s>>>(cand, nq, C, x, n, d, xnorm, q, qnorm, k, out, err, \
                                                         band_abs, band_rel, xn64, test_stall, kb);          \
  } while (0)
    switch (dist) {
      case DIST_ANGULAR: LSHG_RRS(DIST_ANGULAR); break;
      case DIST_JACCARD: LSHG_RRS(DIST_JACCARD); break;
      case DIST_EUCLID: LSHG_RRS(DIST_EUCLID); break;
      case DIST_SQEUCLID: LSHG_RRS(DIST_SQEUCLID); break;
      default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "re-rank: invalid distance function");
    }
#undef LSHG_RRS
    count_launch();
    LSHG_CHECK_LAUNCH();
    return;
  }
  size_t smem = (size_t)C * 8 + (size_t)d * 4 + 16;
  LSHG_REQUIRE(smem <= 200 * 1024, "re-rank: candidate set too large");
  int threads = C >= 256 ? 256 : 128;
#define LSHG_RR(DV)                                                                                       \
  do {                                                                                                    \
    LSHG_CUDA(cudaFuncSetAttribute(rerank_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    rerank_kernel<DV><<<nq, threads, smem, s>>>(cand, nq, C, x, n, d, xnorm, q, qnorm, k, out, band_abs,   \
                                                band_rel, xn64, kb);                                      \
  } while (0)
  switch (dist) {
    case DIST_ANGULAR: LSHG_RR(DIST_ANGULAR); break;
    case DIST_JACCARD: LSHG_RR(DIST_JACCARD); break;
    case DIST_EUCLID: LSHG_RR(DIST_EUCLID); break;
    case DIST_SQEUCLID: LSHG_RR(DIST_SQEUCLID); break;
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "re-rank: invalid distance function");
  }
#undef LSHG_RR
  count_launch();
  LSHG_CHECK_LAUNCH();
}

__global__ void row_norms_fp64_kernel(const float* __restrict__ x, int64_t n, int d, double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double ss = 0.0;
    for (int j = 0; j < d; ++j) {
      const double v = x[i * d + j];
      ss = __dadd_rn(ss, __dmul_rn(v, v));
    }
    out[i] = __dsqrt_rn(ss);
  }
}

void launch_row_norms_fp64(const float* x, int64_t n, int d, double* out, cudaStream_t s) {
  if (n <= 0) return;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 8);
  row_norms_fp64_kernel<<<blocks, 256, 0, s>>>(x, n, d, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_keys_to_points(const uint64_t* keys, int nq, int C, int k, lshg_point* out, cudaStream_t s) {
  if (nq <= 0) return;
  ProfScope _ps("keys_to_points", s);
  int64_t total = (int64_t)nq * k;
  int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 8);
  keys_to_points_kernel<<<blocks, 256, 0, s>>>(keys, nq, C, k, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace lshg
