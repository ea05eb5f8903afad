// SIMT FP32 linear scans over float vectors with fused top-C selection.
//
// Replaces the reference's plain exact scan (memOptimizedLinearScan.cu:20-106, one warp
// per query, each lane walking points lane, lane+32, ...) and the JL sketch scan
// (sketchedDistanceScanners.cuh:102-180).  GB300 form: a CTA owns QB queries and a
// split of the base; the base is stored pre-transposed in 128-point tiles
// (xt[tile][j][128]) so each tile is one contiguous block copied into shared memory;
// each thread computes an MQ x 4 register micro-tile of (query, point) pairs.
//
// Distances keep the reference's arithmetic per pair: the dot product is a sequential
// FMA chain over j in order; magnitudes come precomputed with the same chain; the
// angular distance is 1 - dot / (|q| * |x|) with IEEE division
// (distanceFunctions.cuh:23-40), and generalized Jaccard is 1 - sum(min)/sum(max)
// (distanceFunctions.cuh:10-21).  Exact-scan distances are therefore bit-identical to
// the reference's; only the selection order differs (ties by lower index).
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "profile.h"
#include "select.cuh"

namespace lshg {

namespace {

constexpr int kTile = 128;
constexpr int kBuf = 256;

struct FloatScanSmem {
  size_t xs, qs, qn, kept, buf, thr, cnt, total;
};

__host__ __device__ inline size_t smem_take(size_t& off, size_t bytes) {
  off = (off + 15) / 16 * 16;
  size_t at = off;
  off += bytes;
  return at;
}

__host__ __device__ inline FloatScanSmem float_scan_layout(int d, int QB, int C, int nbuf) {
  FloatScanSmem L;
  size_t off = 0;
  L.xs = smem_take(off, (size_t)nbuf * kTile * d * 4);  // point tile, double-buffered when it fits
  L.qs = smem_take(off, (size_t)QB * d * 4);
  L.qn = smem_take(off, (size_t)QB * 4);
  L.kept = smem_take(off, (size_t)QB * C * 8);
  L.buf = smem_take(off, (size_t)QB * kBuf * 8);
  L.thr = smem_take(off, (size_t)QB * 8);
  L.cnt = smem_take(off, (size_t)QB * 4);
  L.total = off;
  return L;
}

template <int DIST>
__device__ __forceinline__ float finish_distance(float a, float b, float qn, float xn) {
  if (DIST == DIST_ANGULAR) return __fsub_rn(1.0f, __fdiv_rn(a, __fmul_rn(qn, xn)));
  if (DIST == DIST_JACCARD) return __fsub_rn(1.0f, __fdiv_rn(a, b));
  if (DIST == DIST_EUCLID) return __fsqrt_rn(a);
  return a;  // DIST_SQEUCLID
}

// 16-byte asynchronous global -> shared copy (L2 only) and its group fences.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <int DIST, int QB, int MQ>
__global__ void __launch_bounds__((QB / MQ) * 32) scan_float_kernel(
    const float* __restrict__ xt, int64_t n, int d, const float* __restrict__ xnorm, const float* __restrict__ q,
    int nq, const float* __restrict__ qnorm, int C, int tiles_per_split, int splits, int nbuf,
    uint64_t* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const FloatScanSmem L = float_scan_layout(d, QB, C, nbuf);
  float* xs = reinterpret_cast<float*>(smem + L.xs);
  float* qs = reinterpret_cast<float*>(smem + L.qs);
  float* qn = reinterpret_cast<float*>(smem + L.qn);
  TopCShared S{reinterpret_cast<uint64_t*>(smem + L.kept), reinterpret_cast<uint64_t*>(smem + L.buf),
               reinterpret_cast<int*>(smem + L.cnt), reinterpret_cast<uint64_t*>(smem + L.thr), C, kBuf};

  const int q0 = blockIdx.x * QB;
  const int split = blockIdx.y;
  const int ntiles = (int)((n + kTile - 1) / kTile);
  const int t_begin = split * tiles_per_split;
  const int t_end = min(ntiles, t_begin + tiles_per_split);

  for (int i = threadIdx.x; i < QB * d; i += blockDim.x) {
    int qi = i / d, j = i - qi * d;
    qs[j * QB + qi] = (q0 + qi < nq) ? q[(int64_t)(q0 + qi) * d + j] : 0.0f;
  }
  for (int qi = threadIdx.x; qi < QB; qi += blockDim.x)
    qn[qi] = (DIST == DIST_ANGULAR && q0 + qi < nq) ? qnorm[q0 + qi] : 1.0f;
  topc_init(S, QB);
  __syncthreads();

  const int tq = threadIdx.x >> 5;  // queries tq*MQ .. +MQ
  const int tp = threadIdx.x & 31;  // points tp*4 .. +4 within the tile
  uint64_t thr[MQ];
#pragma unroll
  for (int a = 0; a < MQ; ++a) thr[a] = kEmptyKey;
  constexpr int kLimit = kBuf - kTile;  // a tile appends at most kTile keys to a query's buffer
  bool over = false;                    // one of this thread's appends landed above kLimit

  // with two buffers the copy of tile t+1 runs while tile t is scored; with one (large d)
  // each tile is copied, then scored
  const int tile_f4 = kTile * d / 4;
  auto slot = [&](int tile) { return nbuf == 2 ? (tile & 1) : 0; };
  auto issue_tile = [&](int tile) {
    const float4* src = reinterpret_cast<const float4*>(xt + (int64_t)tile * kTile * d);
    float4* dst = reinterpret_cast<float4*>(xs) + (size_t)slot(tile) * tile_f4;
    for (int i = threadIdx.x; i < tile_f4; i += blockDim.x) cp_async16(dst + i, src + i);
    cp_async_commit();
  };
  if (t_begin < t_end) issue_tile(t_begin);
  for (int tile = t_begin; tile < t_end; ++tile) {
    if (nbuf == 2 && tile + 1 < t_end) {
      issue_tile(tile + 1);  // its buffer was last read by tile - 1, finished at the previous flush
      cp_async_wait<1>();
    } else {
      if (nbuf == 1 && tile > t_begin) issue_tile(tile);  // the previous flush ended every read
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* xcur = xs + (size_t)slot(tile) * kTile * d;

    float acc[MQ][4];
    float acc2[MQ][4];
#pragma unroll
    for (int a = 0; a < MQ; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) { acc[a][b] = 0.0f; acc2[a][b] = 0.0f; }

    for (int j = 0; j < d; ++j) {
      float4 xv = *reinterpret_cast<const float4*>(&xcur[j * kTile + 4 * tp]);
      float xb[4] = {xv.x, xv.y, xv.z, xv.w};
      float qa[MQ];
      if (MQ == 4) {
        float4 qv = *reinterpret_cast<const float4*>(&qs[j * QB + tq * MQ]);
        qa[0] = qv.x; qa[1 % MQ] = qv.y; qa[2 % MQ] = qv.z; qa[3 % MQ] = qv.w;
      } else {
#pragma unroll
        for (int a = 0; a < MQ; ++a) qa[a] = qs[j * QB + tq * MQ + a];
      }
#pragma unroll
      for (int a = 0; a < MQ; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          if (DIST == DIST_ANGULAR) {
            acc[a][b] = __fmaf_rn(qa[a], xb[b], acc[a][b]);
          } else if (DIST == DIST_JACCARD) {
            acc[a][b] = __fadd_rn(acc[a][b], fminf(xb[b], qa[a]));
            acc2[a][b] = __fadd_rn(acc2[a][b], fmaxf(xb[b], qa[a]));
          } else {
            float df = __fsub_rn(qa[a], xb[b]);
            acc[a][b] = __fmaf_rn(df, df, acc[a][b]);
          }
        }
    }

    const int64_t pbase = (int64_t)tile * kTile + 4 * tp;
    float xn[4];
#pragma unroll
    for (int b = 0; b < 4; ++b) xn[b] = (DIST == DIST_ANGULAR && pbase + b < n) ? xnorm[pbase + b] : 1.0f;
#pragma unroll
    for (int a = 0; a < MQ; ++a) {
      const int qi = tq * MQ + a;
      if (q0 + qi >= nq) continue;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        if (pbase + b >= n) continue;
        float dist = finish_distance<DIST>(acc[a][b], acc2[a][b], qn[qi], xn[b]);
        const uint64_t key = make_key(dist, (int)(pbase + b));
        if (key < thr[a]) {
          const int pos = atomicAdd(&S.cnt[qi], 1);
          S.buf[(size_t)qi * kBuf + pos] = key;
          over |= pos >= kLimit;
        }
      }
    }
    // one barrier a tile: every read of this tile's buffer is done (the next copy may
    // reuse it) and, only if some buffer passed kLimit, the buffers are folded
    if (__syncthreads_or(over)) {
      topc_flush(S, QB, kLimit);
#pragma unroll
      for (int a = 0; a < MQ; ++a) thr[a] = S.thr[tq * MQ + a];
    }
    over = false;
  }
  topc_flush(S, QB, 0);

  for (int i = threadIdx.x; i < QB * C; i += blockDim.x) {
    int qi = i / C, c = i - qi * C;
    if (q0 + qi < nq) out[((int64_t)(q0 + qi) * splits + split) * C + c] = S.kept[(size_t)qi * C + c];
  }
}

// ---------------------------------------------------------------------------------
// Register-blocked variant for C <= 128 (k <= 128): 64 queries a CTA, warp w owns
// queries 8w .. 8w+7 and lane l points 4l .. 4l+3 of each 128-point tile, so a thread
// keeps an 8 x 4 micro-tile (32 FMAs per dimension step for three shared loads).  A
// query's top-C list lives in shared memory; candidates that beat the query's threshold
// (one warp vote a tile) are appended to its 32-key buffer and merged into the list only
// when the buffer fills -- in a short split nearly every tile brings a candidate, and a
// merge a tile would cost more than the tile's FMAs.  There is no block-level selection
// protocol and no barrier besides the tile copy's.  Held to 128 registers so that two
// CTAs share an SM whenever their shared memory fits (d <= ~106 at C = 32).
// ---------------------------------------------------------------------------------
constexpr int kRegQB = 64;
constexpr int kRegBuf = 32;  // candidate keys a query buffers before a merge
constexpr size_t kRegTwoCtaSmem = 112 * 1024;  // shared memory that lets two CTAs share an SM

__host__ __device__ inline size_t reg_scan_smem(int d, int C, int nbuf) {
  size_t off = 0;
  smem_take(off, (size_t)nbuf * kTile * d * 4);  // point tiles
  smem_take(off, (size_t)kRegQB * d * 4);        // queries, [j][64]
  smem_take(off, (size_t)kRegQB * 4);            // query magnitudes
  smem_take(off, (size_t)kRegQB * C * 8);        // top-C lists
  smem_take(off, (size_t)8 * 32 * 8);            // per-warp scratch
  smem_take(off, (size_t)kRegQB * kRegBuf * 8);  // candidate buffers
  return off;
}

// Merge a query's buffered candidates (cnt <= kRegBuf keys, all below the list's
// threshold when they were added) into its sorted list of C = 32*EC keys; returns the new
// threshold.  Executed by the whole warp.
template <int EC>
__device__ __noinline__ uint64_t fold_candidates(uint64_t* list, const uint64_t* buf, int cnt) {
  const int lane = threadIdx.x & 31;
  uint64_t y[2] = {lane < cnt ? buf[lane] : kEmptyKey, lane + 32 < cnt ? buf[lane + 32] : kEmptyKey};
  warp_bitonic<2>(y, lane, false);  // element e*32 + lane, ascending
  uint64_t x[EC];
#pragma unroll
  for (int e = 0; e < EC; ++e) x[e] = e < 2 ? y[e] : kEmptyKey;  // the 32*EC smallest, ascending
  uint64_t best[EC];
#pragma unroll
  for (int e = 0; e < EC; ++e) best[e] = list[e * 32 + lane];
#pragma unroll
  for (int e = 0; e < EC; ++e) {
    const uint64_t r = __shfl_sync(0xffffffffu, x[EC - 1 - e], 31 - lane);
    best[e] = best[e] < r ? best[e] : r;
  }
  warp_bitonic<EC>(best, lane, true);
#pragma unroll
  for (int e = 0; e < EC; ++e) list[e * 32 + lane] = best[e];
  return __shfl_sync(0xffffffffu, best[EC - 1], 31);
}

// Merge one query's candidates (k0..k3 on every lane: 128 keys, only those below `thr`
// count) into its sorted list of C = 32*EC keys in shared memory; returns the new
// threshold (the list's last key).  Few survivors are compacted to one key a lane and
// sorted; more than 32 sort all 128.  Executed by the whole warp; kept out of line
// because it runs rarely.
template <int EC>
__device__ __noinline__ uint64_t merge_candidates(uint64_t* list, uint64_t k0, uint64_t k1, uint64_t k2,
                                                  uint64_t k3, uint64_t thr, uint64_t* scratch) {
  const int lane = threadIdx.x & 31;
  const int cnt = (k0 < thr) + (k1 < thr) + (k2 < thr) + (k3 < thr);
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  uint64_t x[EC];
  if (total <= 32) {
    int pos = incl - cnt;
    if (k0 < thr) scratch[pos++] = k0;
    if (k1 < thr) scratch[pos++] = k1;
    if (k2 < thr) scratch[pos++] = k2;
    if (k3 < thr) scratch[pos++] = k3;
    __syncwarp();
    x[0] = lane < total ? scratch[lane] : kEmptyKey;
#pragma unroll
    for (int e = 1; e < EC; ++e) x[e] = kEmptyKey;
    __syncwarp();
    warp_bitonic<EC>(x, lane, false);
  } else {
    uint64_t y[4] = {k0 < thr ? k0 : kEmptyKey, k1 < thr ? k1 : kEmptyKey, k2 < thr ? k2 : kEmptyKey,
                     k3 < thr ? k3 : kEmptyKey};
    warp_bitonic<4>(y, lane, false);
#pragma unroll
    for (int e = 0; e < EC; ++e) x[e] = y[e];  // the 32*EC smallest candidates, ascending
  }
  uint64_t best[EC];
#pragma unroll
  for (int e = 0; e < EC; ++e) best[e] = list[e * 32 + lane];
  // best ascending, x ascending: min(best[i], x[C-1-i]) is bitonic and holds the C smallest
#pragma unroll
  for (int e = 0; e < EC; ++e) {
    const uint64_t r = __shfl_sync(0xffffffffu, x[EC - 1 - e], 31 - lane);
    best[e] = best[e] < r ? best[e] : r;
  }
  warp_bitonic<EC>(best, lane, true);
#pragma unroll
  for (int e = 0; e < EC; ++e) list[e * 32 + lane] = best[e];
  return __shfl_sync(0xffffffffu, best[EC - 1], 31);
}

template <int DIST, int EC>
__global__ void __launch_bounds__(256, 2) scan_float_reg_kernel(
    const float* __restrict__ xt, int64_t n, int d, const float* __restrict__ xnorm, const float* __restrict__ q,
    int nq, const float* __restrict__ qnorm, int tiles_per_split, int splits, int nbuf, uint64_t* __restrict__ out) {
  constexpr int C = 32 * EC;
  extern __shared__ __align__(16) unsigned char smem[];
  size_t off = 0;
  float* xs = reinterpret_cast<float*>(smem + smem_take(off, (size_t)nbuf * kTile * d * 4));
  float* qs = reinterpret_cast<float*>(smem + smem_take(off, (size_t)kRegQB * d * 4));
  float* qn = reinterpret_cast<float*>(smem + smem_take(off, (size_t)kRegQB * 4));
  uint64_t* lists = reinterpret_cast<uint64_t*>(smem + smem_take(off, (size_t)kRegQB * C * 8));
  uint64_t* scratch = reinterpret_cast<uint64_t*>(smem + smem_take(off, (size_t)8 * 32 * 8));
  uint64_t* cbuf = reinterpret_cast<uint64_t*>(smem + smem_take(off, (size_t)kRegQB * kRegBuf * 8));

  const int q0 = blockIdx.x * kRegQB;
  const int split = blockIdx.y;
  const int ntiles = (int)((n + kTile - 1) / kTile);
  const int t_begin = split * tiles_per_split;
  const int t_end = min(ntiles, t_begin + tiles_per_split);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (int i = threadIdx.x; i < kRegQB * d; i += blockDim.x) {
    const int qi = i / d, j = i - qi * d;
    qs[j * kRegQB + qi] = (q0 + qi < nq) ? q[(int64_t)(q0 + qi) * d + j] : 0.0f;
  }
  for (int qi = threadIdx.x; qi < kRegQB; qi += blockDim.x)
    qn[qi] = (DIST == DIST_ANGULAR && q0 + qi < nq) ? qnorm[q0 + qi] : 1.0f;
  for (int i = threadIdx.x; i < kRegQB * C; i += blockDim.x) lists[i] = kEmptyKey;
  __syncthreads();  // lists are read by their owning warps (and written out even for an empty split)
  uint64_t thr[8];
  int bcnt[8];  // buffered candidates a query (warp-uniform)
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    thr[a] = kEmptyKey;
    bcnt[a] = 0;
  }
  const unsigned lt_mask = (1u << lane) - 1u;

  const int tile_f4 = kTile * d / 4;
  auto slot = [&](int tile) { return nbuf == 2 ? (tile & 1) : 0; };
  auto issue_tile = [&](int tile) {
    const float4* src = reinterpret_cast<const float4*>(xt + (int64_t)tile * kTile * d);
    float4* dst = reinterpret_cast<float4*>(xs) + (size_t)slot(tile) * tile_f4;
    for (int i = threadIdx.x; i < tile_f4; i += blockDim.x) cp_async16(dst + i, src + i);
    cp_async_commit();
  };
  if (t_begin < t_end) issue_tile(t_begin);
  for (int tile = t_begin; tile < t_end; ++tile) {
    if (nbuf == 2 && tile + 1 < t_end) {
      issue_tile(tile + 1);  // its buffer was last read by tile - 1, finished at the barrier below
      cp_async_wait<1>();
    } else {
      if (nbuf == 1 && tile > t_begin) issue_tile(tile);
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* xcur = xs + (size_t)slot(tile) * kTile * d;

    float acc[8][4], acc2[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) { acc[a][b] = 0.0f; acc2[a][b] = 0.0f; }
#pragma unroll 4
    for (int j = 0; j < d; ++j) {
      const float4 xv = *reinterpret_cast<const float4*>(&xcur[j * kTile + 4 * lane]);
      const float4 qa0 = *reinterpret_cast<const float4*>(&qs[j * kRegQB + 8 * w]);
      const float4 qa1 = *reinterpret_cast<const float4*>(&qs[j * kRegQB + 8 * w + 4]);
      const float xb[4] = {xv.x, xv.y, xv.z, xv.w};
      const float qv[8] = {qa0.x, qa0.y, qa0.z, qa0.w, qa1.x, qa1.y, qa1.z, qa1.w};
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          if (DIST == DIST_ANGULAR) {
            acc[a][b] = __fmaf_rn(qv[a], xb[b], acc[a][b]);
          } else if (DIST == DIST_JACCARD) {
            acc[a][b] = __fadd_rn(acc[a][b], fminf(xb[b], qv[a]));
            acc2[a][b] = __fadd_rn(acc2[a][b], fmaxf(xb[b], qv[a]));
          } else {
            const float df = __fsub_rn(qv[a], xb[b]);
            acc[a][b] = __fmaf_rn(df, df, acc[a][b]);
          }
        }
    }
    const int64_t pbase = (int64_t)tile * kTile + 4 * lane;
    float xn[4], xinv[4];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      xn[b] = (DIST == DIST_ANGULAR && pbase + b < n) ? xnorm[pbase + b] : 1.0f;
      xinv[b] = __frcp_rn(xn[b]);
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int qi = 8 * w + a;
      if (q0 + qi >= nq) continue;  // warp-uniform
      // Angular pre-filter: 1 - dot * (1/|q|) * (1/|x|) is within ~5e-7 of the exact
      // 1 - dot / (|q| |x|), so a pair whose estimate exceeds the threshold's distance by
      // more than 1e-5 cannot enter the list and skips the exact divide; NaN or infinite
      // estimates (zero norms) and an empty list (NaN threshold) always take the exact path.
      const float bound = key_dist(thr[a]) + 1e-5f;
      const float qinv = __frcp_rn(qn[qi]);
      uint64_t k[4];
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        k[b] = kEmptyKey;
        if (pbase + b < n) {
          const bool skip = DIST == DIST_ANGULAR && __fmaf_rn(-acc[a][b], __fmul_rn(qinv, xinv[b]), 1.0f) > bound;
          if (!skip) k[b] = make_key(finish_distance<DIST>(acc[a][b], acc2[a][b], qn[qi], xn[b]), (int)(pbase + b));
        }
      }
      if (!__any_sync(0xffffffffu, k[0] < thr[a] || k[1] < thr[a] || k[2] < thr[a] || k[3] < thr[a])) continue;
      uint64_t* qbuf = cbuf + (size_t)qi * kRegBuf;
      unsigned m[4];
      int nc = 0;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        m[b] = __ballot_sync(0xffffffffu, k[b] < thr[a]);
        nc += __popc(m[b]);
      }
      if (bcnt[a] + nc > kRegBuf) {
        if (bcnt[a] > 0) {  // make room: merge the buffer, then re-filter with the new threshold
          thr[a] = fold_candidates<EC>(lists + (size_t)qi * C, qbuf, bcnt[a]);
          bcnt[a] = 0;
          nc = 0;
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            m[b] = __ballot_sync(0xffffffffu, k[b] < thr[a]);
            nc += __popc(m[b]);
          }
        }
        if (nc > kRegBuf) {  // more than a buffer's worth in one tile: merge them directly
          thr[a] = merge_candidates<EC>(lists + (size_t)qi * C, k[0], k[1], k[2], k[3], thr[a], scratch + w * 32);
          continue;
        }
      }
      int pos = bcnt[a];
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        if (m[b] & (1u << lane)) qbuf[pos + __popc(m[b] & lt_mask)] = k[b];
        pos += __popc(m[b]);
      }
      bcnt[a] = pos;
      __syncwarp();
    }
    __syncthreads();  // every read of this tile's buffer is done: the next copy may reuse it
  }

#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int qi = 8 * w + a;
    if (q0 + qi >= nq) continue;
    if (bcnt[a] > 0) fold_candidates<EC>(lists + (size_t)qi * C, cbuf + (size_t)qi * kRegBuf, bcnt[a]);
#pragma unroll
    for (int e = 0; e < EC; ++e)
      out[((int64_t)(q0 + qi) * splits + split) * C + e * 32 + lane] = lists[(size_t)qi * C + e * 32 + lane];
  }
}

template <int DIST, int EC>
void launch_reg(const float* xt, int64_t n, int d, const float* xnorm, const float* q, int nq, const float* qnorm,
                int splits, int nbuf, uint64_t* out, cudaStream_t s) {
  ProfScope _ps("scan_float", s);
  const size_t smem = reg_scan_smem(d, 32 * EC, nbuf);
  auto kern = scan_float_reg_kernel<DIST, EC>;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int ntiles = ceil_div(n, kTile);
  const int tps = ceil_div(ntiles, splits);
  dim3 grid(ceil_div(nq, kRegQB), splits);
  kern<<<grid, 256, smem, s>>>(xt, n, d, xnorm, q, nq, qnorm, tps, splits, nbuf, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

// The register-blocked kernel serves C <= 128 when its shared memory fits; returns false
// otherwise (the general kernel runs).
template <int DIST>
bool try_launch_reg(const float* xt, int64_t n, int d, const float* xnorm, const float* q, int nq,
                    const float* qnorm, int C, int splits, uint64_t* out, cudaStream_t s) {
  if (C > 128) return false;
  // two CTAs an SM (one tile buffer: while one CTA copies, the other computes) when the
  // shared memory allows, else one CTA with a double-buffered tile
  const size_t cap = 220 * 1024;
  int nbuf = reg_scan_smem(d, C, 1) <= kRegTwoCtaSmem ? 1
             : (reg_scan_smem(d, C, 2) <= cap ? 2 : (reg_scan_smem(d, C, 1) <= cap ? 1 : 0));
  if (!nbuf) return false;
  if (C == 32) launch_reg<DIST, 1>(xt, n, d, xnorm, q, nq, qnorm, splits, nbuf, out, s);
  else if (C == 64) launch_reg<DIST, 2>(xt, n, d, xnorm, q, nq, qnorm, splits, nbuf, out, s);
  else if (C == 128) launch_reg<DIST, 4>(xt, n, d, xnorm, q, nq, qnorm, splits, nbuf, out, s);
  else return false;
  return true;
}

struct FloatCfg {
  int QB, MQ, nbuf;
};

FloatCfg pick_float_cfg(int d, int C) {
  const size_t cap = 220 * 1024;
  for (int nbuf = 2; nbuf >= 1; --nbuf) {
    if (C <= 128 && float_scan_layout(d, 32, C, nbuf).total <= cap) return {32, 4, nbuf};
    if (C <= 1024 && float_scan_layout(d, 8, C, nbuf).total <= cap) return {8, 1, nbuf};
    if (float_scan_layout(d, 2, C, nbuf).total <= cap) return {2, 1, nbuf};
  }
  throw Error(LSHG_ERR_UNSUPPORTED, "float scan: dimension / candidate count too large for shared memory");
}

template <int DIST, int QB, int MQ>
void launch_cfg(const float* xt, int64_t n, int d, const float* xnorm, const float* q, int nq, const float* qnorm,
                int C, int splits, int nbuf, uint64_t* out, cudaStream_t s) {
  ProfScope _ps("scan_float", s);
  size_t smem = float_scan_layout(d, QB, C, nbuf).total;
  auto kern = scan_float_kernel<DIST, QB, MQ>;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int ntiles = ceil_div(n, kTile);
  int tps = ceil_div(ntiles, splits);
  dim3 grid(ceil_div(nq, QB), splits);
  kern<<<grid, (QB / MQ) * 32, smem, s>>>(xt, n, d, xnorm, q, nq, qnorm, C, tps, splits, nbuf, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

template <int DIST>
void launch_dist(const float* xt, int64_t n, int d, const float* xnorm, const float* q, int nq, const float* qnorm,
                 int C, int splits, uint64_t* out, cudaStream_t s) {
  if (try_launch_reg<DIST>(xt, n, d, xnorm, q, nq, qnorm, C, splits, out, s)) return;
  FloatCfg c = pick_float_cfg(d, C);
  if (c.QB == 32) launch_cfg<DIST, 32, 4>(xt, n, d, xnorm, q, nq, qnorm, C, splits, c.nbuf, out, s);
  else if (c.QB == 8) launch_cfg<DIST, 8, 1>(xt, n, d, xnorm, q, nq, qnorm, C, splits, c.nbuf, out, s);
  else launch_cfg<DIST, 2, 1>(xt, n, d, xnorm, q, nq, qnorm, C, splits, c.nbuf, out, s);
}

}  // namespace

int scan_float_splits(int64_t n, int nq, int C) {
  // C <= 128 runs the register-blocked kernel (64-query CTAs; the split count is sized as
  // for one an SM, a second one an SM, where it fits, hides the first one's tile copies),
  // larger C the general one (two CTAs an SM); pick the split count whose grid fills whole waves best
  // among those giving at least ~2 CTAs an SM slot, at most 4x that and 64
  const int QB = C <= 128 ? kRegQB : (C <= 1024 ? 8 : 2);
  const int slots = num_sms() * (C <= 128 ? 1 : 2);
  const int qblocks = ceil_div(nq, QB);
  const int ntiles = ceil_div(n, kTile);
  const int maxs = std::max(1, std::min(ntiles / 4, 64));
  const int want = std::max(1, std::min(maxs, ceil_div((int64_t)slots * 2, qblocks)));
  int best = want;
  double best_eff = 0.0;
  for (int sp = want; sp <= std::min(maxs, 4 * want); ++sp) {
    const int64_t ctas = (int64_t)qblocks * sp;
    const double eff = (double)ctas / (double)(ceil_div(ctas, slots) * (int64_t)slots);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = sp;
    }
  }
  return best;
}

int launch_scan_float(const float* xt, int64_t n, int d, const float* xnorm, const float* q, int nq,
                      const float* qnorm, int dist, int C, int splits, uint64_t* out, cudaStream_t s) {
  if (nq <= 0) return splits;
  LSHG_REQUIRE(n > 0, "float scan: empty base");
  LSHG_REQUIRE(C >= 32 && (C & (C - 1)) == 0, "float scan: C must be a power of two >= 32");
  switch (dist) {
    case DIST_ANGULAR: launch_dist<DIST_ANGULAR>(xt, n, d, xnorm, q, nq, qnorm, C, splits, out, s); break;
    case DIST_JACCARD: launch_dist<DIST_JACCARD>(xt, n, d, xnorm, q, nq, qnorm, C, splits, out, s); break;
    case DIST_EUCLID: launch_dist<DIST_EUCLID>(xt, n, d, xnorm, q, nq, qnorm, C, splits, out, s); break;
    case DIST_SQEUCLID: launch_dist<DIST_SQEUCLID>(xt, n, d, xnorm, q, nq, qnorm, C, splits, out, s); break;
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "float scan: invalid distance function");
  }
  return splits;
}

}  // namespace lshg
