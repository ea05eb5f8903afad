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
  FloatCfg c = pick_float_cfg(d, C);
  if (c.QB == 32) launch_cfg<DIST, 32, 4>(xt, n, d, xnorm, q, nq, qnorm, C, splits, c.nbuf, out, s);
  else if (c.QB == 8) launch_cfg<DIST, 8, 1>(xt, n, d, xnorm, q, nq, qnorm, C, splits, c.nbuf, out, s);
  else launch_cfg<DIST, 2, 1>(xt, n, d, xnorm, q, nq, qnorm, C, splits, c.nbuf, out, s);
}

}  // namespace

int scan_float_splits(int64_t n, int nq, int C) {
  int QB = C <= 128 ? 32 : (C <= 1024 ? 8 : 2);
  int qblocks = ceil_div(nq, QB);
  int ntiles = ceil_div(n, kTile);
  int want = ceil_div((int64_t)num_sms() * 2, qblocks);
  int maxs = std::max(1, ntiles / 4);
  return std::max(1, std::min(std::min(want, maxs), 64));
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
