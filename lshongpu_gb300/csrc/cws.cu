// Consistent weighted sampling (implementation 10): Ioffe's improved consistent weighted
// sampling (ICWS, "Improved Consistent Sampling, Weighted Minhash and L1 Sketching",
// ICDM 2010) for the generalized Jaccard similarity sum(min) / sum(max) of nonnegative
// vectors.  The reference's weighted MinHash is a rejection sampler whose byte samples
// wrap (weightedMinHash.cuh:98-166, built bit for bit in wmh.cu); this sketch keeps
// (index, int32) samples instead, and two vectors' samples agree with probability equal
// to their generalized Jaccard similarity.  The data go through the reference's weighted
// MinHash preprocessing first (shift by |min floor|, L2 normalisation,
// processingUtils.cuh:12-67), so the re-rank is the same generalized Jaccard distance on
// the same rows (distanceFunctions.cuh:102-116).
//
// Sample j of a vector S: for every dimension i with S_i > 0, with r, c ~ Gamma(2, 1) and
// beta ~ U(0, 1) drawn for (j, i) once for all vectors,
//     t_i = floor(ln S_i / r + beta),   ln a_i = ln c - r (t_i - beta + 1),
// and the sample is (i*, t_i*) for i* = argmin ln a_i (the lowest i on ties); a vector with
// no positive entry gets (d, 0).  The draws are a table [d][S] of (r, 1/r, ln c, beta)
// made on the host from a counter-based generator (cws_tables); the per-vector arithmetic
// is single precision, rounded step by step in a fixed order (no fused multiply-adds), with
// its own logarithm, so the samples are a deterministic function of the table and the
// data that a CPU restatement reproduces bit for bit.
//
// Scan: samples are recoded against the base's range of t (a dimension index and an
// offset of t, at most 16 bits; a query sample outside the range gets a code no base
// sample has).  When no sample position holds more than 255 distinct base codes, each
// code is replaced by its rank in its position's dictionary (a byte; 255 for a code the
// base does not have there), so the scan compares bytes like the byte weighted MinHash;
// otherwise the 16-bit codes are kept.  The codes are bit-sliced into 8 or 16 planes and
// go through the byte scan's threshold filter (slice_filter.cuh).  Batches below 64 queries, queries whose
// survivors the filter cannot select exactly, and bases whose codes would need more than
// 16 bits are scanned directly over the (index, t) pairs.  Either way the candidates are
// the exact top-C by (1 - matches / S, id).
#include <cmath>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "profile.h"
#include "select.cuh"
#include "slice_filter.cuh"

namespace lshg {

namespace {

constexpr int kTile = 128;

// Natural logarithm of a positive finite float: x = m 2^e with m in [sqrt(1/2), sqrt(2)],
// ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + s^7/7 + s^9/9), s = (m - 1) / (m + 1)
// (|s| <= 0.1716, so the first omitted term is below 2e-9 of the result), and
// ln x = e ln2 + ln m with ln2 split in a high part that e multiplies exactly and a low
// part.  Every operation is a single correctly rounded one.
__device__ __forceinline__ float cws_logf(float x) {
  int e = 0;
  uint32_t u = __float_as_uint(x);
  if (u < 0x00800000u) {  // subnormal: scale by 2^24 (exact)
    u = __float_as_uint(__fmul_rn(x, 16777216.0f));
    e = -24;
  }
  e += (int)(u >> 23) - 127;
  float m = __uint_as_float((u & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421354f) {
    m = __fmul_rn(m, 0.5f);
    e += 1;
  }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float z = __fmul_rn(s, s);
  float p = 0.222222224f;                           // 2/9
  p = __fadd_rn(__fmul_rn(p, z), 0.285714298f);     // 2/7
  p = __fadd_rn(__fmul_rn(p, z), 0.400000006f);     // 2/5
  p = __fadd_rn(__fmul_rn(p, z), 0.666666687f);     // 2/3
  p = __fadd_rn(__fmul_rn(p, z), 2.0f);
  const float lnm = __fmul_rn(p, s);
  const float ef = (float)e;
  return __fadd_rn(__fmul_rn(ef, 0.693145752f), __fadd_rn(__fmul_rn(ef, 1.42860677e-06f), lnm));
}

// One warp a vector: the logarithms of its positive entries in shared memory (+inf marks
// a dimension that takes no part), then each lane takes samples j = lane, lane + 32, ...
// and walks the dimensions in order.  Table rows [i][j] make a warp's loads of one
// dimension's draws for 32 consecutive samples one contiguous 512-byte read.
__global__ void __launch_bounds__(256) cws_sketch_kernel(const float* __restrict__ x, int64_t rows, int d, int S,
                                                         const float4* __restrict__ tab, int2* __restrict__ out) {
  extern __shared__ float lns[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* L = lns + (size_t)warp * d;
  for (int64_t r = (int64_t)blockIdx.x * 8 + warp; r < rows; r += (int64_t)gridDim.x * 8) {
    for (int i = lane; i < d; i += 32) {
      const float v = x[r * d + i];
      L[i] = (v > 0.0f && v < INFINITY) ? cws_logf(v) : INFINITY;
    }
    __syncwarp();
    for (int j = lane; j < S; j += 32) {
      float best = INFINITY;
      int bk = d, bt = 0;
      for (int i = 0; i < d; ++i) {
        const float l = L[i];
        if (l == INFINITY) continue;  // the same for every lane
        const float4 T = tab[(int64_t)i * S + j];  // r, 1/r, ln c, beta
        float v = __fadd_rn(__fmul_rn(l, T.y), T.w);
        v = fminf(fmaxf(v, -1.0e9f), 1.0e9f);
        const float tf = floorf(v);
        const float la = __fsub_rn(T.z, __fmul_rn(T.x, __fadd_rn(__fsub_rn(tf, T.w), 1.0f)));
        if (la < best) {
          best = la;
          bk = i;
          bt = (int)tf;
        }
      }
      out[r * S + j] = make_int2(bk, bt);
    }
    __syncwarp();
  }
}

// Range of t over every sample of the base: range[0] = min, range[1] = max.
__global__ void cws_range_kernel(const int2* __restrict__ smp, int64_t total, int* __restrict__ range) {
  int lo = INT_MAX, hi = INT_MIN;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int t = smp[i].y;
    lo = min(lo, t);
    hi = max(hi, t);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&range[0], lo);
    atomicMax(&range[1], hi);
  }
}

// Per-position code dictionary of the base: bit `code` of row j of `bits` ([S][2^P / 32]
// words) is set when some base point's sample j has that code.
__global__ void cws_dict_mark_kernel(const int2* __restrict__ smp, int64_t total, int S, int tmin, int tb, int words,
                                     uint32_t* __restrict__ bits) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % S);
    const int2 v = smp[i];
    const uint32_t code = ((uint32_t)v.x << tb) | (uint32_t)(v.y - tmin);  // base samples: always in range
    atomicOr(&bits[(int64_t)j * words + (code >> 5)], 1u << (code & 31));
  }
}

// One block a sample position: rank of every code among the position's set bits (255 for
// codes not set, and for ranks past 254 -- the host then drops the dictionary), and the
// position's code count into *maxcount.
__global__ void __launch_bounds__(256) cws_dict_rank_kernel(const uint32_t* __restrict__ bits, int words,
                                                            uint8_t* __restrict__ rank, int* __restrict__ maxcount) {
  __shared__ int part[256];
  const int j = blockIdx.x, tid = threadIdx.x;
  const uint32_t* b = bits + (int64_t)j * words;
  const int per = (words + 255) / 256, w0 = tid * per, w1 = min(words, w0 + per);
  int own = 0;
  for (int w = w0; w < w1; ++w) own += __popc(b[w]);
  part[tid] = own;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {  // inclusive scan
    const int v = tid >= o ? part[tid - o] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  int base = part[tid] - own;
  uint8_t* r = rank + ((int64_t)j * words << 5);
  for (int w = w0; w < w1; ++w) {
    const uint32_t x = b[w];
    for (int k = 0; k < 32; ++k) {
      const int at = base + __popc(x & ((1u << k) - 1u));
      r[w * 32 + k] = ((x >> k) & 1u) && at < 255 ? (uint8_t)at : (uint8_t)255;
    }
    base += __popc(x);
  }
  if (tid == 255) atomicMax(maxcount, part[255]);
}

// Samples [rows][S] -> codes bit-sliced into rows of ng * PL words (word g PL + b holds
// bit b of the codes of samples 32 g .. 32 g + 31).  code = (i << tb) | (t - tmin) for
// i <= d and t in [tmin, tmin + 2^tb); anything else gets the code (d + 1) << tb, which no
// base sample has.  Samples past S get `pad` (0 for the base, all ones for queries, so
// padding never matches).  One thread a (row, group).
// rank (optional, dictionary codes): [S][2^rlog] bytes, the code's rank among the codes the
// base has at that sample position, 255 for a code no base sample has there.
template <int PL>
__global__ void cws_slice_kernel(const int2* __restrict__ smp, int64_t rows, int S, int ng, int d, int tmin, int tb,
                                 const uint8_t* __restrict__ rank, int rlog, uint32_t pad, uint32_t* __restrict__ out) {
  const int64_t total = rows * ng;
  const uint32_t tspan = 1u << tb, sentinel = (uint32_t)(d + 1) << tb;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = w / ng;
    const int g = (int)(w - r * ng);
    uint32_t code[32];
#pragma unroll
    for (int s = 0; s < 32; ++s) {
      const int j = 32 * g + s;
      uint32_t c = pad;
      if (j < S) {
        const int2 v = smp[r * S + j];
        const int64_t dt = (int64_t)v.y - tmin;
        c = (v.x >= 0 && v.x <= d && dt >= 0 && dt < (int64_t)tspan) ? (((uint32_t)v.x << tb) | (uint32_t)dt)
                                                                      : sentinel;
        if (rank) c = rank[((int64_t)j << rlog) + c];
      }
      code[s] = c;
    }
    uint32_t* o = out + (r * ng + g) * PL;
#pragma unroll
    for (int b = 0; b < PL; ++b) {
      uint32_t word = 0;
#pragma unroll
      for (int s = 0; s < 32; ++s) word |= ((code[s] >> b) & 1u) << s;
      o[b] = word;
    }
  }
}

// LSH keys from CWS samples (keysImplementation 10): table t's key hashes its K samples
// t K .. t K + K - 1 -- h = mix(h ^ (index << 32 | t)) per sample, from the table number,
// with splitmix64's finaliser -- and keeps the top `bits` bits.  Equal samples give equal
// keys, so two vectors share table t's bucket with probability at least J^K.
__device__ __forceinline__ uint64_t key_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void cws_keys_kernel(const int2* __restrict__ smp, int64_t rows, int L, int K, int bits,
                                uint16_t* __restrict__ keys) {
  const int64_t total = rows * L;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = w / L;
    const int t = (int)(w - r * L);
    uint64_t h = 0x9E3779B97F4A7C15ull * (uint64_t)(t + 1);
    for (int j = 0; j < K; ++j) {
      const int2 v = smp[r * (int64_t)L * K + (int64_t)t * K + j];
      h = key_mix(h ^ (((uint64_t)(uint32_t)v.x << 32) | (uint32_t)v.y));
    }
    keys[w] = (uint16_t)(h >> (64 - bits));
  }
}

struct DirectSmem {
  size_t qs, kept, buf, thr, cnt, total;
};

__host__ __device__ inline size_t take(size_t& off, size_t bytes) {
  off = (off + 15) / 16 * 16;
  const size_t at = off;
  off += bytes;
  return at;
}

__host__ __device__ inline DirectSmem direct_layout(int S, int QB, int C, int kbuf) {
  DirectSmem L;
  size_t off = 0;
  L.qs = take(off, (size_t)QB * S * 8);
  L.kept = take(off, (size_t)QB * C * 8);
  L.buf = take(off, (size_t)QB * kbuf * 8);
  L.thr = take(off, (size_t)QB * 8);
  L.cnt = take(off, (size_t)QB * 4);
  L.total = off;
  return L;
}

// Direct scan: the exact top-C by (1 - matches / S, id) of QB = 2 queries a CTA over the
// base's samples, tiled [tile][S / 2][128] in 16-byte chunks (two samples a chunk; the
// lanes of a warp read 32 consecutive points' chunk as one 512-byte run).  Selection as
// in the popcount sketch scan: keys below a query's threshold go to an append buffer that
// is folded into the sorted top-C list every T tiles when a buffer passed its limit.
// list (optional): scan only the queries list[1 .. list[0]], results to their rows.
template <int KBUF, int T>
__global__ void __launch_bounds__(256, 2)
    cws_direct_kernel(const uint4* __restrict__ xst, int64_t n, int S, const int2* __restrict__ qs, int nq, int C,
                      int tiles_per_split, int splits, uint64_t* __restrict__ out, const int* __restrict__ list) {
  constexpr int QB = 2;
  static_assert(KBUF >= T * kTile, "append buffer must absorb T tiles");
  constexpr int kLimit = KBUF - T * kTile;
  extern __shared__ __align__(16) unsigned char smem[];
  const DirectSmem L = direct_layout(S, QB, C, KBUF);
  int2* qsm = reinterpret_cast<int2*>(smem + L.qs);
  TopCShared Sh{reinterpret_cast<uint64_t*>(smem + L.kept), reinterpret_cast<uint64_t*>(smem + L.buf),
                reinterpret_cast<int*>(smem + L.cnt), reinterpret_cast<uint64_t*>(smem + L.thr), C, KBUF};
  const int nqe = list ? list[0] : nq;
  const int q0 = blockIdx.x * QB;
  if (q0 >= nqe) return;  // block-uniform, before any barrier
  const int split = blockIdx.y;
  const int ntiles = (int)((n + kTile - 1) / kTile);
  const int t_begin = split * tiles_per_split;
  const int t_end = min(ntiles, t_begin + tiles_per_split);
  for (int i = threadIdx.x; i < QB * S; i += blockDim.x) {
    const int qi = i / S;
    const int64_t qrow = q0 + qi < nqe ? (list ? list[1 + q0 + qi] : q0 + qi) : 0;
    qsm[i] = q0 + qi < nqe ? qs[qrow * S + (i - qi * S)] : make_int2(-1, 0);
  }
  topc_init(Sh, QB);
  __syncthreads();
  const int qi = threadIdx.x >> 7, pl = threadIdx.x & 127;
  const bool qvalid = q0 + qi < nqe;
  const int nc = S / 2;
  const float fs = (float)S;
  uint64_t thr = kEmptyKey;
  bool over = false;
  const int2* qr = qsm + qi * S;
  for (int tile = t_begin; tile < t_end; ++tile) {
    const int64_t p = (int64_t)tile * kTile + pl;
    if (p < n && qvalid) {
      const uint4* col = xst + (int64_t)tile * nc * kTile + pl;
      int m = 0;
      for (int c = 0; c < nc; ++c) {
        const uint4 v = __ldg(&col[(int64_t)c * kTile]);
        const int2 a = qr[2 * c], b = qr[2 * c + 1];
        m += ((int)v.x == a.x && (int)v.y == a.y) + ((int)v.z == b.x && (int)v.w == b.y);
      }
      const uint64_t key = make_key(__fsub_rn(1.0f, __fdiv_rn((float)m, fs)), (int)p);
      if (key < thr) {
        const int pos = atomicAdd(&Sh.cnt[qi], 1);
        Sh.buf[(size_t)qi * KBUF + pos] = key;
        over |= pos >= kLimit;
      }
    }
    if ((tile - t_begin) % T == T - 1 && tile + 1 < t_end) {  // uniform: same tile loop in every thread
      if (__syncthreads_or(over)) {
        topc_flush(Sh, QB, kLimit);
        thr = Sh.thr[qi];
      }
      over = false;
    }
  }
  topc_flush(Sh, QB, 0);
  for (int i = threadIdx.x; i < QB * C; i += blockDim.x) {
    const int qj = i / C, c = i - qj * C;
    if (q0 + qj < nqe) {
      const int64_t qrow = list ? list[1 + q0 + qj] : q0 + qj;
      out[(qrow * splits + split) * C + c] = Sh.kept[(size_t)qj * C + c];
    }
  }
}

template <int KBUF, int T>
void launch_direct_cfg(const uint32_t* xst, int64_t n, int S, const uint32_t* qs, int nq, int C, int splits,
                       uint64_t* out, const int* list, cudaStream_t s) {
  const size_t smem = direct_layout(S, 2, C, KBUF).total;
  auto kern = cws_direct_kernel<KBUF, T>;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int ntiles = ceil_div(n, kTile);
  const int tps = ceil_div(ntiles, splits);
  dim3 grid(ceil_div(nq, 2), splits);
  kern<<<grid, 256, smem, s>>>(reinterpret_cast<const uint4*>(xst), n, S, reinterpret_cast<const int2*>(qs), nq, C,
                               tps, splits, out, list);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_direct(const uint32_t* xst, int64_t n, int S, const uint32_t* qs, int nq, int C, int splits,
                   uint64_t* out, const int* list, cudaStream_t s) {
  if (nq <= 0) return;
  LSHG_REQUIRE(C >= 32 && C <= 4096 && (C & (C - 1)) == 0, "CWS scan: C must be a power of two in [32, 4096]");
  if (C <= 1024) launch_direct_cfg<1024, 4>(xst, n, S, qs, nq, C, splits, out, list, s);
  else launch_direct_cfg<2048, 8>(xst, n, S, qs, nq, C, splits, out, list, s);
}

}  // namespace

// splitmix64 (Steele, Lea and Flood, "Fast Splittable Pseudorandom Number Generators",
// OOPSLA 2014) as a counter hash: draw m of (sample j, dimension i) is
// mix(seed + (counter + 1) * golden), counter = (j * 65536 + i) * 8 + m, so a draw does
// not depend on the sketch length or the dimension count.
static uint64_t cws_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double cws_uniform(uint64_t seed, int j, int i, int m) {
  const uint64_t c = ((uint64_t)j * 65536u + (uint64_t)i) * 8u + (uint64_t)m;
  const uint64_t z = cws_mix(seed + (c + 1) * 0x9E3779B97F4A7C15ull);
  return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);  // (0, 1)
}

void cws_tables(int d, int S, std::vector<float>& tab, uint64_t seed) {
  tab.assign((size_t)d * S * 4, 0.0f);
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < S; ++j) {
      const double r = -(std::log(cws_uniform(seed, j, i, 0)) + std::log(cws_uniform(seed, j, i, 1)));  // Gamma(2, 1)
      const double c = -(std::log(cws_uniform(seed, j, i, 2)) + std::log(cws_uniform(seed, j, i, 3)));
      const float rf = (float)r;
      float* t = &tab[((size_t)i * S + j) * 4];
      t[0] = rf;
      t[1] = 1.0f / rf;
      t[2] = (float)std::log(c);
      t[3] = (float)cws_uniform(seed, j, i, 4);
    }
}

void launch_cws_keys(const uint32_t* smp, int64_t rows, int L, int K, int bits, uint16_t* keys, cudaStream_t s) {
  const int64_t total = rows * L;
  if (total <= 0) return;
  LSHG_REQUIRE(bits >= 1 && bits <= 16 && K >= 1, "CWS keys: bucketKeyBits in [1, 16], K >= 1");
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  cws_keys_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const int2*>(smp), rows, L, K, bits, keys);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_cws_sketch(const float* x, int64_t rows, int d, int S, const float* tab, uint32_t* out, cudaStream_t s) {
  if (rows <= 0) return;
  LSHG_REQUIRE(d >= 1 && d <= 4096, "CWS: d must be in [1, 4096]");
  const size_t smem = (size_t)8 * d * sizeof(float);
  LSHG_CUDA(cudaFuncSetAttribute(cws_sketch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (int)std::min<int64_t>((rows + 7) / 8, (int64_t)num_sms() * 8);
  cws_sketch_kernel<<<blocks, 256, smem, s>>>(x, rows, d, S, reinterpret_cast<const float4*>(tab),
                                              reinterpret_cast<int2*>(out));
  count_launch();
  LSHG_CHECK_LAUNCH();
}

CwsCodes cws_plan_codes(const uint32_t* xs, int64_t n, int S, int d, cudaStream_t s) {
  CwsCodes c{};
  int h_range[2] = {INT_MAX, INT_MIN};
  DevBuf<int> range(2, s);
  LSHG_CUDA(cudaMemcpyAsync(range.ptr, h_range, sizeof(h_range), cudaMemcpyHostToDevice, s));
  const int64_t total = n * S;
  if (total > 0) {
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 8);
    cws_range_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const int2*>(xs), total, range.ptr);
    count_launch();
    LSHG_CHECK_LAUNCH();
  }
  LSHG_CUDA(cudaMemcpyAsync(h_range, range.ptr, sizeof(h_range), cudaMemcpyDeviceToHost, s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  if (total <= 0) return c;
  int kb = 0;
  while ((1ll << kb) <= (int64_t)d + 1) ++kb;  // indices 0..d, and d + 1 for "no base sample"
  const int64_t span = (int64_t)h_range[1] - h_range[0];
  int tb = 0;
  while ((1ll << tb) <= span) ++tb;
  c.tmin = h_range[0];
  c.tmax = h_range[1];
  c.kb = kb;
  c.tb = tb;
  c.pl = kb + tb <= 8 ? 8 : (kb + tb <= 16 ? 16 : 0);
  return c;
}

bool cws_build_dict(const uint32_t* xs, int64_t n, int S, CwsCodes& c, DevBuf<uint8_t>& rank, cudaStream_t s) {
  const int P = c.kb + c.tb;
  if (c.pl != 16 || n <= 0) return false;  // codes of at most 8 bits need no dictionary
  const int rlog = std::max(P, 5), words = 1 << (rlog - 5);
  DevBuf<uint32_t> bits((size_t)S * words, s);
  LSHG_CUDA(cudaMemsetAsync(bits.ptr, 0, bits.bytes(), s));
  const int64_t total = n * S;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  cws_dict_mark_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const int2*>(xs), total, S, c.tmin, c.tb, words,
                                              bits.ptr);
  count_launch();
  LSHG_CHECK_LAUNCH();
  rank.alloc((size_t)S << rlog, s);
  DevBuf<int> maxc(1, s);
  LSHG_CUDA(cudaMemsetAsync(maxc.ptr, 0, sizeof(int), s));
  cws_dict_rank_kernel<<<S, 256, 0, s>>>(bits.ptr, words, rank.ptr, maxc.ptr);
  count_launch();
  LSHG_CHECK_LAUNCH();
  int h = 0;
  LSHG_CUDA(cudaMemcpyAsync(&h, maxc.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  if (h > 255) {  // some position holds more than 255 codes: keep the 16-plane codes
    rank.release();
    return false;
  }
  c.dict = 1;
  c.pl = 8;
  c.rlog = rlog;
  c.rank = rank.ptr;
  return true;
}

void launch_cws_slice(const uint32_t* smp, int64_t rows, int S, int d, const CwsCodes& c, bool query, uint32_t* out,
                      cudaStream_t s) {
  const int ng = (S + 31) / 32;
  const int64_t total = rows * ng;
  if (total <= 0) return;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  const int2* v = reinterpret_cast<const int2*>(smp);
  if (c.pl == 8)
    cws_slice_kernel<8><<<blocks, 256, 0, s>>>(v, rows, S, ng, d, c.tmin, c.tb, c.rank, c.rlog, query ? 0xFFu : 0u,
                                               out);
  else
    cws_slice_kernel<16><<<blocks, 256, 0, s>>>(v, rows, S, ng, d, c.tmin, c.tb, nullptr, 0, query ? 0xFFFFu : 0u,
                                                out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_cws_scan(const uint32_t* xsl_t, const uint32_t* xst, int64_t n, int S, int d, const CwsCodes& c,
                     const uint32_t* qs, int nq, int C, uint64_t* out, int* err, cudaStream_t s) {
  if (nq <= 0) return;
  LSHG_REQUIRE(n > 0, "CWS scan: empty base");
  ProfScope _ps("scan_cws", s);
  const int ng = (S + 31) / 32;
  int fs = 0, fr = 0, fc = 0;
  if (c.pl && xsl_t && nq >= 64 && byte_filter_plan(n, C, &fs, &fr, &fc)) {
    DevBuf<uint32_t> qsl((size_t)nq * ng * c.pl, s);
    launch_cws_slice(qs, nq, S, d, c, true, qsl.ptr, s);
    DevBuf<int> list((size_t)nq + 1, s);
    if (c.pl == 8) sliced_filter_select<8>(xsl_t, n, ng, S, qsl.ptr, nq, C, out, list.ptr, err, s);
    else sliced_filter_select<16>(xsl_t, n, ng, S, qsl.ptr, nq, C, out, list.ptr, err, s);
    launch_direct(xst, n, S, qs, nq, C, 1, out, list.ptr, s);  // listed queries: exact direct rescan
    return;
  }
  // direct scan of every query, the base split so that the grid fills the GPU
  const int qblocks = ceil_div(nq, 2);
  const int ntiles = ceil_div(n, kTile);
  const int splits = std::max(1, std::min(std::max(1, ntiles / 4), ceil_div((int64_t)num_sms() * 2, qblocks)));
  if (splits == 1) {
    launch_direct(xst, n, S, qs, nq, C, 1, out, nullptr, s);
    return;
  }
  DevBuf<uint64_t> part((size_t)nq * splits * C, s);
  launch_direct(xst, n, S, qs, nq, C, splits, part.ptr, nullptr, s);
  launch_merge_splits(part.ptr, nq, splits, C, out, s);
}

}  // namespace lshg
