// Threshold-filter scan of byte weighted-MinHash samples (implementation 4) for long
// candidate lists: the reference's scanJaccardDistance (sketchedDistanceScanners.cuh:
// 194-274) with the byte distance 1 - (#equal samples) / sketchDim (distanceFunctions.cuh:
// 102-116), for C > 128 candidates and batches of 64 queries or more.
//
// Two changes from the per-query top-C scan of scan_bits.cu:
//  * bit-sliced samples: a row holds, for every group of 32 samples, 8 words -- word i
//    has bit s set when bit i of sample 32g + s is set.  Samples s of a query and a point
//    are equal when all 8 of their bits are, so OR-ing the 8 XORed words of a group gives
//    the unequal samples, and 32 - popc(that) the equal ones: about 10 integer operations
//    for 32 samples, where comparing packed bytes takes about 14 for 8;
//  * no per-query list state: a query's top-C lists (32 KB at C = 4,096) left room for two
//    queries a CTA, so the base was streamed Q/2 times.  Instead a prepass over every S-th
//    tile builds each query's histogram of exact match counts (shared-memory atomics,
//    then one flush a block); hist_tau_kernel takes tau[q] = the match count at which the
//    sample's count from the top reaches r = C/S + 4 sqrt(C/S) + 8 (the query's C-th best
//    point puts about C/S sampled points above it); the filter pass keeps every point with
//    at least tau matches.  32 queries share a CTA, so the base streams Q/32 times.
// The survivors then go through the tensor-core sketch scan's integer select (the match
// count is the score) and queries with fewer than C survivors, or more than their array
// holds, are rescanned exactly by the per-query scan on the device; the candidate set is
// always the exact top-C by (distance, id).
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "profile.h"
#include "tc_filter.h"

namespace lshg {

int launch_scan_bits_listed(const uint32_t* xst, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq,
                            int op, int C, const int* list, uint64_t* out, cudaStream_t s);

namespace {

constexpr int kTile = 128;   // points a tile (one a thread of each half of the CTA)
constexpr int kFQB = 32;     // queries a CTA
constexpr int kMaxBins = 257;  // match counts 0..256

// Packed byte rows [n][wp] (byte j in bits 8 (j % 4) of word j / 4; bytes past wp * 4 are
// `pad`) -> bit-sliced rows [rows][8 * groups]: word 8 g + i, bit s = bit i of byte 32 g + s.
__global__ void slice_bytes_kernel(const uint32_t* __restrict__ xs, int64_t n, int wp, int groups, int64_t rows,
                                   uint32_t pad, uint32_t* __restrict__ out) {
  const int64_t total = rows * groups * 8;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / (groups * 8);
    const int gi = (int)(t - r * groups * 8), g = gi >> 3, bit = gi & 7;
    uint32_t w = 0;
#pragma unroll 4
    for (int s = 0; s < 32; ++s) {
      const int j = 32 * g + s;
      uint32_t b = pad;
      if (r < n && j < 4 * wp) b = (xs[r * wp + (j >> 2)] >> (8 * (j & 3))) & 0xFFu;
      w |= ((b >> bit) & 1u) << s;
    }
    out[t] = w;
  }
}

// MODE 0: histogram of match counts over the sampled positions (hist [nq][bins]);
// MODE 1: keep every point with at least tau[q] matches (keys make_key(-matches, id)).
// The sliced base is tiled as the popcount scan's ([tile][chunk][128] 16-byte chunks); a
// position p covers tile p * tstride.  NG: 32-sample groups a row.
template <int MODE, int NG>
__global__ void __launch_bounds__(256, 2)
    bytes_filter_kernel(const uint4* __restrict__ xst, int64_t n, const uint32_t* __restrict__ qsl, int nq, int NP,
                        int tstride, int per_split, const int* __restrict__ tau, int* __restrict__ hist, int bins,
                        int* __restrict__ cnt, uint64_t* __restrict__ cand, int cap) {
  constexpr int W = NG * 8, NCH = W / 4;
  __shared__ __align__(16) uint32_t qsm[kFQB * W];
  __shared__ int stau[kFQB];
  __shared__ int shist[MODE == 0 ? kFQB * kMaxBins : 1];
  const int q0 = blockIdx.x * kFQB, tid = threadIdx.x, lane = tid & 31;
  for (int i = tid; i < kFQB * W; i += blockDim.x) {
    const int qi = i / W;
    qsm[i] = q0 + qi < nq ? qsl[(int64_t)(q0 + qi) * W + (i - qi * W)] : 0u;
  }
  if (MODE == 1)
    for (int i = tid; i < kFQB; i += blockDim.x) stau[i] = q0 + i < nq ? tau[q0 + i] : INT_MAX;
  if (MODE == 0)
    for (int i = tid; i < kFQB * kMaxBins; i += blockDim.x) shist[i] = 0;
  __syncthreads();
  const int half = tid >> 7, pl = tid & 127;
  const int pbeg = blockIdx.y * per_split, pend = min(NP, pbeg + per_split);
  const unsigned lt = (1u << lane) - 1u;
  for (int pos = pbeg; pos < pend; ++pos) {
    const int64_t tile = (int64_t)pos * tstride;
    const int64_t p = tile * kTile + pl;
    const bool valid = p < n;
    uint4 xr[NCH];
#pragma unroll
    for (int c = 0; c < NCH; ++c) xr[c] = __ldg(&xst[(tile * NCH + c) * kTile + pl]);
#pragma unroll 1
    for (int a = 0; a < kFQB / 2; ++a) {
      const int qi = half + 2 * a;
      if (q0 + qi >= nq) break;  // the same for every thread of the half
      const uint4* qv = reinterpret_cast<const uint4*>(qsm + qi * W);
      int acc = 0;
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const uint4 x0 = xr[2 * g], x1 = xr[2 * g + 1], y0 = qv[2 * g], y1 = qv[2 * g + 1];
        const uint32_t o = (x0.x ^ y0.x) | (x0.y ^ y0.y) | (x0.z ^ y0.z) | (x0.w ^ y0.w) | (x1.x ^ y1.x) |
                           (x1.y ^ y1.y) | (x1.z ^ y1.z) | (x1.w ^ y1.w);
        acc += 32 - __popc(o);
      }
      if (MODE == 0) {
        if (valid) atomicAdd(&shist[qi * kMaxBins + acc], 1);
      } else {
        const bool surv = valid && acc >= stau[qi];
        const unsigned mask = __ballot_sync(0xffffffffu, surv);
        if (mask) {
          const int leader = __ffs(mask) - 1;
          int base = 0;
          if (lane == leader) base = atomicAdd(&cnt[q0 + qi], __popc(mask));
          base = __shfl_sync(0xffffffffu, base, leader);
          if (surv) {
            const int at = base + __popc(mask & lt);
            if (at < cap) cand[(int64_t)(q0 + qi) * cap + at] = make_key(-(float)acc, (int)p);
          }
        }
      }
    }
  }
  if (MODE == 0) {
    __syncthreads();
    for (int i = tid; i < kFQB * bins; i += blockDim.x) {
      const int qi = i / bins, b = i - qi * bins;
      const int v = shist[qi * kMaxBins + b];
      if (v && q0 + qi < nq) atomicAdd(&hist[(int64_t)(q0 + qi) * bins + b], v);
    }
  }
}

// tau[q] = the match count at which the histogram's count from the top first reaches
// `rank` (0 -- keep everything -- when the sample holds fewer); one warp a query.
__global__ void hist_tau_kernel(const int* __restrict__ hist, int nq, int bins, int rank, int* __restrict__ tau) {
  const int lane = threadIdx.x & 31;
  const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (q >= nq) return;  // warp-uniform
  const int* h = hist + (int64_t)q * bins;
  // lane l owns bins top - l * per .. : chunks from the top
  const int per = (bins + 31) / 32;
  const int hi0 = bins - 1 - lane * per, lo0 = max(-1, hi0 - per);
  int own = 0;
  for (int b = hi0; b > lo0; --b) own += h[b];
  int incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const unsigned hit = __ballot_sync(0xffffffffu, incl >= rank);
  if (!hit) {
    if (lane == 0) tau[q] = 0;
    return;
  }
  const int L = __ffs(hit) - 1;
  if (lane == L) {
    int acc = incl - own, t = 0;
    for (int b = hi0; b > lo0; --b) {
      acc += h[b];
      if (acc >= rank) {
        t = b;
        break;
      }
    }
    tau[q] = t;
  }
}

template <int MODE>
void run_bytes_filter(int ng, const uint4* xst, int64_t n, const uint32_t* qsl, int nq, int NP, int tstride,
                      const int* tau, int* hist, int bins, int* cnt, uint64_t* cand, int cap, cudaStream_t s) {
  const int qblocks = ceil_div(nq, kFQB);
  const int splits = std::max(1, std::min(NP, ceil_div((int64_t)num_sms() * 4, qblocks)));
  const int per = ceil_div(NP, splits);
  dim3 grid(qblocks, ceil_div(NP, per));
#define LSHG_BF(NGV)                                                                                           \
  bytes_filter_kernel<MODE, NGV><<<grid, 256, 0, s>>>(xst, n, qsl, nq, NP, tstride, per, tau, hist, bins, cnt, \
                                                       cand, cap)
  switch (ng) {
    case 1: LSHG_BF(1); break;
    case 2: LSHG_BF(2); break;
    case 3: LSHG_BF(3); break;
    case 4: LSHG_BF(4); break;
    case 5: LSHG_BF(5); break;
    case 6: LSHG_BF(6); break;
    case 7: LSHG_BF(7); break;
    case 8: LSHG_BF(8); break;
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "byte filter scan: 1..8 groups of 32 samples");
  }
#undef LSHG_BF
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace

int byte_slice_words(int wp) { return (wp + 7) / 8 * 8; }

void launch_slice_bytes(const uint32_t* xs, int64_t n, int wp, int64_t rows, uint8_t pad, uint32_t* out,
                        cudaStream_t s) {
  const int groups = byte_slice_words(wp) / 8;
  const int64_t total = rows * groups * 8;
  if (total <= 0) return;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  slice_bytes_kernel<<<blocks, 256, 0, s>>>(xs, n, wp, groups, rows, pad, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

bool byte_filter_plan(int64_t n, int C, int* stride, int* rank, int* cap) {
  const int NT = ceil_div(n, kTile);
  for (int S : {16, 8, 4, 2}) {
    const double m = (double)C / S;
    const int r = (int)std::ceil(m + 4.0 * std::sqrt(m) + 8.0);
    if ((int64_t)ceil_div(NT, S) * kTile >= 4 * (int64_t)r && r < C) {
      *stride = S;
      *rank = r;
      int64_t c = 1024;
      while (c < 3 * (int64_t)r * S + 2048) c <<= 1;
      *cap = (int)std::min<int64_t>(16384, c);
      return *cap >= C;
    }
  }
  return false;
}

void launch_byte_filter_scan(const uint32_t* xsl_t, const uint32_t* xst, int64_t n, int wp, int sbytes,
                             const uint32_t* qs, int nq, int C, uint64_t* out, cudaStream_t s) {
  if (nq <= 0) return;
  int stride = 0, rank = 0, cap = 0;
  LSHG_REQUIRE(byte_filter_plan(n, C, &stride, &rank, &cap), "byte filter scan: base too small for C");
  const int wsl = byte_slice_words(wp), ng = wsl / 8;
  const int bins = std::min(kMaxBins, 4 * wp + 1);
  ProfScope _ps("scan_bytes_filter", s);
  DevBuf<uint32_t> qsl((size_t)nq * wsl, s);
  launch_slice_bytes(qs, nq, wp, nq, 0xFF, qsl.ptr, s);
  const int NT = ceil_div(n, kTile);
  DevBuf<int> hist((size_t)nq * bins, s);
  LSHG_CUDA(cudaMemsetAsync(hist.ptr, 0, hist.bytes(), s));
  const uint4* base = reinterpret_cast<const uint4*>(xsl_t);
  run_bytes_filter<0>(ng, base, n, qsl.ptr, nq, ceil_div(NT, stride), stride, nullptr, hist.ptr, bins, nullptr,
                      nullptr, 0, s);
  DevBuf<int> tau((size_t)nq, s);
  hist_tau_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(hist.ptr, nq, bins, rank, tau.ptr);
  count_launch();
  LSHG_CHECK_LAUNCH();
  DevBuf<int> cnt((size_t)nq, s);
  LSHG_CUDA(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes(), s));
  DevBuf<uint64_t> cand((size_t)nq * cap, s);
  run_bytes_filter<1>(ng, base, n, qsl.ptr, nq, NT, 1, tau.ptr, nullptr, bins, cnt.ptr, cand.ptr, cap, s);
  DevBuf<int> ovf((size_t)nq + 1, s);
  LSHG_CUDA(cudaMemsetAsync(ovf.ptr, 0, sizeof(int), s));
  // scores are match counts 0..4 wp: the integer select with "bits" = 4 wp
  tc::launch_int_select(cnt.ptr, cand.ptr, cap, (int)std::min<int64_t>(C, n), C, 4 * wp, nq, out, ovf.ptr, s);
  launch_scan_bits_listed(xst, n, wp, (sbytes + 3) / 4, sbytes, qs, nq, OP_BYTE_JACCARD, C, ovf.ptr, out, s);
}

}  // namespace lshg
