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
//    at least tau matches.  64 queries share a CTA, so the base streams Q/64 times.
// The survivors then go through the tensor-core sketch scan's integer select (the match
// count is the score) and queries with fewer than C survivors, or more than their array
// holds, are rescanned exactly by the per-query scan on the device; the candidate set is
// always the exact top-C by (distance, id).
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "profile.h"
#include "slice_filter.cuh"

namespace lshg {

int launch_scan_bits_listed(const uint32_t* xst, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq,
                            int op, int C, const int* list, uint64_t* out, cudaStream_t s);

namespace {

using sf::kTile;
using sf::kMaxBins;

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

void launch_hist_tau(const int* hist, int nq, int bins, int rank, int* tau, cudaStream_t s) {
  if (nq <= 0) return;
  hist_tau_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(hist, nq, bins, rank, tau);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_byte_filter_scan(const uint32_t* xsl_t, const uint32_t* xst, int64_t n, int wp, int sbytes,
                             const uint32_t* qs, int nq, int C, uint64_t* out, int* err, cudaStream_t s) {
  if (nq <= 0) return;
  const int wsl = byte_slice_words(wp), ng = wsl / 8;
  ProfScope _ps("scan_bytes_filter", s);
  DevBuf<uint32_t> qsl((size_t)nq * wsl, s);
  launch_slice_bytes(qs, nq, wp, nq, 0xFF, qsl.ptr, s);
  DevBuf<int> list((size_t)nq + 1, s);
  // match counts 0..4 wp (the padding bytes of a packed row never match)
  sliced_filter_select<8>(xsl_t, n, ng, 4 * wp, qsl.ptr, nq, C, out, list.ptr, err, s);
  launch_scan_bits_listed(xst, n, wp, (sbytes + 3) / 4, sbytes, qs, nq, OP_BYTE_JACCARD, C, list.ptr, out, s);
}

}  // namespace lshg
