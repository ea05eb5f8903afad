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
#include "tc_filter.h"
#include "tc_ptx.cuh"

namespace lshg {

int launch_scan_bits_listed(const uint32_t* xst, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq,
                            int op, int C, const int* list, uint64_t* out, cudaStream_t s);

namespace {

constexpr int kTile = 128;   // points a tile
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
// The sliced base is tiled as the popcount scan's ([tile][chunk][128] 16-byte chunks, NG
// 32-sample groups = 2 NG chunks a point); a position p covers tile p * tstride.
//
// One CTA of 16 warps an SM serves 64 queries at a time.  Work is the flat sequence of
// (query block, position) items, query block major; each CTA takes an equal contiguous
// range, so it changes query block at most a few times and no CTA gets more than one
// tile above the average.  Tiles are staged in shared memory by 1-D bulk copies, STAGES
// ahead; the last warp to finish a tile issues the copy that refills its buffer, so warps
// never wait on one another between tiles.  A thread owns two points of a tile (p and
// p + 64) and 8 of the 64 queries: each query word it loads from shared memory (the same
// address across the warp) serves both points.  A tile is consumed in passes over at most
// 4 groups, so a thread holds 4 groups of its two points and 16 counts of unequal samples.
constexpr int kBQ = 64;          // queries a CTA
constexpr int kQT = 8;           // queries a thread
constexpr int kBThreads = 512;
constexpr int kBWarps = kBThreads / 32;
constexpr int kPassGroups = 4;

template <int MODE, int NG>
struct BFLayout {
  static constexpr int W = NG * 8;                           // sliced words a row
  static constexpr int TB = NG * 2 * kTile * 16;             // bytes a tile
  static constexpr int STAGES = MODE == 0 ? 3 : 4;
  static constexpr int Q_OFF = STAGES * TB;                  // query rows [kBQ][W]
  static constexpr int TAU_OFF = Q_OFF + kBQ * W * 4;
  static constexpr int H_OFF = TAU_OFF + kBQ * 4;            // MODE 0: histograms [kBQ][kMaxBins]
  static constexpr int BAR_OFF = H_OFF + (MODE == 0 ? kBQ * kMaxBins * 4 : 0);
  // full barriers [STAGES], then per stage the last item issued (int64) and the warps
  // done (int); the abort flag
  static constexpr int LAST_OFF = BAR_OFF + 8 * STAGES;
  static constexpr int CNT_OFF = LAST_OFF + 8 * STAGES;
  static constexpr int ABORT_OFF = CNT_OFF + 4 * STAGES;
  static constexpr int SMEM = ABORT_OFF + 16;
  static_assert(Q_OFF % 16 == 0 && BAR_OFF % 8 == 0 && LAST_OFF % 8 == 0 && CNT_OFF % 4 == 0, "alignment");
  static_assert(SMEM <= 232448, "shared memory per CTA");
};

template <int MODE, int NG>
__global__ void __launch_bounds__(kBThreads, 1)
    bytes_filter_kernel(const uint4* __restrict__ xst, int64_t n, const uint32_t* __restrict__ qsl, int nq, int NP,
                        int tstride, const int* __restrict__ tau, int* __restrict__ hist, int bins,
                        int* __restrict__ cnt, uint64_t* __restrict__ cand, int cap, int* __restrict__ err) {
  using LY = BFLayout<MODE, NG>;
  constexpr int W = LY::W, NCH = 2 * NG, ST = LY::STAGES;
  constexpr int NPASS = (NG + kPassGroups - 1) / kPassGroups;
  extern __shared__ __align__(128) uint8_t smem[];
  uint32_t* qsm = reinterpret_cast<uint32_t*>(smem + LY::Q_OFF);
  int* stau = reinterpret_cast<int*>(smem + LY::TAU_OFF);
  int* shist = reinterpret_cast<int*>(smem + LY::H_OFF);
  int* sdone = reinterpret_cast<int*>(smem + LY::CNT_OFF);
  int64_t* slast = reinterpret_cast<int64_t*>(smem + LY::LAST_OFF);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + LY::ABORT_OFF);
  const uint32_t bar0 = tc::smem_u32(smem + LY::BAR_OFF);
  const int tid = threadIdx.x, lane = tid & 31, pl = tid & 63, qo = (tid >> 6) * kQT;
  const unsigned lt = (1u << lane) - 1u;

  const int64_t total = (int64_t)((nq + kBQ - 1) / kBQ) * NP;
  const int64_t beg = total * blockIdx.x / gridDim.x, end = total * (blockIdx.x + 1) / gridDim.x;
  // item `it` -> its tile copied into stage (it - beg) % ST
  auto issue = [&](int64_t it) {
    const int qb = (int)(it / NP), pos = (int)(it - (int64_t)qb * NP);
    const int st = (int)((it - beg) % ST);
    const uint32_t bar = bar0 + 8 * st;
    slast[st] = it;
    tc::mbar_expect_tx(bar, LY::TB);
    tc::bulk_load(tc::smem_u32(smem + st * LY::TB), xst + (int64_t)pos * tstride * NCH * kTile, LY::TB, bar);
  };
  if (tid == 0) {
    for (int s = 0; s < ST; ++s) {
      tc::mbar_init(bar0 + 8 * s, 1);
      sdone[s] = 0;
      slast[s] = -1;
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int64_t it = beg; it < end && it < beg + ST; ++it) issue(it);
  }
  __syncthreads();

  bool live = true;  // false once a wait gave up: the rest of the range is walked without work
  int cur = -1;
  for (int64_t it = beg; it < end; ++it) {
    const int qb = (int)(it / NP), pos = (int)(it - (int64_t)qb * NP);
    const int q0 = qb * kBQ;
    if (qb != cur) {  // all warps meet here: reload the block's queries
      __syncthreads();
      if (MODE == 0 && cur >= 0) {
        for (int i = tid; i < kBQ * bins; i += kBThreads) {
          const int qi = i / bins, b = i - qi * bins;
          const int v = shist[qi * kMaxBins + b];
          if (v && cur * kBQ + qi < nq) atomicAdd(&hist[(int64_t)(cur * kBQ + qi) * bins + b], v);
        }
        __syncthreads();
      }
      for (int i = tid; i < kBQ * W; i += kBThreads) {
        const int qi = i / W;
        qsm[i] = q0 + qi < nq ? qsl[(int64_t)(q0 + qi) * W + (i - qi * W)] : 0u;
      }
      if (MODE == 1)
        for (int i = tid; i < kBQ; i += kBThreads) stau[i] = q0 + i < nq ? tau[q0 + i] : INT_MAX;
      if (MODE == 0)
        for (int i = tid; i < kBQ * kMaxBins; i += kBThreads) shist[i] = 0;
      cur = qb;
      __syncthreads();
    }
    if (!live) continue;
    const int st = (int)((it - beg) % ST);
    if (!tc::mbar_wait(bar0 + 8 * st, (uint32_t)(((it - beg) / ST) & 1), abort_flag)) {
      live = false;
      continue;
    }
    const uint4* xt = reinterpret_cast<const uint4*>(smem + st * LY::TB);
    const int64_t p0 = (int64_t)pos * tstride * kTile + pl;
    int uneq[2][kQT];
#pragma unroll
    for (int a = 0; a < kQT; ++a) uneq[0][a] = uneq[1][a] = 0;
#pragma unroll
    for (int ps = 0; ps < NPASS; ++ps) {
      constexpr int GP = kPassGroups;
      uint4 xr[2][2 * GP];
#pragma unroll
      for (int j = 0; j < 2 * GP; ++j)
        if (ps * GP * 2 + j < NCH) {
          xr[0][j] = xt[(ps * GP * 2 + j) * kTile + pl];
          xr[1][j] = xt[(ps * GP * 2 + j) * kTile + pl + 64];
        }
#pragma unroll
      for (int a = 0; a < kQT; ++a) {
        const uint4* qv = reinterpret_cast<const uint4*>(qsm + (qo + a) * W) + ps * GP * 2;
#pragma unroll
        for (int g = 0; g < GP; g += 2) {  // two groups a step: one three-way add of their counts
          if (ps * GP + g < NG) {
            const bool two = ps * GP + g + 1 < NG;
            const uint4 y0 = qv[2 * g], y1 = qv[2 * g + 1];
            const uint4 y2 = two ? qv[2 * g + 2] : y0, y3 = two ? qv[2 * g + 3] : y1;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint4 x0 = xr[h][2 * g], x1 = xr[h][2 * g + 1];
              const uint32_t o = (x0.x ^ y0.x) | (x0.y ^ y0.y) | (x0.z ^ y0.z) | (x0.w ^ y0.w) | (x1.x ^ y1.x) |
                                 (x1.y ^ y1.y) | (x1.z ^ y1.z) | (x1.w ^ y1.w);
              uint32_t o2 = 0;
              if (two) {
                const uint4 x2 = xr[h][2 * g + 2], x3 = xr[h][2 * g + 3];
                o2 = (x2.x ^ y2.x) | (x2.y ^ y2.y) | (x2.z ^ y2.z) | (x2.w ^ y2.w) | (x3.x ^ y3.x) | (x3.y ^ y3.y) |
                     (x3.z ^ y3.z) | (x3.w ^ y3.w);
              }
              uneq[h][a] += __popc(o) + __popc(o2);
            }
          }
        }
      }
    }
    // every load of the tile has been consumed: the last warp refills the buffer
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      if (atomicAdd(&sdone[st], 1) == kBWarps - 1) {
        sdone[st] = 0;
        if (it + ST < end) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue(it + ST);
        }
      }
    }
    if (MODE == 0) {
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int a = 0; a < kQT; ++a)
          if (p0 + 64 * h < n && q0 + qo + a < nq) atomicAdd(&shist[(qo + a) * kMaxBins + 32 * NG - uneq[h][a]], 1);
    } else {
      // survivors: one ballot a point slot and query, one global count reservation a
      // query for both slots, all of a tile's reservations in flight before the first
      // result is used
      unsigned mk[2][kQT];
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int a = 0; a < kQT; ++a)
          mk[h][a] = __ballot_sync(0xffffffffu, p0 + 64 * h < n && 32 * NG - uneq[h][a] >= stau[qo + a]);
      int bs[kQT];
#pragma unroll
      for (int a = 0; a < kQT; ++a) {
        const int tot = __popc(mk[0][a]) + __popc(mk[1][a]);
        bs[a] = 0;
        if (tot && lane == 0) bs[a] = atomicAdd(&cnt[q0 + qo + a], tot);
      }
#pragma unroll
      for (int a = 0; a < kQT; ++a) {
        if (mk[0][a] | mk[1][a]) {  // the same for every lane
          int base = __shfl_sync(0xffffffffu, bs[a], 0);
          uint64_t* row = cand + (int64_t)(q0 + qo + a) * cap;
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if ((mk[h][a] >> lane) & 1u) {
              const int at = base + __popc(mk[h][a] & lt);
              if (at < cap) row[at] = make_key(-(float)(32 * NG - uneq[h][a]), (int)(p0 + 64 * h));
            }
            base += __popc(mk[h][a]);
          }
        }
      }
    }
  }
  __syncthreads();
  if (*abort_flag) {  // a tile never arrived: report, and let the copies in flight land first
    if (tid == 0) {
      for (int s = 0; s < ST; ++s)
        if (slast[s] >= 0)
          tc::mbar_wait(bar0 + 8 * s, (uint32_t)(((slast[s] - beg) / ST) & 1), abort_flag, true);
      atomicExch(err, 2);
    }
    return;
  }
  if (MODE == 0 && cur >= 0) {
    for (int i = tid; i < kBQ * bins; i += kBThreads) {
      const int qi = i / bins, b = i - qi * bins;
      const int v = shist[qi * kMaxBins + b];
      if (v && cur * kBQ + qi < nq) atomicAdd(&hist[(int64_t)(cur * kBQ + qi) * bins + b], v);
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

template <int MODE, int NG>
void run_bytes_filter_ng(const uint4* xst, int64_t n, const uint32_t* qsl, int nq, int NP, int tstride,
                         const int* tau, int* hist, int bins, int* cnt, uint64_t* cand, int cap, int* err,
                         cudaStream_t s) {
  constexpr int smem = BFLayout<MODE, NG>::SMEM;
  auto kern = bytes_filter_kernel<MODE, NG>;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int per_sm = 0;
  LSHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBThreads, smem));
  const int64_t total = (int64_t)ceil_div(nq, kBQ) * NP;
  const int grid = (int)std::min<int64_t>(total, (int64_t)num_sms() * std::max(1, per_sm));
  kern<<<grid, kBThreads, smem, s>>>(xst, n, qsl, nq, NP, tstride, tau, hist, bins, cnt, cand, cap, err);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

template <int MODE>
void run_bytes_filter(int ng, const uint4* xst, int64_t n, const uint32_t* qsl, int nq, int NP, int tstride,
                      const int* tau, int* hist, int bins, int* cnt, uint64_t* cand, int cap, int* err,
                      cudaStream_t s) {
  if (NP <= 0) return;
#define LSHG_BF(NGV) \
  run_bytes_filter_ng<MODE, NGV>(xst, n, qsl, nq, NP, tstride, tau, hist, bins, cnt, cand, cap, err, s)
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
                             const uint32_t* qs, int nq, int C, uint64_t* out, int* err, cudaStream_t s) {
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
                      nullptr, 0, err, s);
  DevBuf<int> tau((size_t)nq, s);
  hist_tau_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(hist.ptr, nq, bins, rank, tau.ptr);
  count_launch();
  LSHG_CHECK_LAUNCH();
  DevBuf<int> cnt((size_t)nq, s);
  LSHG_CUDA(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes(), s));
  DevBuf<uint64_t> cand((size_t)nq * cap, s);
  run_bytes_filter<1>(ng, base, n, qsl.ptr, nq, NT, 1, tau.ptr, nullptr, bins, cnt.ptr, cand.ptr, cap, err, s);
  DevBuf<int> ovf((size_t)nq + 1, s);
  LSHG_CUDA(cudaMemsetAsync(ovf.ptr, 0, sizeof(int), s));
  // scores are match counts 0..4 wp: the integer select with "bits" = 4 wp
  tc::launch_int_select(cnt.ptr, cand.ptr, cap, (int)std::min<int64_t>(C, n), C, 4 * wp, nq, out, ovf.ptr, s);
  launch_scan_bits_listed(xst, n, wp, (sbytes + 3) / 4, sbytes, qs, nq, OP_BYTE_JACCARD, C, ovf.ptr, out, s);
}

}  // namespace lshg
