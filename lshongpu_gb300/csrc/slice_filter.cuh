// Threshold filter over bit-sliced sample codes: the scan kernel shared by the byte
// weighted-MinHash scan (8 planes: one byte a sample, scan_filter.cu) and the consistent
// weighted sampling scan (16 planes: one (index, t) code a sample, cws.cu).
//
// Layout: for every group of 32 samples a row holds PL words, word b carrying bit b of
// the 32 samples' codes; two samples are equal when all PL of their bits are, so the
// unequal samples of a (query, point) pair in a group are the set bits of
// OR_b (x_b XOR q_b): PL three-input logic operations and one popcount for 32 samples.
// The base is tiled [tile][chunk][128] in 16-byte chunks (NG groups = NG * PL / 4 chunks a
// point), the queries are plain rows of NG * PL words.
//
// MODE 0: histogram of match counts over the sampled positions (hist [nq][bins]);
// MODE 1: keep every point with at least tau[q] matches (keys make_key(-matches, id)).
// A position p covers tile p * tstride.
//
// One CTA of 16 warps an SM serves 64 queries at a time.  Each CTA walks its own sequence
// of (query block, position) items (make_walk / locate below), within one chunk or one
// tile of every other CTA's length.  Tiles are staged in shared memory by 1-D bulk copies, STAGES
// ahead; the last warp to finish a tile issues the copy that refills its buffer, so warps
// never wait on one another between tiles.  A thread owns two points of a tile (p and
// p + 64) and 8 of the 64 queries: each query word it loads from shared memory (the same
// address across the warp) serves both points.  A tile is consumed in passes over 32 / PL
// groups, so a thread holds 64 words of its two points and 16 counts of unequal samples.
#pragma once

#include <algorithm>

#include "common.cuh"
#include "launch_count.h"
#include "tc_filter.h"
#include "tc_ptx.cuh"

namespace lshg {
namespace sf {

constexpr int kTile = 128;     // points a tile
constexpr int kMaxBins = 257;  // match counts 0..256
constexpr int kBQ = 64;        // queries a CTA
constexpr int kQT = 8;         // queries a thread
constexpr int kBThreads = 512;
constexpr int kBWarps = kBThreads / 32;
constexpr int kSmemMax = 232448;  // shared memory a CTA may use
constexpr int64_t kL2Half = 64ll << 20;  // bases above this are walked chunk-major

template <int MODE, int NG, int PL>
struct Layout {
  static constexpr int W = NG * PL;                          // sliced words a row
  static constexpr int TB = W * kTile * 4;                   // bytes a tile
  static constexpr int QBYTES = kBQ * W * 4;                 // query rows [kBQ][W]
  static constexpr int HBYTES = MODE == 0 ? kBQ * kMaxBins * 4 : 0;
  static constexpr int FIXED = QBYTES + kBQ * 4 + HBYTES + 512;
  static constexpr int STAGES_FIT = (kSmemMax - FIXED) / TB;
  static constexpr int STAGES = STAGES_FIT > 4 ? 4 : STAGES_FIT;
  static constexpr int Q_OFF = STAGES * TB;
  static constexpr int TAU_OFF = Q_OFF + QBYTES;
  static constexpr int H_OFF = TAU_OFF + kBQ * 4;            // MODE 0: histograms [kBQ][kMaxBins]
  static constexpr int BAR_OFF = H_OFF + HBYTES;
  // full barriers [STAGES], then per stage the last item issued (int64) and the warps
  // done (int); the abort flag
  static constexpr int LAST_OFF = BAR_OFF + 8 * STAGES;
  static constexpr int CNT_OFF = LAST_OFF + 8 * STAGES;
  static constexpr int ABORT_OFF = CNT_OFF + 4 * STAGES;
  static constexpr int SMEM = ABORT_OFF + 16;
  static_assert(STAGES >= 2, "two tile stages must fit");
  static_assert(Q_OFF % 16 == 0 && BAR_OFF % 8 == 0 && LAST_OFF % 8 == 0 && CNT_OFF % 4 == 0, "alignment");
  static_assert(SMEM <= kSmemMax, "shared memory per CTA");
};

// A base larger than half the L2 is walked in chunks of `chunk` positions (8..64: at least
// ~24 units a CTA, so that the last units leave little imbalance).  A unit is (chunk, query
// block),
// numbered chunk-major, and CTA b takes units b, b + G, b + 2G, ...: the G CTAs then work
// on the same chunk at a time, so a base tile comes from DRAM about once a batch and from
// L2 for the other query blocks (a CTA walking one query block through the whole base,
// about as large as L2, had read it from DRAM about once a query block).  Otherwise
// (chunk = 0: the prepass, which samples a small part of the base, and bases that stay in
// L2) each CTA takes an equal contiguous range of (query block, position) items, query
// block major: fewer query-block switches (and histogram flushes).
// This CTA's items, local index li in [0, len).
struct Walk {
  int64_t beg = 0, len = 0;  // MODE 0: global items [beg, beg + len)
  int nf = 0, wl = 0;        // MODE 1: units in full chunks, width of the last chunk
};

__device__ __forceinline__ Walk make_walk(int NP, int QB, int chunk) {
  Walk w;
  const int G = gridDim.x, b = blockIdx.x;
  if (chunk == 0) {
    const int64_t total = (int64_t)QB * NP;
    w.beg = total * b / G;
    w.len = total * (b + 1) / G - w.beg;
    return w;
  }
  const int nch = (NP + chunk - 1) / chunk;
  w.wl = NP - (nch - 1) * chunk;
  const int64_t U = (int64_t)nch * QB, Uf = (int64_t)(nch - 1) * QB;
  const int64_t mine = U > b ? (U - b + G - 1) / G : 0;
  w.nf = (int)(Uf > b ? (Uf - b + G - 1) / G : 0);
  w.len = (int64_t)w.nf * chunk + (mine - w.nf) * w.wl;
  return w;
}

// (query block, position) of local item li.
__device__ __forceinline__ void locate(const Walk& w, int64_t li, int NP, int QB, int chunk, int& qb, int& pos) {
  if (chunk == 0) {
    const int64_t it = w.beg + li;
    qb = (int)(it / NP);
    pos = (int)(it - (int64_t)qb * NP);
    return;
  }
  int64_t k, j;
  if (li < (int64_t)w.nf * chunk) {
    k = li / chunk;
    j = li - k * chunk;
  } else {
    const int64_t l2 = li - (int64_t)w.nf * chunk;
    k = w.nf + l2 / w.wl;
    j = l2 - (k - w.nf) * w.wl;
  }
  const int64_t u = blockIdx.x + k * gridDim.x;
  const int c = (int)(u / QB);
  qb = (int)(u - (int64_t)c * QB);
  pos = c * chunk + (int)j;
}

// The same sequence stepped one item at a time (no division but one a unit), for the
// per-item loop every thread runs; locate() serves the copies issued ahead.
struct Cursor {
  int qb = 0, pos = 0;
  int j = 0, width = 0;  // chunk walk: position within the unit, the unit's width
  int64_t u = 0;         // chunk walk: unit number
  __device__ __forceinline__ void unit(int NP, int QB, int chunk) {
    const int c = (int)(u / QB);
    qb = (int)(u - (int64_t)c * QB);
    width = min(chunk, NP - c * chunk);
    pos = c * chunk;
    j = 0;
  }
  __device__ __forceinline__ void start(const Walk& w, int NP, int QB, int chunk) {
    if (chunk == 0) {
      qb = (int)(w.beg / NP);
      pos = (int)(w.beg - (int64_t)qb * NP);
      return;
    }
    u = blockIdx.x;
    unit(NP, QB, chunk);
  }
  __device__ __forceinline__ void next(int NP, int QB, int chunk) {
    if (chunk == 0) {
      if (++pos == NP) {
        pos = 0;
        ++qb;
      }
      return;
    }
    ++pos;
    if (++j == width) {
      u += gridDim.x;
      unit(NP, QB, chunk);
    }
  }
};

template <int MODE, int NG, int PL>
__global__ void __launch_bounds__(kBThreads, 1)
    sliced_filter_kernel(const uint4* __restrict__ xst, int64_t n, const uint32_t* __restrict__ qsl, int nq, int NP,
                         int tstride, int chunk, const int* __restrict__ tau, int* __restrict__ hist, int bins,
                         int* __restrict__ cnt, uint64_t* __restrict__ cand, int cap, int* __restrict__ err) {
  using LY = Layout<MODE, NG, PL>;
  constexpr int W = LY::W, NCH = W / 4, ST = LY::STAGES;
  constexpr int CPG = PL / 4;                 // chunks a group
  constexpr int GP = 32 / PL;                 // groups a pass (64 words of two points)
  constexpr int NPASS = (NG + GP - 1) / GP;
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

  const int QB = (nq + kBQ - 1) / kBQ;
  const Walk wk = make_walk(NP, QB, chunk);
  const int64_t beg = 0, end = wk.len;  // local item indices
  // item `it` -> its tile copied into stage (it - beg) % ST
  auto issue = [&](int64_t it) {
    int qb, pos;
    locate(wk, it, NP, QB, chunk, qb, pos);
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
  Cursor cs;
  cs.start(wk, NP, QB, chunk);
  for (int64_t it = beg; it < end; ++it, cs.next(NP, QB, chunk)) {
    const int qb = cs.qb, pos = cs.pos;
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
      constexpr int PC = GP * CPG;  // chunks a pass
      uint4 xr[2][PC];
#pragma unroll
      for (int j = 0; j < PC; ++j)
        if (ps * PC + j < NCH) {
          xr[0][j] = xt[(ps * PC + j) * kTile + pl];
          xr[1][j] = xt[(ps * PC + j) * kTile + pl + 64];
        }
#pragma unroll
      for (int a = 0; a < kQT; ++a) {
        const uint4* qv = reinterpret_cast<const uint4*>(qsm + (qo + a) * W) + ps * PC;
#pragma unroll
        for (int g = 0; g < GP; g += 2) {  // two groups a step: one three-way add of their counts
          if (ps * GP + g < NG) {
            const bool two = GP > 1 && ps * GP + g + 1 < NG;
            uint4 y[2 * CPG];
#pragma unroll
            for (int c = 0; c < CPG; ++c) {
              y[c] = qv[g * CPG + c];
              y[CPG + c] = two ? qv[(g + 1) * CPG + c] : y[c];
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              uint32_t o = 0, o2 = 0;
#pragma unroll
              for (int c = 0; c < CPG; ++c) {
                const uint4 x = xr[h][g * CPG + c];
                o |= (x.x ^ y[c].x) | (x.y ^ y[c].y) | (x.z ^ y[c].z) | (x.w ^ y[c].w);
              }
              if (two) {
#pragma unroll
                for (int c = 0; c < CPG; ++c) {
                  const uint4 x = xr[h][(g + 1) * CPG + c];
                  o2 |= (x.x ^ y[CPG + c].x) | (x.y ^ y[CPG + c].y) | (x.z ^ y[CPG + c].z) | (x.w ^ y[CPG + c].w);
                }
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

template <int MODE, int NG, int PL>
void run_ng(const uint4* xst, int64_t n, const uint32_t* qsl, int nq, int NP, int tstride, const int* tau, int* hist,
            int bins, int* cnt, uint64_t* cand, int cap, int* err, cudaStream_t s) {
  constexpr int smem = Layout<MODE, NG, PL>::SMEM;
  auto kern = sliced_filter_kernel<MODE, NG, PL>;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int per_sm = 0;
  LSHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBThreads, smem));
  const int64_t slots = (int64_t)num_sms() * std::max(1, per_sm);
  const int64_t items = (int64_t)ceil_div(nq, kBQ) * NP;
  const bool big = MODE == 1 && (int64_t)NP * Layout<MODE, NG, PL>::TB > kL2Half;
  const int chunk = big ? (int)std::max<int64_t>(8, std::min<int64_t>(64, items / (slots * 24))) : 0;
  const int64_t total = chunk ? (int64_t)ceil_div(nq, kBQ) * ceil_div(NP, chunk) : items;  // units or items
  const int grid = (int)std::min<int64_t>(total, slots);
  kern<<<grid, kBThreads, smem, s>>>(xst, n, qsl, nq, NP, tstride, chunk, tau, hist, bins, cnt, cand, cap, err);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

// One pass of the filter over groups ng (1..8) of PL-plane codes.
template <int MODE, int PL>
void run_pass(int ng, const uint4* xst, int64_t n, const uint32_t* qsl, int nq, int NP, int tstride, const int* tau,
              int* hist, int bins, int* cnt, uint64_t* cand, int cap, int* err, cudaStream_t s) {
  if (NP <= 0 || nq <= 0) return;
#define LSHG_SF(NGV) run_ng<MODE, NGV, PL>(xst, n, qsl, nq, NP, tstride, tau, hist, bins, cnt, cand, cap, err, s)
  switch (ng) {
    case 1: LSHG_SF(1); break;
    case 2: LSHG_SF(2); break;
    case 3: LSHG_SF(3); break;
    case 4: LSHG_SF(4); break;
    case 5: LSHG_SF(5); break;
    case 6: LSHG_SF(6); break;
    case 7: LSHG_SF(7); break;
    case 8: LSHG_SF(8); break;
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "sliced filter scan: 1..8 groups of 32 samples");
  }
#undef LSHG_SF
}

}  // namespace sf

// tau[q] = the match count at which the histogram's count from the top first reaches
// `rank` (scan_filter.cu).
void launch_hist_tau(const int* hist, int nq, int bins, int rank, int* tau, cudaStream_t s);

// Sampled plan of the filter for a base of n points and C candidates: stride of the
// prepass positions, rank of the threshold in the sample, survivor array capacity; false
// when the base is too small for a sampled threshold (scan_filter.cu).
bool byte_filter_plan(int64_t n, int C, int* stride, int* rank, int* cap);

// The whole threshold-filter selection over PL-plane sliced codes: prepass histograms,
// thresholds, filter, exact integer select into out [nq][C].  Queries whose survivors are
// fewer than C or overflow their array are listed in `list` (count, then query indices)
// for the caller's exact rescan.  `samples` is the number of real samples a row (match
// counts 0..samples).
template <int PL>
void sliced_filter_select(const uint32_t* base_t, int64_t n, int ng, int samples, const uint32_t* qsl, int nq, int C,
                          uint64_t* out, int* list, int* err, cudaStream_t s) {
  int stride = 0, rank = 0, cap = 0;
  LSHG_REQUIRE(byte_filter_plan(n, C, &stride, &rank, &cap), "sliced filter scan: base too small for C");
  LSHG_REQUIRE(samples >= 1 && samples < sf::kMaxBins && samples <= 32 * ng, "sliced filter scan: bad sample count");
  const int bins = samples + 1;
  const int NT = ceil_div(n, sf::kTile);
  const uint4* base = reinterpret_cast<const uint4*>(base_t);
  DevBuf<int> hist((size_t)nq * bins, s);
  LSHG_CUDA(cudaMemsetAsync(hist.ptr, 0, hist.bytes(), s));
  sf::run_pass<0, PL>(ng, base, n, qsl, nq, ceil_div(NT, stride), stride, nullptr, hist.ptr, bins, nullptr, nullptr,
                      0, err, s);
  DevBuf<int> tau((size_t)nq, s);
  launch_hist_tau(hist.ptr, nq, bins, rank, tau.ptr, s);
  DevBuf<int> cnt((size_t)nq, s);
  LSHG_CUDA(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes(), s));
  DevBuf<uint64_t> cand((size_t)nq * cap, s);
  sf::run_pass<1, PL>(ng, base, n, qsl, nq, NT, 1, tau.ptr, nullptr, bins, cnt.ptr, cand.ptr, cap, err, s);
  LSHG_CUDA(cudaMemsetAsync(list, 0, sizeof(int), s));
  // scores are match counts 0..samples: the integer select with "bits" = samples
  tc::launch_int_select(cnt.ptr, cand.ptr, cap, (int)std::min<int64_t>(C, n), C, samples, nq, out, list, s);
}

}  // namespace lshg
