// Threshold-filter tensor-core scan: the kernels behind implementation 8's main path.
//
// Selecting the top-CT cosine scores of every query out of a Q x N BF16 GEMM is done in
// two GEMM passes that share one persistent tcgen05 pipeline (tc_filter_kernel):
//
//   pass 0 (MODE_GROUPMAX) runs on a strided subsample of the base tiles (every S-th) and
//     writes, per query row, the maximum score of every GW-column group of every sampled
//     tile.  Each group maximum is the score of a real base point, so the CT-th largest
//     of them, tau[q] (tau_select_kernel), is a lower bound of the query's true CT-th best
//     score: every point of the exact top-CT has score >= tau[q].
//   pass 1 (MODE_FILTER) runs on the whole base.  The epilogue compares each score with
//     its row's tau; the (rare) survivors are staged per row in shared memory and moved
//     to the query's candidate array in global memory with one atomicAdd a batch (at the
//     end of each work unit, or when the 8-entry staging is full).  There is no per-row
//     selection state on chip, so the common case is a 64-wide maximum and a warp vote.
//
// cand_select_kernel then sorts each query's survivors and keeps the first CT keys
// (score descending, ties by lower id) -- exactly the top-CT by tensor-core score.  A query
// with more survivors than the candidate array holds (possible only with massive ties,
// e.g. duplicated points or a zero query) is listed for the exact per-row list kernel in
// tc_scan.cu, which runs on the device-side list without a host round trip.
//
// Work decomposition of tc_filter_kernel: a unit is (query tile, chunk of CH consecutive
// base positions); units are numbered chunk-major and dealt round-robin to one CTA per
// SM.  At any moment the CTAs therefore work on the same one or two chunks for different
// query tiles, so each base tile is read from HBM about once and served from L2 to the
// other query tiles; the query tile of a unit is double-buffered in shared memory.
//
// Tiles are 128 queries x 256 base points (tcgen05.mma M = 128, N = 256).  Warp roles (640
// threads): warp 0 TMA producer, warp 1 MMA issuer (one elected thread), warp 2 TMEM
// allocator (2 accumulators x 256 columns = 512), warp 3 idle, warps 4-19 the epilogue:
// warpgroup g (warps 4+4g .. 7+4g) reads TMEM columns [64g, 64g+64) of every accumulator,
// thread (warp & 3) * 32 + lane owns query row = TMEM lane.  Every mbarrier
// wait is bounded; a CTA that times out raises the error flag, drains its own copies and
// MMAs, frees TMEM and returns.
#include "index.h"
#include "launch_count.h"
#include "profile.h"
#include "select.cuh"
#include "tc_filter.h"
#include "tc_ptx.cuh"

namespace lshg {
namespace tc {

namespace {

constexpr int F_THREADS = 640;
constexpr int TN = FILTER_TN;                   // base points a tile = UMMA N
constexpr int B_HALF = TN * KHALF * 2;          // 32 KB: one 64-column half of a BF16 base tile
constexpr int F_NACC = 2;                       // TMEM accumulators of TN columns
constexpr int F_TMEM_COLS = F_NACC * TN;        // 512 = all of TMEM (one CTA per SM)
constexpr int F_EPI_WARPS = 16;  // four warpgroups, one 64-column piece each

constexpr int F_SBUF = 8;  // staged survivors a row and warpgroup (flushed with one atomic)
constexpr int kTauRegs = 80;  // group maxima a lane holds in the register threshold select

// Shared-memory layout by operand format.  BF16: a tile row is two 128-byte swizzle rows
// (64 columns each); E4M3: one (all 128 columns), so tiles are half the size and the
// base ring has twice the stages.
template <bool F8>
struct FLayout {
  static constexpr int A_BYTES = F8 ? BM * 128 : TILE_BYTES;  // query tile: 16 or 32 KB
  static constexpr int B_BYTES = F8 ? TN * 128 : 2 * B_HALF;  // base tile: 32 or 64 KB
  static constexpr int STAGES = F8 ? 4 : 2;
  static constexpr int A_OFF = 0;                             // two query tiles
  static constexpr int B_OFF = 2 * A_BYTES;                   // STAGES base tiles
  static constexpr int S_OFF = B_OFF + STAGES * B_BYTES;      // survivor staging: scores then ids, [4][F_SBUF][BM]
  static constexpr int BAR_OFF = S_OFF + 4 * F_SBUF * BM * 8;
  static constexpr int SMEM = BAR_OFF + 256 + 1024;           // + barriers + 1 KB alignment slack
  static_assert(SMEM <= 232448, "shared memory per CTA");
  static_assert(8 * (4 * STAGES + 5 + 2 * F_NACC) + 8 <= 256, "barrier area");
};

struct FilterArgs {
  int nq;
  int64_t n;
  int QT;        // query tiles
  int NP;        // base positions scanned (tiles NP of them, base tile = p * dstride)
  int dstride;
  int CH;        // positions per unit
  int NCH;       // chunks = ceil(NP / CH)
  float* gmax;   // MODE_GROUPMAX: [nq][M] group maxima
  int M;
  const float* tau;  // MODE_FILTER: per-query threshold (nullptr = keep everything)
  int* cnt;          // survivors per query
  uint64_t* cand;    // [nq][cap] survivor keys
  int cap;
  int ksteps;    // MMA K steps covering the data dimension (K = 16 BF16 or 32 E4M3 a step)
  int hi_cols;   // columns loaded of the second 64-column half of a base tile
  int* err;
};

// Move a row's staged survivors (score, id; stride BM in shared memory) to the query's
// candidate array: one atomicAdd reserves the slots.
__device__ __forceinline__ void flush_staged(int* cnt, uint64_t* dst, int cap, const float* ssc, const int* sid,
                                          int& scnt) {
  if (scnt > 0) {
    const int base = atomicAdd(cnt, scnt);
    for (int e = 0; e < scnt; ++e)
      if (base + e < cap) dst[base + e] = make_key(-ssc[e * BM], sid[e * BM]);
    scnt = 0;
  }
}

// F8: E4M3 operands (kind::f8f6f4); mapBhi is unused.
template <int MODE, int GW, bool F8>
__global__ void __launch_bounds__(F_THREADS, 1)
    tc_filter_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                     const __grid_constant__ CUtensorMap mapBhi, const FilterArgs a) {
  using LY = FLayout<F8>;
  constexpr int F_STAGES = LY::STAGES;
  constexpr int F_A_OFF = LY::A_OFF, F_B_OFF = LY::B_OFF, F_S_OFF = LY::S_OFF, F_BAR_OFF = LY::BAR_OFF;
  constexpr int A_BYTES = LY::A_BYTES, B_TILE = LY::B_BYTES;
  static_assert(MODE == MODE_GROUPMAX || GW == 64, "the filter reads whole 64-column pieces");
  static_assert(GW == 64 || GW == 8, "group width");
  const int U = a.NCH * a.QT;
  if ((int)blockIdx.x >= U) return;  // no unit for this CTA: leave before any barrier or TMEM use

  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t s0 = smem_u32(sm);
  const uint32_t bar0 = s0 + F_BAR_OFF;
  auto FULL = [&](int s) { return bar0 + 8u * s; };
  auto EMPTY = [&](int s) { return bar0 + 8u * (F_STAGES + s); };
  auto A_FULL = [&](int s) { return bar0 + 8u * (2 * F_STAGES + s); };
  auto A_EMPTY = [&](int s) { return bar0 + 8u * (2 * F_STAGES + 2 + s); };
  auto ACC_FULL = [&](int b) { return bar0 + 8u * (2 * F_STAGES + 4 + b); };
  auto ACC_EMPTY = [&](int b) { return bar0 + 8u * (2 * F_STAGES + 4 + F_NACC + b); };
  const uint32_t DONE = bar0 + 8u * (2 * F_STAGES + 4 + 2 * F_NACC);
  // Prepass (BF16): the second 64-column half of a base stage has barriers of its own
  // (FULL / EMPTY cover the first), so the first half is refilled once its four K steps
  // are done.  The prepass reads every S-th tile and its epilogue is light, so it waits on
  // the copies: split, it ran 16% faster at 1.2M x 100.  The filter pass ran 6% slower
  // split and keeps one pair of barriers a stage.
  constexpr bool SPLIT = !F8 && MODE == MODE_GROUPMAX;
  auto FULL_HI = [&](int s) { return bar0 + 8u * (2 * F_STAGES + 5 + 2 * F_NACC + s); };
  auto EMPTY_HI = [&](int s) { return bar0 + 8u * (3 * F_STAGES + 5 + 2 * F_NACC + s); };
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + F_BAR_OFF + 8 * (4 * F_STAGES + 5 + 2 * F_NACC));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < F_STAGES; ++s) {
      mbar_init(FULL(s), 1);
      mbar_init(EMPTY(s), 1);
      mbar_init(FULL_HI(s), 1);
      mbar_init(EMPTY_HI(s), 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(A_FULL(s), 1);
      mbar_init(A_EMPTY(s), 1);
    }
    for (int b = 0; b < F_NACC; ++b) {
      mbar_init(ACC_FULL(b), 1);
      mbar_init(ACC_EMPTY(b), F_EPI_WARPS);
    }
    mbar_init(DONE, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) tmem_alloc(smem_u32(tmem_slot), F_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0, ua = 0;
      bool ok = true, last_hi = true;  // last_hi: the last tile's second half was issued
      for (int u = blockIdx.x; u < U && ok; u += gridDim.x, ++ua) {
        const int qt = u % a.QT, c = u / a.QT;
        const int p0 = c * a.CH, p1 = min(a.NP, p0 + a.CH);
        const int ab = ua & 1;
        if (!mbar_wait(A_EMPTY(ab), ((ua >> 1) & 1) ^ 1, abort_flag)) break;
        mbar_expect_tx(A_FULL(ab), A_BYTES);
        tma_load_2d(s0 + F_A_OFF + ab * A_BYTES, &mapA, 0, qt * BM, A_FULL(ab));
        if (!F8) tma_load_2d(s0 + F_A_OFF + ab * A_BYTES + HALF_BYTES, &mapA, KHALF, qt * BM, A_FULL(ab));
        for (int p = p0; p < p1; ++p) {
          const int st = it % F_STAGES, rd = it / F_STAGES;
          if (!mbar_wait(EMPTY(st), (rd & 1) ^ 1, abort_flag)) { ok = false; break; }
          const uint32_t dst = s0 + F_B_OFF + st * B_TILE;
          const int row = p * a.dstride * TN;
          if (F8) {
            mbar_expect_tx(FULL(st), B_TILE);
            tma_load_2d(dst, &mapB, 0, row, FULL(st));
          } else if (!SPLIT) {
            mbar_expect_tx(FULL(st), B_HALF + TN * a.hi_cols * 2);
            tma_load_2d(dst, &mapB, 0, row, FULL(st));
            tma_load_2d(dst + B_HALF, &mapBhi, KHALF, row, FULL(st));
          } else {
            mbar_expect_tx(FULL(st), B_HALF);
            tma_load_2d(dst, &mapB, 0, row, FULL(st));
            if (!mbar_wait(EMPTY_HI(st), (rd & 1) ^ 1, abort_flag)) { ++it; last_hi = false; ok = false; break; }
            mbar_expect_tx(FULL_HI(st), TN * a.hi_cols * 2);
            tma_load_2d(dst + B_HALF, &mapBhi, KHALF, row, FULL_HI(st));
          }
          ++it;
        }
      }
      // drain: every issued copy has landed before the CTA may exit -- the last F_STAGES
      // tiles.  Split stages: the second halves too, except the last tile's when it was
      // never issued; then the second half of the tile before the window may still be in
      // flight (only its first half's MMAs had to finish before the last tile was issued)
      for (int j = max(0, it - F_STAGES - 1); j < it; ++j) {
        if (j >= it - F_STAGES) mbar_wait(FULL(j % F_STAGES), (j / F_STAGES) & 1, abort_flag, true);
        if (SPLIT && (last_hi ? j >= it - F_STAGES : j < it - 1))
          mbar_wait(FULL_HI(j % F_STAGES), (j / F_STAGES) & 1, abort_flag, true);
      }
      for (int j = max(0, ua - 2); j < ua; ++j) mbar_wait(A_FULL(j & 1), (j >> 1) & 1, abort_flag, true);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int it = 0, ua = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < U && ok; u += gridDim.x, ++ua) {
        const int c = u / a.QT;
        const int p0 = c * a.CH, p1 = min(a.NP, p0 + a.CH);
        const int ab = ua & 1;
        if (!mbar_wait(A_FULL(ab), (ua >> 1) & 1, abort_flag)) break;
        tc_fence_after();
        for (int p = p0; p < p1; ++p) {
          const int b = it % F_NACC, ub = it / F_NACC;
          if (!mbar_wait(ACC_EMPTY(b), (ub & 1) ^ 1, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const int st = it % F_STAGES, rd = it / F_STAGES;
          if (!mbar_wait(FULL(st), rd & 1, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t dt = tmem + (uint32_t)(b * TN), as = s0 + F_A_OFF + ab * A_BYTES;
          const uint32_t bs = s0 + F_B_OFF + st * B_TILE;
          if (F8) {
            umma_tile_e4m3<TN>(dt, as, bs, a.ksteps);
            umma_commit(EMPTY(st));
          } else if (!SPLIT) {
            umma_tile<TN>(dt, as, bs, a.ksteps);
            umma_commit(EMPTY(st));
          } else {
            umma_steps<TN>(dt, as, bs, 0, min(4, a.ksteps));
            umma_commit(EMPTY(st));
            if (!mbar_wait(FULL_HI(st), rd & 1, abort_flag)) { ok = false; break; }
            tc_fence_after();
            umma_steps<TN>(dt, as, bs, 4, a.ksteps);
            umma_commit(EMPTY_HI(st));
          }
          umma_commit(ACC_FULL(b));
          ++it;
        }
        umma_commit(A_EMPTY(ab));  // the query tile is free once this unit's MMAs complete
      }
      // drain: all issued MMAs complete before TMEM is released
      umma_commit(DONE);
      mbar_wait(DONE, 0, abort_flag, true);
    }
    __syncwarp();
  } else if (warp >= 4) {
    // ---------------- epilogue ----------------
    const int g = (warp - 4) >> 2;               // warpgroup: columns [64g, 64g+64) of every accumulator
    const int r = (warp & 3) * 32 + lane;        // query row within the tile = TMEM lane
    const uint32_t tbase = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(g * 64);
    // Survivors are staged per row in shared memory as (score, id) -- this thread's own
    // column of the warpgroup's [F_SBUF][BM] arrays, so no synchronisation is needed --
    // and reach the query's global array in batches: one atomicAdd a flush instead of
    // one a survivor, and the ordering keys are built only then.
    float* ssc = reinterpret_cast<float*>(sm + F_S_OFF) + (size_t)g * F_SBUF * BM + r;
    int* sid = reinterpret_cast<int*>(sm + F_S_OFF + 4 * F_SBUF * BM * 4) + (size_t)g * F_SBUF * BM + r;
    int scnt = 0;
    int it = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < U && ok; u += gridDim.x) {
      const int qt = u % a.QT, c = u / a.QT;
      const int p0 = c * a.CH, p1 = min(a.NP, p0 + a.CH);
      const int q = qt * BM + r;
      float tau = INFINITY;
      if (MODE == MODE_FILTER && q < a.nq) tau = a.tau ? a.tau[q] : -INFINITY;
      for (int p = p0; p < p1; ++p) {
        const int b = it % F_NACC, ub = it / F_NACC;
        if (!mbar_wait(ACC_FULL(b), ub & 1, abort_flag)) { ok = false; break; }
        tc_fence_after();
        uint32_t v[64];
        tmem_ld64(tbase + (uint32_t)(b * TN), v);
        tmem_wait_ld();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(ACC_EMPTY(b));  // scores are in registers: the MMA may reuse the buffer
        ++it;
        const int64_t cbase = (int64_t)p * a.dstride * TN + g * 64;  // base id of v[0]
        const int piece = 4 * p + g;  // index of this 64-column piece among the row's sampled pieces
        if (MODE == MODE_GROUPMAX) {
          if (cbase + 64 > a.n) {  // last base tile: padding rows are not points
#pragma unroll
            for (int j = 0; j < 64; ++j)
              if (cbase + j >= a.n) v[j] = __float_as_uint(-INFINITY);
          }
          if (q < a.nq) {
            if (GW == 64) {
              float m[8];
#pragma unroll
              for (int gg = 0; gg < 8; ++gg) m[gg] = max8(v, gg);
              a.gmax[(int64_t)q * a.M + piece] =
                  max3f(max3f(m[0], m[1], m[2]), max3f(m[3], m[4], m[5]), fmaxf(m[6], m[7]));
            } else {
              float4 lo, hi;
              lo.x = max8(v, 0); lo.y = max8(v, 1); lo.z = max8(v, 2); lo.w = max8(v, 3);
              hi.x = max8(v, 4); hi.y = max8(v, 5); hi.z = max8(v, 6); hi.w = max8(v, 7);
              float4* dst = reinterpret_cast<float4*>(a.gmax + (int64_t)q * a.M + 8 * piece);
              dst[0] = lo;
              dst[1] = hi;
            }
          }
        } else {
          if (cbase + 64 > a.n) {  // last base tile: padding rows become NaN, which never passes
#pragma unroll
            for (int j = 0; j < 64; ++j)
              if (cbase + j >= a.n) v[j] = 0x7fc00000u;
          }
          float m[8];
#pragma unroll
          for (int gg = 0; gg < 8; ++gg) m[gg] = max8(v, gg);
          const float tm = max3f(max3f(m[0], m[1], m[2]), max3f(m[3], m[4], m[5]), fmaxf(m[6], m[7]));
          if (__any_sync(0xffffffffu, tm >= tau)) {
            const int ibase = (int)cbase;  // ids fit in 32 bits (n < 2^31)
#pragma unroll
            for (int gg = 0; gg < 8; ++gg) {
              if (!__any_sync(0xffffffffu, m[gg] >= tau)) continue;
              int ng = 0;  // this lane's survivors in the group
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) ng += __uint_as_float(v[8 * gg + jj]) >= tau ? 1 : 0;
              if (scnt + ng > F_SBUF) flush_staged(a.cnt + q, a.cand + (int64_t)q * a.cap, a.cap, ssc, sid, scnt);
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const float s = __uint_as_float(v[8 * gg + jj]);
                if (s >= tau) {
                  ssc[scnt * BM] = s;
                  sid[scnt * BM] = ibase + 8 * gg + jj;
                  ++scnt;
                }
              }
            }
          }
        }
      }
      if (MODE == MODE_FILTER && scnt > 0)  // the next unit is another query tile
        flush_staged(a.cnt + q, a.cand + (int64_t)q * a.cap, a.cap, ssc, sid, scnt);
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 2) {
    tc_fence_after();
    tmem_dealloc(tmem, F_TMEM_COLS);
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(a.err, 2);
}

// Descending scan of one warp's 256-bin histogram: digit = the bin where the count of keys
// in bins >= digit first reaches kk, rem = kk minus the count in the bins above it.  Lane l
// owns bins 255-8l .. 248-8l.  False (digit, rem untouched) when the bins hold fewer than
// kk keys.
__device__ __forceinline__ bool digit_of_rank(const unsigned* hist, int kk, int lane, int& digit, int& rem) {
  unsigned own = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) own += hist[255 - 8 * lane - j];
  unsigned incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (__shfl_sync(0xffffffffu, incl, 31) < (unsigned)kk) return false;
  const unsigned hit = __ballot_sync(0xffffffffu, incl >= (unsigned)kk);
  const int L = __ffs(hit) - 1;
  int dg = 0, rm = 0;
  if (lane == L) {
    unsigned acc = incl - own;
    for (int j = 0; j < 8; ++j) {
      const int d = 255 - 8 * lane - j;
      const unsigned h = hist[d];
      if (acc + h >= (unsigned)kk) {
        dg = d;
        rm = kk - (int)acc;
        break;
      }
      acc += h;
    }
  }
  digit = __shfl_sync(0xffffffffu, dg, L);
  rem = __shfl_sync(0xffffffffu, rm, L);
  return true;
}

// tau[q] = (CT-th largest of the row's M group maxima) - margin, or -inf when the row has
// fewer than CT finite-or-infinite (non-NaN) maxima.  One warp per query: a 4-pass
// 8-bit radix select on order-preserving keys, histogram in shared memory.
__global__ void __launch_bounds__(256) tau_select_kernel(const float* __restrict__ gmax, int nq, int M, int CT,
                                                          float margin, float* __restrict__ tau) {
  __shared__ unsigned hist[8][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = blockIdx.x * 8 + w;
  if (q >= nq) return;  // warp-uniform; only __syncwarp below
  const float* row = gmax + (int64_t)q * M;
  uint32_t prefix = 0, pmask = 0;
  int kk = CT;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (int i = lane; i < 256; i += 32) hist[w][i] = 0;
    __syncwarp();
    for (int i = lane; i < M; i += 32) {
      const float f = row[i];
      if (f != f) continue;  // NaN maxima are not scores
      const uint32_t key = float_to_ordered(f);
      if ((key & pmask) == prefix) atomicAdd(&hist[w][(key >> shift) & 255u], 1u);
    }
    __syncwarp();
    int digit = 0, rem = 0;
    if (!digit_of_rank(hist[w], kk, lane, digit, rem)) {  // fewer than CT usable maxima (first pass only)
      if (lane == 0) tau[q] = -INFINITY;
      return;
    }
    prefix |= (uint32_t)digit << shift;
    pmask |= 255u << shift;
    kk = rem;
    __syncwarp();
  }
  if (lane == 0) tau[q] = ordered_to_float(prefix) - margin;
}

// tau_select_kernel for rows of at most 32 * R maxima (a multiple of 4), read once into
// registers by 16-byte loads.  It
// returns a lower bound of the CT-th largest maximum (minus the margin), which is all the
// filter needs -- a lower threshold only keeps more survivors, and the candidates
// selected from them are the same: a bisection on the order-preserving key between the
// row's smallest and largest maximum above -inf keeps lo with at least CT keys >= lo (so
// lo never passes the CT-th largest) and stops at 1/65536 of the range; each probe is a
// compare a key and one warp reduction (no histogram atomics, whose bins the clustered
// keys share).  With fewer than CT maxima above -inf (NaN is not a score) the CT-th
// largest is -inf, and so is tau, as in the exact select.
template <int R>
__global__ void __launch_bounds__(256) tau_select_reg_kernel(const float* __restrict__ gmax, int nq, int M, int CT,
                                                              float margin, float* __restrict__ tau) {
  const int lane = threadIdx.x & 31;
  const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (q >= nq) return;  // warp-uniform
  // all R/4 16-byte loads issued before any is used (M % 4 == 0: rows are 16-byte aligned)
  const float4* row = reinterpret_cast<const float4*>(gmax + (int64_t)q * M);
  float4 raw[R / 4];
#pragma unroll
  for (int j = 0; j < R / 4; ++j) {
    const int i4 = j * 32 + lane;
    raw[j] = 4 * i4 < M ? __ldg(row + i4) : make_float4(-INFINITY, -INFINITY, -INFINITY, -INFINITY);
  }
  uint32_t key[R];  // ordered keys; 0 = no value (no float but a NaN maps to 0)
  int valid = 0;
  uint32_t kmax = 0u, kmin = 0xffffffffu;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const float4 r4 = raw[j / 4];
    const float f = (j & 3) == 0 ? r4.x : (j & 3) == 1 ? r4.y : (j & 3) == 2 ? r4.z : r4.w;
    key[j] = (f == f && f != -INFINITY) ? float_to_ordered(f) : 0u;
    if (key[j]) {
      ++valid;
      kmax = max(kmax, key[j]);
      kmin = min(kmin, key[j]);
    }
  }
  if (__reduce_add_sync(0xffffffffu, valid) < CT) {
    if (lane == 0) tau[q] = -INFINITY;
    return;
  }
  kmax = __reduce_max_sync(0xffffffffu, kmax);
  kmin = __reduce_min_sync(0xffffffffu, kmin);
  uint64_t lo = kmin, hi = (uint64_t)kmax + 1;  // count(>= lo) >= CT > count(>= hi)
  const uint64_t stop = ((hi - lo) >> 16) + 1;
  while (hi - lo > stop) {  // warp-uniform
    const uint32_t mid = (uint32_t)(lo + ((hi - lo) >> 1));
    int c = 0;
#pragma unroll
    for (int j = 0; j < R; ++j) c += key[j] >= mid ? 1 : 0;  // empty slots (0) never count: mid >= kmin >= 1
    if (__reduce_add_sync(0xffffffffu, c) >= CT) lo = mid;
    else hi = mid;
  }
  if (lane == 0) tau[q] = ordered_to_float((uint32_t)lo) - margin;
}

// Per query (one warp): the CT = 32*E smallest keys of the survivors -- sort each chunk of
// CT keys and merge it into the running result with a bitonic "min + merge" step.  Lists
// queries whose survivors overflowed the candidate array (ovf[0] = count, ovf[1..] = ids).
template <int E>
__global__ void __launch_bounds__(256) cand_select_kernel(const int* __restrict__ cnt,
                                                           const uint64_t* __restrict__ cand, int cap, int need,
                                                           int nq, uint64_t* __restrict__ out,
                                                           int* __restrict__ ovf) {
  constexpr int CT = 32 * E;
  const int lane = threadIdx.x & 31;
  const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (q >= nq) return;  // warp-uniform
  const int c = cnt[q];
  uint64_t* dst = out + (int64_t)q * CT;
  if (c > cap || c < need) {
#pragma unroll
    for (int e = 0; e < E; ++e) dst[e * 32 + lane] = kEmptyKey;
    if (lane == 0) ovf[1 + atomicAdd(ovf, 1)] = q;
    return;
  }
  const uint64_t* src = cand + (int64_t)q * cap;
  uint64_t best[E];
#pragma unroll
  for (int e = 0; e < E; ++e) best[e] = kEmptyKey;
  for (int base = 0; base < c; base += CT) {
    uint64_t x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int i = base + e * 32 + lane;
      x[e] = i < c ? src[i] : kEmptyKey;
    }
    warp_bitonic<E>(x, lane, false);
    // best ascending, x ascending: min(best[i], x[CT-1-i]) is bitonic and holds the CT
    // smallest of the union
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const uint64_t r = __shfl_sync(0xffffffffu, x[E - 1 - e], 31 - lane);
      best[e] = best[e] < r ? best[e] : r;
    }
    warp_bitonic<E>(best, lane, true);
  }
#pragma unroll
  for (int e = 0; e < E; ++e) dst[e * 32 + lane] = best[e];
}

// Compact the bf16 rows of the listed queries into rows 0..count-1 of `dst` (the rest of
// the last 128-row tile is zeroed).
__global__ void gather_rows_kernel(const uint16_t* __restrict__ src, const int* __restrict__ ovf,
                                   uint16_t* __restrict__ dst) {
  const int cntq = ovf[0];
  const int64_t rows = (int64_t)((cntq + BM - 1) / BM) * BM;
  const int64_t chunks = rows * (KD / 8);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < chunks; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / (KD / 8);
    const int c = (int)(t % (KD / 8));
    uint4 val = make_uint4(0, 0, 0, 0);
    if (i < cntq) val = reinterpret_cast<const uint4*>(src + (int64_t)ovf[1 + i] * KD)[c];
    reinterpret_cast<uint4*>(dst + i * KD)[c] = val;
  }
}

// Merge the list kernel's per-CTA partial lists of every listed query and write the
// result over the query's row of `out`.  The split arithmetic repeats the list kernel's
// (tc_list_geometry).
__global__ void merge_fallback_kernel(const uint64_t* __restrict__ part, const int* __restrict__ ovf, int NT,
                                      int grid, int CT, uint64_t* __restrict__ out) {
  extern __shared__ uint64_t ms[];
  const int cntq = ovf[0];
  if (cntq == 0) return;
  const ListGeometry geo = tc_list_geometry(cntq, NT, grid);
  for (int i = blockIdx.x; i < cntq; i += gridDim.x) {
    const int qt = i / BM;
    const int first = (int)(((int64_t)qt * NT) / geo.per);
    const int last = (int)(((int64_t)qt * NT + NT - 1) / geo.per);
    const uint64_t* src = part + (int64_t)i * geo.maxp * CT;
    for (int j = threadIdx.x; j < CT; j += blockDim.x) ms[j] = src[j];
    __syncthreads();
    for (int s = 1; s <= last - first; ++s) {
      const uint64_t* lst = src + (int64_t)s * CT;
      for (int j = threadIdx.x; j < CT; j += blockDim.x) {
        const uint64_t b = lst[CT - 1 - j];
        if (b < ms[j]) ms[j] = b;
      }
      __syncthreads();
      block_bitonic_merge(ms, CT);
    }
    const int q = ovf[1 + i];
    for (int j = threadIdx.x; j < CT; j += blockDim.x) out[(int64_t)q * CT + j] = ms[j];
    __syncthreads();
  }
}

template <int MODE, int GW, bool F8>
void run_filter(const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& mbhi, FilterArgs a, const char* name,
                cudaStream_t s) {
  // chunk size: long enough to amortise the query-tile switch (at most 32 tiles), short
  // enough for >= 16 units per CTA so the last unit leaves little imbalance
  const int G = num_sms();
  const int64_t work = (int64_t)a.NP * a.QT;
  a.CH = (int)std::max<int64_t>(1, std::min<int64_t>(32, (work + 16 * G - 1) / (16 * G)));
  a.NCH = ceil_div(a.NP, a.CH);
  const int U = a.NCH * a.QT;
  const int grid = std::min(G, U);
  auto kern = tc_filter_kernel<MODE, GW, F8>;
  constexpr int smem = FLayout<F8>::SMEM;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  ProfScope _ps(name, s);
  kern<<<grid, F_THREADS, smem, s>>>(ma, mb, mbhi, a);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace

// Prepass parameters in units of TN-point tiles.  Large bases sample every S-th tile
// (S <= 16) and take tau at rank r = CT/S + 4 sqrt(CT/S) + 8 of the sample's 64-column
// maxima: the query's CT-th best point puts about CT/S points of the sample above it, so
// tau stays at or below that point unless the count exceeds its mean by four standard
// deviations, and about r * S points survive (CT * S with r = CT).  A query with fewer
// than CT survivors is rescanned exactly by the list kernel (cand_select lists it), so
// the rank only trades survivors against fallbacks.  S is the largest that leaves at
// least 4 r maxima a row, so that the r-th largest is a tight bound.
FilterPlan plan_filter(int64_t n, int CT) {
  FilterPlan p{};
  const int NT = ceil_div(n, TN);
  p.NT = NT;
  p.rank = CT;
  if (NT >= CT) {  // 64-column maxima: 4 a tile
    p.GW = 64;
    p.S = 1;
    for (int S : {16, 8, 4, 2}) {
      const double m = (double)CT / S;
      const int r = std::min(CT, (int)std::ceil(m + 4.0 * std::sqrt(m) + 8.0));
      if (4 * ceil_div(NT, S) >= 4 * r) {
        p.S = S;
        p.rank = r;
        break;
      }
    }
    p.NS = ceil_div(NT, p.S);
    p.M = 4 * p.NS;
    p.cap = std::max(1024, 4 * p.rank * p.S);
  } else if (NT * 32 >= 4 * CT) {  // 8-column maxima: 32 a tile
    p.GW = 8;
    p.S = 1;
    p.NS = NT;
    p.M = 32 * NT;
    p.cap = std::max(1024, 4 * CT);
  } else {  // a few thousand points: keep every one
    p.GW = 0;
    p.S = 1;
    p.NS = 0;
    p.M = 0;
    p.cap = NT * TN;
  }
  p.cap = std::min<int64_t>(p.cap, (int64_t)NT * TN);
  return p;
}

void launch_filter_scan(const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& mbhi, int hi_cols,
                        const FilterPlan& plan, int nq, int64_t n, int d, int QT, int CT, float* tau, int* cnt,
                        uint64_t* cand, int* err, bool e4m3, cudaStream_t s) {
  FilterArgs a{};
  a.hi_cols = hi_cols;
  a.nq = nq;
  a.ksteps = e4m3 ? tc_ksteps_e4m3(d) : tc_ksteps(d);
  // scores of E4M3 codes carry the factor kE4M3Scale^2
  const float margin = e4m3 ? kTauMargin * kE4M3Scale * kE4M3Scale : kTauMargin;
  a.n = n;
  a.QT = QT;
  a.err = err;
  if (plan.M > 0) {
    DevBuf<float> gmax((size_t)nq * plan.M, s);
    a.NP = plan.NS;
    a.dstride = plan.S;
    a.gmax = gmax.ptr;
    a.M = plan.M;
    if (e4m3) {
      if (plan.GW == 64) run_filter<MODE_GROUPMAX, 64, true>(ma, mb, mbhi, a, "tc_prepass", s);
      else run_filter<MODE_GROUPMAX, 8, true>(ma, mb, mbhi, a, "tc_prepass", s);
    } else {
      if (plan.GW == 64) run_filter<MODE_GROUPMAX, 64, false>(ma, mb, mbhi, a, "tc_prepass", s);
      else run_filter<MODE_GROUPMAX, 8, false>(ma, mb, mbhi, a, "tc_prepass", s);
    }
    launch_tau_select(gmax.ptr, nq, plan.M, plan.rank, margin, tau, s);
  }
  a.gmax = nullptr;
  a.M = 0;
  a.NP = plan.NT;
  a.dstride = 1;
  a.tau = plan.M > 0 ? tau : nullptr;
  a.cnt = cnt;
  a.cand = cand;
  a.cap = plan.cap;
  if (e4m3) run_filter<MODE_FILTER, 64, true>(ma, mb, mbhi, a, "tc_filter", s);
  else run_filter<MODE_FILTER, 64, false>(ma, mb, mbhi, a, "tc_filter", s);
}

void launch_tau_select(const float* gmax, int nq, int M, int rank, float margin, float* tau, cudaStream_t s) {
  ProfScope _ps("tc_tau_select", s);
  // the register slots a lane walks in every bisection step: as few as cover M
  if (M <= 32 * (kTauRegs / 2) && M % 4 == 0)
    tau_select_reg_kernel<kTauRegs / 2><<<ceil_div(nq, 8), 256, 0, s>>>(gmax, nq, M, rank, margin, tau);
  else if (M <= 32 * kTauRegs && M % 4 == 0)
    tau_select_reg_kernel<kTauRegs><<<ceil_div(nq, 8), 256, 0, s>>>(gmax, nq, M, rank, margin, tau);
  else
    tau_select_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(gmax, nq, M, rank, margin, tau);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_cand_select(const int* cnt, const uint64_t* cand, int nq, int cap, int need, int CT, uint64_t* out,
                        int* ovf, cudaStream_t s) {
  ProfScope _ps("tc_cand_select", s);
  if (CT == 32) cand_select_kernel<1><<<ceil_div(nq, 8), 256, 0, s>>>(cnt, cand, cap, need, nq, out, ovf);
  else if (CT == 64) cand_select_kernel<2><<<ceil_div(nq, 8), 256, 0, s>>>(cnt, cand, cap, need, nq, out, ovf);
  else if (CT == 128) cand_select_kernel<4><<<ceil_div(nq, 8), 256, 0, s>>>(cnt, cand, cap, need, nq, out, ovf);
  else throw Error(LSHG_ERR_INVALID_ARGUMENT, "tensor-core scan: candidate count must be 32, 64 or 128");
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_gather_rows(const uint16_t* src, const int* ovf, int nq, uint16_t* dst, cudaStream_t s) {
  const int64_t chunks = (int64_t)ceil_div(nq, BM) * BM * (KD / 8);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((chunks + 255) / 256, (int64_t)num_sms() * 4));
  gather_rows_kernel<<<blocks, 256, 0, s>>>(src, ovf, dst);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_merge_fallback(const uint64_t* part, const int* ovf, int nq, int NT, int grid, int CT, uint64_t* out,
                           cudaStream_t s) {
  const size_t smem = (size_t)CT * 8;
  merge_fallback_kernel<<<std::min(nq, num_sms() * 4), 128, smem, s>>>(part, ovf, NT, grid, CT, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace tc
}  // namespace lshg
