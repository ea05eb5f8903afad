// Tensor-core sketch scan: the Hamming distance of bit sketches as a +-1 E4M3 GEMM
// (implementations 3 and 5 -- SimHash and one-bit weighted MinHash -- in place of the
// XOR/popcount scan of scan_bits.cu for batches that fill the tensor cores; the
// reference's scanHammingDistance, sketchedDistanceScanners.cuh:14-100, and its one-bit
// scanJaccardDistance, :194-274).
//
// Bit b of a sketch becomes the E4M3 value 1 - 2b: +1.0 (0x38) or -1.0 (0xB8).  For two
// sketches of B = 32 * words bits the dot product of those rows is (#equal bits) -
// (#different bits) = B - 2 * hamming.  Every product is +-1 and every partial sum an
// integer of magnitude <= B <= 1024, which FP32 holds exactly, so the accumulator gives
// hamming = (B - dot) / 2 exactly, and the top-C by (hamming, id) equals the popcount
// scan's.  The one-bit Jaccard distance 1 - (B - hamming) / B orders points the same way.
// Rows are padded to whole 128-byte chunks with 0x00 (+0.0), which adds nothing.
//
// Selection, as in the threshold-filter scan of tc_filter.cu, in two GEMM passes:
//   prepass  on every S-th base tile writes each query's group maxima of the score (the
//            best score of each 64- or 8-point group of a sampled tile); tau[q] = the
//            r-th largest of them (launch_tau_select).  With S = 1, r = C and every point
//            of the exact top-C scores >= tau.  With S > 1, r = C/S + 4 sqrt(C/S) + 8 -- the
//            C-th best point of the base would put about C/S points of the sample above
//            it, so tau stays at or below it unless that count exceeds its mean by four
//            standard deviations -- and about r * S ~ 1.5 C points survive instead of C * S;
//   filter   on the whole base keeps the points whose score reaches tau[q], staged per row
//            in shared memory and moved to the query's candidate array with one atomicAdd
//            a batch;
//   select   keeps each query's first C survivors by (score desc, id asc): a warp sort for
//            C <= 128, a histogram of the integer scores and a sort of the ties at the
//            C-th score beyond.
//            A query with fewer than C survivors (tau above its C-th best score: the
//            sample was unrepresentative) or more than its array holds (massive ties) is
//            listed and rescanned exactly by the popcount scan on the device, so the result
//            is always the exact top-C.
//
// tc_hamming_kernel: persistent, one CTA per SM, 640 threads.  A unit is (query tile of 128
// rows, chunk of up to 32 consecutive base tiles of 256 points), numbered chunk-major so
// that all SMs stream the same base tiles at a time (each read from HBM about once a batch,
// then from L2).  The query tile stays in shared memory for the unit (KC chunks of 128 rows
// x 128 bytes); the base tile streams through a ring of one-chunk stages (256 rows x 128
// bytes).  Warp 0 issues the TMA copies, warp 1 the MMAs (tcgen05.mma kind::f8f6f4, A and
// B both E4M3, M = 128, N = 256, K = 32 each; 4 a chunk, 4 * KC a tile), warp 2 owns the
// 512 TMEM columns (two 256-column FP32 accumulators), warps 4-19 are the epilogue
// (warpgroup g reads columns [64g, 64g + 64), one query row a thread).  Every mbarrier
// wait is bounded (2 s); a CTA that times out raises error 2, drains its copies and MMAs,
// frees TMEM and returns.
#include "index.h"
#include "launch_count.h"
#include "profile.h"
#include "select.cuh"
#include "tc_filter.h"
#include "tc_ptx.cuh"

#include <cuda_bf16.h>

namespace lshg {

int launch_scan_bits_listed(const uint32_t* xst, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq,
                            int op, int C, const int* list, uint64_t* out, cudaStream_t s);

namespace tc {

namespace {

constexpr int H_THREADS = 640;
constexpr int HN = 256;           // base points a tile (UMMA N)
constexpr int H_CHUNK = 128;      // bytes of a row in one K chunk (one 128-byte swizzle row)
constexpr int H_NACC = 2;         // TMEM accumulators of HN columns
constexpr int H_TMEM_COLS = H_NACC * HN;
constexpr int H_EPI_WARPS = 16;
constexpr int H_SEL_MAX = 16384;  // survivors a query the block select sorts at most
constexpr int kHTauRegs = 80;

constexpr int kSmemLimit = 232448;  // dynamic shared memory a CTA may opt into

// Shared-memory layout for rows of KC chunks.  The survivor staging takes what is left
// (8, 4, 2 or 1 entries a row and warpgroup; none: each survivor takes its own slot).
template <int KC>
struct HLayout {
  static constexpr int A_BYTES = KC * BM * H_CHUNK;  // resident query tile
  static constexpr int B_BYTES = HN * H_CHUNK;       // one chunk of a base tile: 32 KB
  static constexpr int STAGES = KC <= 4 ? 4 : 3;
  static constexpr int FIXED = A_BYTES + STAGES * B_BYTES + 256 + 1024;  // + barriers + alignment slack
  static constexpr int ROOM = (kSmemLimit - FIXED) / (4 * BM * 8);
  static constexpr int SBUF = ROOM >= 8 ? 8 : ROOM >= 4 ? 4 : ROOM >= 2 ? 2 : ROOM >= 1 ? 1 : 0;
  static constexpr int A_OFF = 0;
  static constexpr int B_OFF = A_BYTES;
  static constexpr int S_OFF = B_OFF + STAGES * B_BYTES;  // scores then ids, [4][SBUF][BM] each
  static constexpr int BAR_OFF = S_OFF + 4 * SBUF * BM * 8;
  static constexpr int SMEM = BAR_OFF + 256 + 1024;
  static_assert(SMEM <= kSmemLimit, "shared memory per CTA");
  static_assert(8 * (2 * STAGES + 2 + 2 * H_NACC + 1) + 12 <= 256, "barrier area");
};

constexpr int MODE_SIGNS = 2;  // SimHash projections: sign bits, uncertain ones listed

struct HArgs {
  int nq;
  int64_t n;
  int QT;           // query tiles
  int NP;           // base positions scanned (base tile = p * dstride)
  int dstride;
  int CH;           // positions a unit
  int NCH;          // chunks of positions
  float* gmax;      // MODE_GROUPMAX: [nq][M] group maxima
  int M;
  const float* tau; // MODE_FILTER: threshold a query (nullptr: keep every point)
  int* cnt;         // survivors a query
  uint64_t* cand;   // [nq][cap] survivor keys
  int cap;
  int* err;
  // MODE_SIGNS: rows are points, the "base" is the planes
  const float* rown;   // point norms
  const float* pnorm;  // plane norms (padded to whole tiles with zeros)
  float band;          // a sign is certain when |score| > band * |x| * |r|
  uint32_t* out32;     // [nq][words] sign bits
  int words, P;        // words a point, planes (32 * words)
  uint2* list;         // [grid][list_cap] (point, plane) of the uncertain signs, a segment a CTA
  int* list_cnt;       // [grid] entries a segment (may exceed list_cap: overflow)
  int list_cap;
};

// Out of line: called from every group of the unrolled survivor path, inlined copies would
// crowd the instruction cache.
__device__ __noinline__ void h_flush(int* cnt, uint64_t* dst, int cap, const float* ssc, const int* sid, int scnt) {
  const int base = atomicAdd(cnt, scnt);
  for (int e = 0; e < scnt; ++e)
    if (base + e < cap) dst[base + e] = make_key(-ssc[e * BM], sid[e * BM]);
}

// BF: operands are BF16 (kind::f16, 64 elements a 128-byte chunk) instead of E4M3.
template <int MODE, int GW, int KC, bool BF = false>
__global__ void __launch_bounds__(H_THREADS, 1)
    tc_hamming_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                      const HArgs a) {
  using LY = HLayout<KC>;
  constexpr int STAGES = LY::STAGES, SBUF = LY::SBUF;
  static_assert(MODE != MODE_FILTER || GW == 64, "the filter reads whole 64-column pieces");
  static_assert(GW == 64 || GW == 8, "group width");
  const int U = a.NCH * a.QT;
  if ((int)blockIdx.x >= U) return;  // no unit for this CTA: leave before any barrier or TMEM use

  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t s0 = smem_u32(sm);
  const uint32_t bar0 = s0 + LY::BAR_OFF;
  auto FULL = [&](int s) { return bar0 + 8u * s; };
  auto EMPTY = [&](int s) { return bar0 + 8u * (STAGES + s); };
  const uint32_t A_FULL = bar0 + 8u * (2 * STAGES);
  const uint32_t A_EMPTY = bar0 + 8u * (2 * STAGES + 1);
  auto ACC_FULL = [&](int b) { return bar0 + 8u * (2 * STAGES + 2 + b); };
  auto ACC_EMPTY = [&](int b) { return bar0 + 8u * (2 * STAGES + 2 + H_NACC + b); };
  const uint32_t DONE = bar0 + 8u * (2 * STAGES + 2 + 2 * H_NACC);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + LY::BAR_OFF + 8 * (2 * STAGES + 3 + 2 * H_NACC));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(FULL(s), 1);
      mbar_init(EMPTY(s), 1);
    }
    mbar_init(A_FULL, 1);
    mbar_init(A_EMPTY, 1);
    for (int b = 0; b < H_NACC; ++b) {
      mbar_init(ACC_FULL(b), 1);
      mbar_init(ACC_EMPTY(b), H_EPI_WARPS);
    }
    mbar_init(DONE, 1);
    *abort_flag = 0;
    *reinterpret_cast<int*>(tmem_slot + 2) = 0;  // MODE_SIGNS list count
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) tmem_alloc(smem_u32(tmem_slot), H_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0, na = 0;  // base chunks and query tiles issued
      bool ok = true;
      for (int u = blockIdx.x; u < U && ok; u += gridDim.x) {
        const int qt = u % a.QT, c = u / a.QT;
        const int p0 = c * a.CH, p1 = min(a.NP, p0 + a.CH);
        // The unit's first STAGES base chunks are issued before its query tile: their
        // stages free up as the previous unit's MMAs consume the ring, so the copies run
        // while those MMAs finish.  There is one query-tile buffer: it is reloaded once
        // the previous unit's MMAs have completed.
        const int total = (p1 - p0) * KC, pre = min(STAGES, total);
        for (int ci = 0; ci <= total; ++ci) {
          if (ci == pre) {
            if (!mbar_wait(A_EMPTY, (na & 1) ^ 1, abort_flag)) { ok = false; break; }
            mbar_expect_tx(A_FULL, LY::A_BYTES);
#pragma unroll
            for (int kc = 0; kc < KC; ++kc)
              tma_load_2d(s0 + LY::A_OFF + kc * BM * H_CHUNK, &mapA, kc * H_CHUNK, qt * BM, A_FULL);
            ++na;
          }
          if (ci == total) break;
          const int p = p0 + ci / KC, kc = ci % KC;
          const int st = it % STAGES, rd = it / STAGES;
          if (!mbar_wait(EMPTY(st), (rd & 1) ^ 1, abort_flag)) { ok = false; break; }
          mbar_expect_tx(FULL(st), LY::B_BYTES);
          tma_load_2d(s0 + LY::B_OFF + st * LY::B_BYTES, &mapB, kc * H_CHUNK, p * a.dstride * HN, FULL(st));
          ++it;
        }
      }
      // drain: every issued copy has landed before the CTA may exit
      for (int j = max(0, it - STAGES); j < it; ++j) mbar_wait(FULL(j % STAGES), (j / STAGES) & 1, abort_flag, true);
      if (na > 0) mbar_wait(A_FULL, (na - 1) & 1, abort_flag, true);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = BF ? idesc_bf16(BM, HN) : idesc_e4m3(BM, HN);
      int it = 0, ia = 0, ua = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < U && ok; u += gridDim.x, ++ua) {
        const int c = u / a.QT;
        const int p0 = c * a.CH, p1 = min(a.NP, p0 + a.CH);
        if (!mbar_wait(A_FULL, ua & 1, abort_flag)) break;
        tc_fence_after();
        for (int p = p0; p < p1 && ok; ++p) {
          const int b = ia % H_NACC, ub = ia / H_NACC;
          if (!mbar_wait(ACC_EMPTY(b), (ub & 1) ^ 1, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const uint32_t d_tmem = tmem + (uint32_t)(b * HN);
          for (int kc = 0; kc < KC; ++kc) {
            const int st = it % STAGES, rd = it / STAGES;
            if (!mbar_wait(FULL(st), rd & 1, abort_flag)) { ok = false; break; }
            tc_fence_after();
            const uint32_t a_base = s0 + LY::A_OFF + kc * BM * H_CHUNK;
            const uint32_t b_base = s0 + LY::B_OFF + st * LY::B_BYTES;
#pragma unroll
            for (int kk = 0; kk < H_CHUNK / 32; ++kk) {  // 32 bytes a step: K = 32 E4M3 or 16 BF16
              if (BF)
                umma_bf16(d_tmem, smem_desc(a_base + kk * 32), smem_desc(b_base + kk * 32), idesc,
                          (kc > 0 || kk > 0) ? 1u : 0u);
              else
                umma_e4m3(d_tmem, smem_desc(a_base + kk * 32), smem_desc(b_base + kk * 32), idesc,
                          (kc > 0 || kk > 0) ? 1u : 0u);
            }
            umma_commit(EMPTY(st));
            ++it;
          }
          if (!ok) break;
          umma_commit(ACC_FULL(b));
          ++ia;
        }
        umma_commit(A_EMPTY);  // the query tile is free once this unit's MMAs complete
      }
      // drain: all issued MMAs complete before TMEM is released
      umma_commit(DONE);
      mbar_wait(DONE, 0, abort_flag, true);
    }
    __syncwarp();
  } else if (warp >= 4) {
    // ---------------- epilogue ----------------
    const int g = (warp - 4) >> 2;         // warpgroup: columns [64g, 64g+64) of every accumulator
    const int r = (warp & 3) * 32 + lane;  // query row within the tile = TMEM lane
    const uint32_t tbase = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(g * 64);
    float* ssc = reinterpret_cast<float*>(sm + LY::S_OFF) + (size_t)g * SBUF * BM + r;
    int* sid = reinterpret_cast<int*>(sm + LY::S_OFF + 4 * SBUF * BM * 4) + (size_t)g * SBUF * BM + r;
    int scnt = 0;
    int ia = 0;
    bool ok = true;
    int* seg_cnt = reinterpret_cast<int*>(tmem_slot + 2);  // MODE_SIGNS: this CTA's list count
    uint2* seg = MODE == MODE_SIGNS ? a.list + (int64_t)blockIdx.x * a.list_cap : nullptr;
    for (int u = blockIdx.x; u < U && ok; u += gridDim.x) {
      const int qt = u % a.QT, c = u / a.QT;
      const int p0 = c * a.CH, p1 = min(a.NP, p0 + a.CH);
      const int q = qt * BM + r;
      float tau = INFINITY;
      if (MODE == MODE_FILTER && q < a.nq) tau = a.tau ? a.tau[q] : -INFINITY;
      for (int p = p0; p < p1; ++p) {
        const int b = ia % H_NACC, ub = ia / H_NACC;
        if (!mbar_wait(ACC_FULL(b), ub & 1, abort_flag)) { ok = false; break; }
        tc_fence_after();
        uint32_t v[64];
        tmem_ld64(tbase + (uint32_t)(b * HN), v);
        tmem_wait_ld();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(ACC_EMPTY(b));  // scores are in registers: the MMA may reuse the buffer
        ++ia;
        const int64_t cbase = (int64_t)p * a.dstride * HN + g * 64;  // base id of v[0]
        const int piece = 4 * p + g;
        if (MODE == MODE_SIGNS) {
          // bit = score >= 0, as the reference's sign test; a sign within the split-BF16
          // error bound of zero is listed for the exact recheck
          if (q < a.nq && cbase < a.P) {
            const float bx = a.band * a.rown[q];
            const float4* pn4 = reinterpret_cast<const float4*>(a.pnorm + cbase);
            uint32_t w0 = 0, w1 = 0;
#pragma unroll
            for (int j4 = 0; j4 < 16; ++j4) {
              const float4 pn = __ldg(pn4 + j4);
              const float pv[4] = {pn.x, pn.y, pn.z, pn.w};
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const int j = 4 * j4 + e;
                const float sc = __uint_as_float(v[j]);
                const uint32_t bit = sc >= 0.0f ? 1u : 0u;
                if (j < 32) w0 |= bit << j;
                else w1 |= bit << (j - 32);
                if (fabsf(sc) <= bx * pv[e] && cbase + j < a.P) {
                  const int pos = atomicAdd(seg_cnt, 1);
                  if (pos < a.list_cap) seg[pos] = make_uint2((uint32_t)q, (uint32_t)(cbase + j));
                }
              }
            }
            uint32_t* row = a.out32 + (int64_t)q * a.words + (cbase >> 5);
            row[0] = w0;
            if (cbase + 32 < a.P) row[1] = w1;
          }
        } else if (MODE == MODE_GROUPMAX) {
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
          if (cbase + 64 > a.n) {  // padding rows become NaN, which never passes
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
            int* qcnt = a.cnt + q;
            uint64_t* qdst = a.cand + (int64_t)q * a.cap;
#pragma unroll
            for (int gg = 0; gg < 8; ++gg) {
              if (!__any_sync(0xffffffffu, m[gg] >= tau)) continue;
              if (SBUF > 0) {
                int ng = 0;
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) ng += __uint_as_float(v[8 * gg + jj]) >= tau ? 1 : 0;
                if (scnt + ng > SBUF) {
                  h_flush(qcnt, qdst, a.cap, ssc, sid, scnt);
                  scnt = 0;
                }
              }
#pragma unroll
              for (int jj = 0; jj < 8; ++jj) {
                const float sc = __uint_as_float(v[8 * gg + jj]);
                if (sc >= tau) {
                  if (SBUF >= 8 || (SBUF > 0 && scnt < SBUF)) {  // 8 entries always fit after a flush
                    ssc[scnt * BM] = sc;
                    sid[scnt * BM] = ibase + 8 * gg + jj;
                    ++scnt;
                  } else {  // no staging room: a slot of its own
                    const int pos = atomicAdd(qcnt, 1);
                    if (pos < a.cap) qdst[pos] = make_key(-sc, ibase + 8 * gg + jj);
                  }
                }
              }
            }
          }
        }
      }
      if (MODE == MODE_FILTER && SBUF > 0 && scnt > 0) {  // the next unit is another query tile
        h_flush(a.cnt + q, a.cand + (int64_t)q * a.cap, a.cap, ssc, sid, scnt);
        scnt = 0;
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 2) {
    tc_fence_after();
    tmem_dealloc(tmem, H_TMEM_COLS);
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(a.err, 2);
  if (MODE == MODE_SIGNS && threadIdx.x == 0) a.list_cnt[blockIdx.x] = *reinterpret_cast<int*>(tmem_slot + 2);
}

// Sketch rows of wp words (the first `words` real) -> E4M3 rows of kp bytes: bit b of word w
// (LSB first) -> byte 32w + b = 0x38 (+1) for a 0 bit, 0xB8 (-1) for a 1 bit; bytes past
// 32 * words and rows past n are 0x00.  One thread writes 16 bytes (half a word).
__global__ void expand_bits_kernel(const uint32_t* __restrict__ xs, int64_t n, int wp, int words, int kp,
                                   int64_t rows_pad, uint4* __restrict__ out) {
  const int per_row = kp / 16;
  const int64_t total = rows_pad * per_row;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / per_row;
    const int h = (int)(t - i * per_row);  // 16-byte piece of the row: bits 16h .. 16h + 15
    const int w = h >> 1;
    uint4 o = make_uint4(0, 0, 0, 0);
    if (i < n && w < words) {
      const uint32_t bits = xs[i * wp + w] >> (16 * (h & 1));
      uint32_t r[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const uint32_t nib = (bits >> (4 * e)) & 0xFu;
        // bit j of the nibble -> bit 7 of byte j (the sign of +-1.0)
        const uint32_t spread = (nib & 1u) << 7 | (nib & 2u) << 14 | (nib & 4u) << 21 | (nib & 8u) << 28;
        r[e] = 0x38383838u | spread;
      }
      o = make_uint4(r[0], r[1], r[2], r[3]);
    }
    out[t] = o;
  }
}

// Top-C (C <= 128) of each query's survivors, one warp a query; a query whose survivor count
// is below `need` or above `cap` is listed in ovf (ovf[0] = count, ovf[1..] = queries).
template <int E>
__global__ void __launch_bounds__(256) hsel_warp_kernel(const int* __restrict__ cnt, const uint64_t* __restrict__ cand,
                                                        int cap, int need, int nq, uint64_t* __restrict__ out,
                                                        int* __restrict__ ovf) {
  constexpr int CT = 32 * E;
  const int lane = threadIdx.x & 31;
  const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (q >= nq) return;  // warp-uniform
  const int c = cnt[q];
  uint64_t* dst = out + (int64_t)q * CT;
  if (c > cap || c < need) {
    if (lane == 0) ovf[1 + atomicAdd(ovf, 1)] = q;
    return;  // the rescan writes this row
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
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const uint64_t rr = __shfl_sync(0xffffffffu, x[E - 1 - e], 31 - lane);
      best[e] = best[e] < rr ? best[e] : rr;
    }
    warp_bitonic<E>(best, lane, true);
  }
#pragma unroll
  for (int e = 0; e < E; ++e) dst[e * 32 + lane] = best[e];
}

// Top-C (C > 128) of each query's survivors as a set, one block a query, using the integer
// scores: a histogram of the scores (2 * bits + 1 bins) gives the score t of the C-th best
// survivor; every survivor above t is in, and of those at t the ones with the lowest ids
// (the survivors' keys sorted in shared memory: they order by id within one score).  The
// set goes out unordered -- the re-rank sorts it.  A query whose survivors at t exceed
// H_TIE_MAX is listed for the exact rescan, as are those with fewer than `need` or more
// than `cap` survivors.
constexpr int H_TIE_MAX = 4096;
constexpr int H_BINS_MAX = 2049;

__global__ void __launch_bounds__(512) hsel_hist_kernel(const int* __restrict__ cnt, const uint64_t* __restrict__ cand,
                                                        int cap, int need, int C, int bits,
                                                        uint64_t* __restrict__ out, int* __restrict__ ovf) {
  __shared__ uint64_t tie[H_TIE_MAX];
  __shared__ int hist[H_BINS_MAX];
  __shared__ int s_t, s_below, s_nout, s_ntie;
  const int q = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
  const int c = cnt[q];
  if (c > cap || c < need) {
    if (tid == 0) ovf[1 + atomicAdd(ovf, 1)] = q;
    return;
  }
  const uint64_t* src = cand + (int64_t)q * cap;
  uint64_t* dst = out + (int64_t)q * C;
  if (c <= C) {  // a base of fewer than C points: all of them, then empty keys
    for (int i = tid; i < C; i += blockDim.x) dst[i] = i < c ? src[i] : kEmptyKey;
    return;
  }
  const int nb = 2 * bits + 1;
  for (int i = tid; i < nb; i += blockDim.x) hist[i] = 0;
  if (tid == 0) {
    s_nout = 0;
    s_ntie = 0;
  }
  __syncthreads();
  // a key holds -score; bin = bits - score: 0 is the best score
  for (int i = tid; i < c; i += blockDim.x) atomicAdd(&hist[(int)key_dist(src[i]) + bits], 1);
  __syncthreads();
  if (tid < 32) {  // the bin where the running count reaches C
    const int per = (nb + 31) / 32, b0 = lane * per, b1 = min(nb, b0 + per);
    int own = 0;
    for (int b = b0; b < b1; ++b) own += hist[b];
    int incl = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, incl >= C);
    const int L = __ffs(hit) - 1;  // hit != 0: the bins hold c > C keys
    if (lane == L) {
      int acc = incl - own;
      for (int b = b0; b < b1; ++b) {
        if (acc + hist[b] >= C) {
          s_t = b;
          s_below = acc;
          break;
        }
        acc += hist[b];
      }
    }
  }
  __syncthreads();
  const int t = s_t, below = s_below;
  const int nt = hist[t];
  if (nt > H_TIE_MAX) {  // block-uniform
    if (tid == 0) ovf[1 + atomicAdd(ovf, 1)] = q;
    return;
  }
  for (int i = tid; i < c; i += blockDim.x) {
    const uint64_t key = src[i];
    const int b = (int)key_dist(key) + bits;
    if (b < t) dst[atomicAdd(&s_nout, 1)] = key;
    else if (b == t) tie[atomicAdd(&s_ntie, 1)] = key;
  }
  __syncthreads();
  int P = 64;
  while (P < nt) P <<= 1;
  for (int i = nt + tid; i < P; i += blockDim.x) tie[i] = kEmptyKey;
  __syncthreads();
  block_bitonic_sort(tie, P);
  for (int i = tid; i < C - below; i += blockDim.x) dst[below + i] = tie[i];
}

// Rows of kp bytes (a multiple of 128); boxes of 128 bytes x box_rows rows, 128-byte swizzle.
CUtensorMap map_sketch_rows(const void* base, int64_t rows, int kp, int box_rows) {
  LSHG_REQUIRE(((uintptr_t)base & 15) == 0 && kp % H_CHUNK == 0, "sketch rows: 16-byte base, 128-byte rows");
  return make_map_bytes(base, rows, kp, box_rows);
}

template <int MODE, int GW, int KC, bool BF = false>
void run_hamming(const CUtensorMap& ma, const CUtensorMap& mb, HArgs a, const char* name, cudaStream_t s,
                 int* grid_out = nullptr) {
  const int G = num_sms();
  const int64_t work = (int64_t)a.NP * a.QT;
  a.CH = (int)std::max<int64_t>(1, std::min<int64_t>(32, (work + 8 * G - 1) / (8 * G)));
  a.NCH = ceil_div(a.NP, a.CH);
  const int U = a.NCH * a.QT;
  const int grid = std::min(G, U);
  if (grid_out) *grid_out = grid;
  auto kern = tc_hamming_kernel<MODE, GW, KC, BF>;
  constexpr int smem = HLayout<KC>::SMEM;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  ProfScope _ps(name, s);
  kern<<<grid, H_THREADS, smem, s>>>(ma, mb, a);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

template <int MODE, int GW>
void run_hamming_kc(int kc, const CUtensorMap& ma, const CUtensorMap& mb, const HArgs& a, const char* name,
                    cudaStream_t s) {
  switch (kc) {
    case 1: run_hamming<MODE, GW, 1>(ma, mb, a, name, s); break;
    case 2: run_hamming<MODE, GW, 2>(ma, mb, a, name, s); break;
    case 3: run_hamming<MODE, GW, 3>(ma, mb, a, name, s); break;
    case 4: run_hamming<MODE, GW, 4>(ma, mb, a, name, s); break;
    case 5: run_hamming<MODE, GW, 5>(ma, mb, a, name, s); break;
    case 6: run_hamming<MODE, GW, 6>(ma, mb, a, name, s); break;
    case 7: run_hamming<MODE, GW, 7>(ma, mb, a, name, s); break;
    case 8: run_hamming<MODE, GW, 8>(ma, mb, a, name, s); break;
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "tensor-core sketch scan: rows of 1..8 chunks of 128 bits");
  }
}

// ---- SimHash projections on the tensor cores ---------------------------------------------
// A float v is split into two BF16 values hi = bf16(v), lo = bf16(v - hi) (the subtraction
// is exact), so v - hi - lo is within 2^-16 |v|.  Points become rows [hi | hi | lo] and
// planes [hi | lo | hi] (each part padded to kp columns), and one BF16 GEMM with K = 3 kp
// gives x_hi r_hi + x_hi r_lo + x_lo r_hi, within 3 * 2^-16 sum |x_j r_j| <= 3 * 2^-16 |x||r|
// of the exact x.r before the FP32 accumulation's own rounding.  norms: the rows' L2 norms.
__global__ void split_bf16_kernel(const float* __restrict__ x, int64_t n, int d, int kp, int64_t rows_pad, int order,
                                  __nv_bfloat16* __restrict__ out, float* __restrict__ norms) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < rows_pad; i += nw) {
    __nv_bfloat16* row = out + i * 3 * kp;
    float ss = 0.0f;
    for (int j = lane; j < kp; j += 32) {
      const float v = (i < n && j < d) ? x[i * d + j] : 0.0f;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
      row[j] = hi;
      row[kp + j] = order == 0 ? hi : lo;
      row[2 * kp + j] = order == 0 ? lo : hi;
      ss = fmaf(v, v, ss);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    if (lane == 0) norms[i] = sqrtf(ss);
  }
}

// Exact signs of the listed (point, plane) pairs: the reference's single-precision FMA chain
// over the dimensions in order (the same arithmetic as project_kernel), written into the
// sign bit.  A segment whose count exceeds its capacity raises *overflow.
__global__ void sign_recheck_kernel(const uint2* __restrict__ list, const int* __restrict__ cnt, int cap, int segs,
                                    const float* __restrict__ x, const float* __restrict__ planes, int d,
                                    uint32_t* __restrict__ out32, int words, int* __restrict__ overflow) {
  const int64_t total = (int64_t)segs * cap;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int seg = (int)(t / cap), i = (int)(t - (int64_t)seg * cap);
    const int c = cnt[seg];
    if (i == 0 && c > cap) atomicExch(overflow, 1);
    if (i >= c) continue;
    const uint2 e = list[t];
    const float* xr = x + (int64_t)e.x * d;
    const float* rr = planes + (int64_t)e.y * d;
    float acc = 0.0f;
    for (int j = 0; j < d; ++j) acc = __fmaf_rn(xr[j], rr[j], acc);
    uint32_t* w = out32 + (int64_t)e.x * words + (e.y >> 5);
    const uint32_t bit = 1u << (e.y & 31);
    if (acc >= 0.0f) atomicOr(w, bit);
    else atomicAnd(w, ~bit);
  }
}

}  // namespace

int signs_part_cols(int d) { return d <= 64 ? 64 : 128; }

void launch_split_bf16(const float* x, int64_t n, int d, int64_t rows_pad, int order, uint16_t* out, float* norms,
                       cudaStream_t s) {
  LSHG_REQUIRE(d >= 1 && d <= 128, "tensor-core projections: d must be <= 128");
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((rows_pad * 32 + 255) / 256, (int64_t)num_sms() * 16));
  split_bf16_kernel<<<blocks, 256, 0, s>>>(x, n, d, signs_part_cols(d), rows_pad, order,
                                           reinterpret_cast<__nv_bfloat16*>(out), norms);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_tc_signs(const float* x, int64_t n, int d, const uint16_t* planes_split, const float* pnorm,
                     const float* planes, int P, int words, uint32_t* out32, int* err, cudaStream_t s) {
  if (n <= 0) return;
  LSHG_REQUIRE(P == 32 * words && P >= 32, "tensor-core projections: whole 32-plane words");
  const int kp = signs_part_cols(d), kc = 3 * kp * 2 / H_CHUNK;
  const int64_t rows_pad = (int64_t)ceil_div(n, BM) * BM;
  const int64_t ppad = (int64_t)ceil_div(P, HN) * HN;
  LSHG_REQUIRE(rows_pad / BM * (ppad / HN) < (int64_t)INT_MAX, "tensor-core projections: problem too large");
  ProfScope _ps("tc_project", s);
  DevBuf<uint16_t> xa((size_t)rows_pad * 3 * kp, s);
  DevBuf<float> xn((size_t)rows_pad, s);
  launch_split_bf16(x, n, d, rows_pad, 0, xa.ptr, xn.ptr, s);
  const CUtensorMap ma = map_sketch_rows(xa.ptr, rows_pad, 6 * kp, BM);
  const CUtensorMap mb = map_sketch_rows(planes_split, ppad, 6 * kp, HN);
  // about 0.1% of the signs of unit points and N(0, 1) planes fall inside the band; each
  // CTA's segment holds 4x its share, and the SIMT projection redoes everything if one
  // overflows
  const int G = num_sms();
  const int64_t expect = (int64_t)n * P / 1000 / G + 1;
  const int cap = (int)std::min<int64_t>(1 << 22, std::max<int64_t>(4096, 4 * expect));
  DevBuf<uint2> list((size_t)G * cap, s);
  DevBuf<int> cnt((size_t)G + 1, s);
  LSHG_CUDA(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes(), s));
  HArgs a{};
  a.nq = (int)n;
  a.n = P;
  a.QT = (int)(rows_pad / BM);
  a.NP = (int)(ppad / HN);
  a.dstride = 1;
  a.err = err;
  a.rown = xn.ptr;
  a.pnorm = pnorm;
  a.band = 1.0f / 8192.0f;  // 2^-13: 2.7x the split's 3 * 2^-16, plus the accumulations' rounding
  a.out32 = out32;
  a.words = words;
  a.P = P;
  a.list = list.ptr;
  a.list_cnt = cnt.ptr;
  a.list_cap = cap;
  int grid = 0;
  if (kc == 3) run_hamming<MODE_SIGNS, 64, 3, true>(ma, mb, a, "tc_project_gemm", s, &grid);
  else run_hamming<MODE_SIGNS, 64, 6, true>(ma, mb, a, "tc_project_gemm", s, &grid);
  int* overflow = cnt.ptr + G;
  {
    const int64_t total = (int64_t)grid * cap;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)G * 16));
    sign_recheck_kernel<<<blocks, 256, 0, s>>>(list.ptr, cnt.ptr, cap, grid, x, planes, d, out32, words, overflow);
    count_launch();
    LSHG_CHECK_LAUNCH();
  }
  // an overflowing segment lost entries: the SIMT projection then redoes every sign (its
  // blocks leave at once when nothing overflowed)
  launch_project_gated(x, n, d, planes, P, words, out32, overflow, s);
}

HammingPlan plan_hamming(int64_t n, int C) {
  HammingPlan p{};
  p.ok = true;
  const int NT = ceil_div(n, HN);
  p.NT = NT;
  p.GW = 0;
  p.S = 1;
  p.NS = 0;
  p.M = 0;
  p.rank = C;
  if ((int64_t)NT * HN <= (C <= 128 ? 8192 : H_SEL_MAX)) {  // small base: every point survives
    p.cap = NT * HN;
    return p;
  }
  for (int S : {16, 8, 4, 2, 1}) {
    const int NS = ceil_div(NT, S);
    const double m = (double)C / S;
    const int r = S == 1 ? C : std::min(C, (int)std::ceil(m + 4.0 * std::sqrt(m) + 8.0));
    for (int GW : {64, 8}) {
      const int64_t M = (int64_t)NS * (HN / GW);
      if (M >= 4 * (int64_t)r) {
        p.S = S;
        p.NS = NS;
        p.GW = GW;
        p.M = (int)M;
        p.rank = r;
        const int64_t want = 3 * (int64_t)r * S + 2048;
        int64_t cap = 1024;
        while (cap < want) cap <<= 1;
        if (C > 128) cap = std::min<int64_t>(cap, H_SEL_MAX);
        p.cap = (int)std::min<int64_t>(cap, (int64_t)NT * HN);
        return p;
      }
    }
  }
  // fewer than 4 C group maxima even without sampling: the popcount scan serves it
  p.ok = false;
  return p;
}

int hamming_chunks(int words) { return (words + 3) / 4; }

void launch_expand_bits(const uint32_t* xs, int64_t n, int wp, int words, int64_t rows_pad, uint8_t* out,
                        cudaStream_t s) {
  const int kp = hamming_chunks(words) * H_CHUNK;
  const int64_t total = rows_pad * (kp / 16);
  if (total <= 0) return;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  expand_bits_kernel<<<blocks, 256, 0, s>>>(xs, n, wp, words, kp, rows_pad, reinterpret_cast<uint4*>(out));
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_int_select(const int* cnt, const uint64_t* cand, int cap, int need, int C, int bits, int nq, uint64_t* out,
                       int* ovf, cudaStream_t s) {
  ProfScope _ps("tc_hamming_select", s);
  LSHG_REQUIRE(bits >= 1 && 2 * bits + 1 <= H_BINS_MAX, "integer select: scores of at most 1024 bits");
  if (C <= 128) {
    if (C == 32) hsel_warp_kernel<1><<<ceil_div(nq, 8), 256, 0, s>>>(cnt, cand, cap, need, nq, out, ovf);
    else if (C == 64) hsel_warp_kernel<2><<<ceil_div(nq, 8), 256, 0, s>>>(cnt, cand, cap, need, nq, out, ovf);
    else hsel_warp_kernel<4><<<ceil_div(nq, 8), 256, 0, s>>>(cnt, cand, cap, need, nq, out, ovf);
  } else {
    hsel_hist_kernel<<<nq, 512, 0, s>>>(cnt, cand, cap, need, C, bits, out, ovf);
  }
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_tc_hamming(const uint8_t* xse, int64_t n, const uint32_t* xst, int wp, int words, const uint32_t* qs,
                       int nq, int op, int C, uint64_t* out, int* err, cudaStream_t s) {
  if (nq <= 0) return;
  LSHG_REQUIRE(words >= 1 && words <= 32, "tensor-core sketch scan: 1..32 words a sketch");
  LSHG_REQUIRE(C >= 32 && C <= 4096 && (C & (C - 1)) == 0, "tensor-core sketch scan: C must be a power of two");
  const int kc = hamming_chunks(words), kp = kc * H_CHUNK;
  const int64_t qpad = (int64_t)ceil_div(nq, BM) * BM;
  const int QT = (int)(qpad / BM);
  const int64_t npad = (int64_t)ceil_div(n, HN) * HN;
  const HammingPlan plan = plan_hamming(n, C);
  LSHG_REQUIRE(plan.ok, "tensor-core sketch scan: C too large for this base");
  LSHG_REQUIRE((int64_t)QT * plan.NT < (int64_t)INT_MAX, "tensor-core sketch scan: problem too large");
  DevBuf<uint8_t> qe((size_t)qpad * kp, s);
  {
    ProfScope _ps("tc_hamming_expand", s);
    launch_expand_bits(qs, nq, wp, words, qpad, qe.ptr, s);
  }
  const CUtensorMap ma = map_sketch_rows(qe.ptr, qpad, kp, BM);
  const CUtensorMap mb = map_sketch_rows(xse, npad, kp, HN);
  HArgs a{};
  a.nq = nq;
  a.n = n;
  a.QT = QT;
  a.err = err;
  DevBuf<float> tau(nq, s);
  if (plan.M > 0) {
    DevBuf<float> gmax((size_t)nq * plan.M, s);
    a.NP = plan.NS;
    a.dstride = plan.S;
    a.gmax = gmax.ptr;
    a.M = plan.M;
    if (plan.GW == 64) run_hamming_kc<MODE_GROUPMAX, 64>(kc, ma, mb, a, "tc_hamming_prepass", s);
    else run_hamming_kc<MODE_GROUPMAX, 8>(kc, ma, mb, a, "tc_hamming_prepass", s);
    // scores are integers, computed the same way in both passes: no margin
    launch_tau_select(gmax.ptr, nq, plan.M, plan.rank, 0.0f, tau.ptr, s);
  }
  DevBuf<int> cnt(nq, s);
  LSHG_CUDA(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes(), s));
  DevBuf<uint64_t> cand((size_t)nq * plan.cap, s);
  a.gmax = nullptr;
  a.M = 0;
  a.NP = plan.NT;
  a.dstride = 1;
  a.tau = plan.M > 0 ? tau.ptr : nullptr;
  a.cnt = cnt.ptr;
  a.cand = cand.ptr;
  a.cap = plan.cap;
  run_hamming_kc<MODE_FILTER, 64>(kc, ma, mb, a, "tc_hamming", s);
  DevBuf<int> ovf((size_t)nq + 1, s);
  LSHG_CUDA(cudaMemsetAsync(ovf.ptr, 0, sizeof(int), s));
  launch_int_select(cnt.ptr, cand.ptr, plan.cap, (int)std::min<int64_t>(C, n), C, 32 * words, nq, out, ovf.ptr, s);
  // listed queries: exact popcount rescan written straight into their rows of `out`
  launch_scan_bits_listed(xst, n, wp, words, 0, qs, nq, op, C, ovf.ptr, out, s);
}

}  // namespace tc
}  // namespace lshg
