// Tensor-core exact scan (implementation 8; no reference counterpart -- it replaces the
// reference's FP32 exact scan, memOptimizedLinearScan.cu:20-106, for angular k-NN).
//
// Pipeline per query batch (launch_tc_scan):
//   1. queries -> unit rows in BF16, zero-padded to 128 dims (the base was converted the
//      same way at build: x / |x|);
//   2. threshold prepass + filter pass on the tensor cores (tc_filter.cu): every query
//      collects the base points whose cosine score reaches a lower bound of its CT-th best
//      score;
//   3. cand_select: the top-CT of those survivors by (score desc, id asc);
//   4. overflow fallback, entirely on the device: queries whose survivors did not fit
//      their candidate array are gathered and rescanned by tc_list_kernel below, which
//      keeps an exact per-row top-CT list in shared memory (no thresholds needed);
//   5. exact FP32 re-rank of the CT candidates with the reference's angular formula
//      (launch_rerank), top-k.
//
// tc_list_kernel is persistent (one CTA per SM) with a stream-K split of the (query tile,
// base tile) space; its CTA count and split are derived on the device from the gathered
// row count, so the fallback costs three near-empty launches when nothing overflowed.
// Warp roles:
//   warp 0  TMA producer (cp.async.bulk.tensor, 128B swizzle, mbarrier complete_tx)
//   warp 1  MMA issuer (one thread: tcgen05.mma kind::f16, M=128 N=128 K=16 x 8)
//   warp 2  TMEM allocator (four 128-column FP32 accumulators)
//   warps 4-7 epilogue: thread r owns query row r (TMEM lane r); per tile it loads its
//           128 scores with two tcgen05.ld .x64, releases the accumulator, filters with
//           a two-level maximum against the row's threshold, appends survivors to a
//           per-row buffer and folds nearly full buffers into the sorted per-row top-CT
//           lists with shuffle bitonic networks (warp_fold_row).
// Every mbarrier wait is bounded (~2 s of %globaltimer); on timeout the CTA raises the
// error flag, drains its own in-flight copies and MMAs (bounded again), frees TMEM and
// returns.
#include "index.h"
#include "launch_count.h"
#include "profile.h"
#include "tc_filter.h"
#include "tc_ptx.cuh"

#include <cuda_fp8.h>

namespace lshg {

void launch_merge_splits(const uint64_t* in, int nq, int splits, int C, uint64_t* out, cudaStream_t s);

namespace tc {

namespace {

constexpr int NTHREADS = 256;
constexpr int NACC = 4;                  // TMEM accumulator buffers of BN columns
constexpr int TMEM_COLS = NACC * BN;     // 512 = all of TMEM (one CTA per SM)
constexpr int BUFN = 32;                 // per-row append buffer (candidates awaiting a warp fold)

struct TcLayout {
  int stages, ct;
  int a_off, b_off, sc_off, id_off, bsc_off, bid_off, bar_off, total;
};

__host__ __device__ constexpr TcLayout tc_layout(int stages, int ct) {
  return TcLayout{stages,
                  ct,
                  0,
                  TILE_BYTES,
                  TILE_BYTES * (1 + stages),
                  TILE_BYTES * (1 + stages) + ct * BM * 4,
                  TILE_BYTES * (1 + stages) + ct * BM * 8,
                  TILE_BYTES * (1 + stages) + ct * BM * 8 + BUFN * BM * 4,
                  TILE_BYTES * (1 + stages) + ct * BM * 8 + BUFN * BM * 8,
                  TILE_BYTES * (1 + stages) + ct * BM * 8 + BUFN * BM * 8 + 256 + 1024};
}

// Row lists and append buffers are stored entry-major ([entry][row]) with the row index
// XOR-swizzled by the entry index, so both access patterns are bank-conflict free: one
// lane per row (appends, write-out) and one warp per row (folds).
__device__ __forceinline__ int sw(int entry, int row) { return entry * BM + (row ^ (entry & 31)); }

// (score, id) order: higher score first, then lower id.
__device__ __forceinline__ bool better(float as, int ai, float bs, int bi) {
  return as > bs || (as == bs && ai < bi);
}

// Fold the append buffer of row `rr` (cnt entries) into its sorted list of 32*E entries.
// Executed by the whole warp; returns the row's new threshold (its last list entry).
template <int E>
__device__ __noinline__ float warp_fold_row(float* lsc, int* lid, const float* bsc, const int* bid, int rr, int cnt,
                                               int lane) {
  // 1. sort the buffer (one entry per lane) descending with a 32-wide bitonic network
  float bs = lane < cnt ? bsc[sw(lane, rr)] : -INFINITY;
  int bi = lane < cnt ? bid[sw(lane, rr)] : INT_MAX;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      float os = __shfl_xor_sync(0xffffffffu, bs, j);
      int oi = __shfl_xor_sync(0xffffffffu, bi, j);
      bool desc = (lane & k) == 0 || k == 32;
      bool lower = (lane & j) == 0;
      bool take = (lower == desc) ? better(os, oi, bs, bi) : better(bs, bi, os, oi);
      if (take) { bs = os; bi = oi; }
    }
  }
  // 2. list element e*32 + lane; first bitonic-merge stage against the reversed buffer
  float ls[E];
  int li[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    ls[e] = lsc[sw(e * 32 + lane, rr)];
    li[e] = lid[sw(e * 32 + lane, rr)];
  }
  {
    float rs = __shfl_sync(0xffffffffu, bs, 31 - lane);
    int ri = __shfl_sync(0xffffffffu, bi, 31 - lane);
    if (better(rs, ri, ls[E - 1], li[E - 1])) { ls[E - 1] = rs; li[E - 1] = ri; }
  }
  // 3. bitonic merge (descending) of the 32*E list
#pragma unroll
  for (int st = E / 2; st > 0; st >>= 1) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if ((e & st) == 0) {
        if (better(ls[e | st], li[e | st], ls[e], li[e])) {
          float ts = ls[e]; int ti = li[e];
          ls[e] = ls[e | st]; li[e] = li[e | st];
          ls[e | st] = ts; li[e | st] = ti;
        }
      }
    }
  }
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    bool lower = (lane & j) == 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      float os = __shfl_xor_sync(0xffffffffu, ls[e], j);
      int oi = __shfl_xor_sync(0xffffffffu, li[e], j);
      bool take = lower ? better(os, oi, ls[e], li[e]) : better(ls[e], li[e], os, oi);
      if (take) { ls[e] = os; li[e] = oi; }
    }
  }
#pragma unroll
  for (int e = 0; e < E; ++e) {
    lsc[sw(e * 32 + lane, rr)] = ls[e];
    lid[sw(e * 32 + lane, rr)] = li[e];
  }
  return __shfl_sync(0xffffffffu, ls[E - 1], 31);
}


template <int STAGES, int CT>
__global__ void __launch_bounds__(NTHREADS, 1)
    tc_list_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const int* __restrict__ rows_dev, int64_t n, int NT, int ksteps, uint64_t* __restrict__ part,
                   int* err) {
  constexpr TcLayout L = tc_layout(STAGES, CT);
  constexpr int fold_limit = BUFN - 8;
  const int nq = *rows_dev;  // gathered query rows (0: nothing to do)
  const ListGeometry geo = tc_list_geometry(nq, NT, gridDim.x);
  const int QT = geo.QT, per = geo.per, maxp = geo.maxp;
  if ((int64_t)blockIdx.x * per >= geo.total) return;  // no tiles: leave before any barrier or TMEM use
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t s0 = smem_u32(sm);
  float* lsc = reinterpret_cast<float*>(sm + L.sc_off);
  int* lid = reinterpret_cast<int*>(sm + L.id_off);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L.bar_off);
  const uint32_t bar0 = smem_u32(bars);
  auto FULL = [&](int s) { return bar0 + 8u * s; };
  auto EMPTY = [&](int s) { return bar0 + 8u * (STAGES + s); };
  const uint32_t A_FULL = bar0 + 8u * (2 * STAGES);
  const uint32_t A_EMPTY = A_FULL + 8;
  auto ACC_FULL = [&](int b) { return bar0 + 8u * (2 * STAGES + 2 + b); };
  auto ACC_EMPTY = [&](int b) { return bar0 + 8u * (2 * STAGES + 2 + NACC + b); };
  const uint32_t DONE = bar0 + 8u * (2 * STAGES + 2 + 2 * NACC);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 3 + 2 * NACC);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int total = QT * NT;
  const int t_begin = blockIdx.x * per;
  const int t_end = min(total, t_begin + per);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(FULL(s), 1);
      mbar_init(EMPTY(s), 1);
    }
    mbar_init(A_FULL, 1);
    mbar_init(A_EMPTY, 1);
    for (int b = 0; b < NACC; ++b) {
      mbar_init(ACC_FULL(b), 1);
      mbar_init(ACC_EMPTY(b), 4);
    }
    mbar_init(DONE, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) tmem_alloc(smem_u32(tmem_slot), TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int cur_qt = -1, a_round = 0, it = 0;
      for (int t = t_begin; t < t_end; ++t) {
        const int qt = t / NT, dt = t - qt * NT;
        if (qt != cur_qt) {
          if (!mbar_wait(A_EMPTY, (a_round & 1) ^ 1, abort_flag)) break;
          mbar_expect_tx(A_FULL, TILE_BYTES);
          tma_load_2d(s0 + L.a_off, &mapA, 0, qt * BM, A_FULL);
          tma_load_2d(s0 + L.a_off + HALF_BYTES, &mapA, KHALF, qt * BM, A_FULL);
          cur_qt = qt;
          ++a_round;
        }
        const int st = it % STAGES, rd = it / STAGES;
        if (!mbar_wait(EMPTY(st), (rd & 1) ^ 1, abort_flag)) break;
        const uint32_t dst = s0 + L.b_off + st * TILE_BYTES;
        mbar_expect_tx(FULL(st), TILE_BYTES);
        tma_load_2d(dst, &mapB, 0, dt * BN, FULL(st));
        tma_load_2d(dst + HALF_BYTES, &mapB, KHALF, dt * BN, FULL(st));
        ++it;
      }
      // drain: every issued copy has landed before the CTA may exit
      for (int j = max(0, it - STAGES); j < it; ++j) mbar_wait(FULL(j % STAGES), (j / STAGES) & 1, abort_flag, true);
      if (a_round > 0) mbar_wait(A_FULL, (a_round - 1) & 1, abort_flag, true);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int cur_qt = -1, a_round = 0, it = 0;
      for (int t = t_begin; t < t_end; ++t) {
        const int qt = t / NT;
        if (qt != cur_qt) {
          if (!mbar_wait(A_FULL, a_round & 1, abort_flag)) break;
          tc_fence_after();
          cur_qt = qt;
          ++a_round;
        }
        const int b = it % NACC, ub = it / NACC;  // ub-th use of accumulator b
        if (!mbar_wait(ACC_EMPTY(b), (ub & 1) ^ 1, abort_flag)) break;
        tc_fence_after();
        const int st = it % STAGES, rd = it / STAGES;
        if (!mbar_wait(FULL(st), rd & 1, abort_flag)) break;
        tc_fence_after();
        umma_tile<BN>(tmem + (uint32_t)(b * BN), s0 + L.a_off, s0 + L.b_off + st * TILE_BYTES, ksteps);
        umma_commit(EMPTY(st));
        umma_commit(ACC_FULL(b));
        const bool last_of_qt = (t + 1 == t_end) || ((t + 1) / NT != qt);
        if (last_of_qt) umma_commit(A_EMPTY);
        ++it;
      }
      // drain: all issued MMAs complete before TMEM is released
      umma_commit(DONE);
      mbar_wait(DONE, 0, abort_flag, true);
    }
    __syncwarp();
  } else if (warp >= 4) {
    // ---------------- epilogue: per-row top-CT ----------------
    // Lanes append candidates that beat their row's threshold to the row's buffer; the
    // warp folds full buffers into the sorted row lists (warp_fold_row) and the
    // thresholds tighten.  Thresholds may lag between folds; that only admits extra
    // candidates, never drops one.
    const int r = threadIdx.x - 128;  // query row within the tile == TMEM lane
    const int row0 = r - lane;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    float* bsc = reinterpret_cast<float*>(sm + L.bsc_off);
    int* bid = reinterpret_cast<int*>(sm + L.bid_off);
    for (int i = 0; i < CT; ++i) {
      lsc[sw(i, r)] = -INFINITY;
      lid[sw(i, r)] = INT_MAX;
    }
    __syncwarp();
    float thr = -INFINITY;
    int cnt = 0;
    auto fold_all = [&](int limit) {
      unsigned m = __ballot_sync(0xffffffffu, cnt > limit);
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const int c_src = __shfl_sync(0xffffffffu, cnt, src);
        const float nt = warp_fold_row<CT / 32>(lsc, lid, bsc, bid, row0 + src, c_src, lane);
        if (lane == src) { thr = nt; cnt = 0; }
      }
      __syncwarp();
    };
    // 8-column group of the tile held in registers: append what beats the threshold
    auto group = [&](const uint32_t (&v)[64], int g, int64_t cbase) {
      const float gm = max3f(max3f(__uint_as_float(v[8 * g]), __uint_as_float(v[8 * g + 1]),
                                   __uint_as_float(v[8 * g + 2])),
                             max3f(__uint_as_float(v[8 * g + 3]), __uint_as_float(v[8 * g + 4]),
                                   __uint_as_float(v[8 * g + 5])),
                             fmaxf(__uint_as_float(v[8 * g + 6]), __uint_as_float(v[8 * g + 7])));
      if (!__any_sync(0xffffffffu, gm > thr)) return;
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const float s = __uint_as_float(v[8 * g + jj]);
        const int64_t pid = cbase + 8 * g + jj;
        if (s > thr && pid < n) {
          bsc[sw(cnt, r)] = s;
          bid[sw(cnt, r)] = (int)pid;
          ++cnt;
        }
      }
      if (__any_sync(0xffffffffu, cnt > BUFN - 8)) fold_all(fold_limit);
    };
    auto half_max = [&](const uint32_t (&v)[64]) {
      float m[22];
#pragma unroll
      for (int i = 0; i < 21; ++i)
        m[i] = max3f(__uint_as_float(v[3 * i]), __uint_as_float(v[3 * i + 1]), __uint_as_float(v[3 * i + 2]));
      m[21] = __uint_as_float(v[63]);
#pragma unroll
      for (int i = 0; i < 7; ++i) m[i] = max3f(m[3 * i], m[3 * i + 1], m[3 * i + 2]);
      m[7] = m[21];
      const float a = max3f(m[0], m[1], m[2]), b = max3f(m[3], m[4], m[5]);
      return max3f(a, b, fmaxf(m[6], m[7]));
    };
    int it = 0;
    for (int t = t_begin; t < t_end; ++t) {
      const int qt = t / NT, dt = t - qt * NT;
      const int b = it % NACC, ub = it / NACC;
      if (!mbar_wait(ACC_FULL(b), ub & 1, abort_flag)) break;
      tc_fence_after();
      const int64_t pbase = (int64_t)dt * BN;
      const uint32_t ta = tmem + lane_base + (uint32_t)(b * BN);
      uint32_t v0[64], v1[64];
      tmem_ld64(ta + 0, v0);
      tmem_ld64(ta + 64, v1);
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(ACC_EMPTY(b));  // scores are in registers: the MMA may reuse the buffer
      const float tm = fmaxf(half_max(v0), half_max(v1));
      if (__any_sync(0xffffffffu, tm > thr)) {
#pragma unroll
        for (int g = 0; g < 8; ++g) group(v0, g, pbase);
#pragma unroll
        for (int g = 0; g < 8; ++g) group(v1, g, pbase + 64);
      }
      ++it;
      const bool last_of_qt = (t + 1 == t_end) || ((t + 1) / NT != qt);
      if (last_of_qt) {
        fold_all(0);
        const int q = qt * BM + r;
        if (q < nq) {
          const int slot = blockIdx.x - (int)(((int64_t)qt * NT) / per);
          uint64_t* dst = part + ((int64_t)q * maxp + slot) * CT;
          for (int i = 0; i < CT; ++i) {
            const int id = lid[sw(i, r)];
            dst[i] = id == INT_MAX ? kEmptyKey : make_key(-lsc[sw(i, r)], id);
          }
        }
        for (int i = 0; i < CT; ++i) {
          lsc[sw(i, r)] = -INFINITY;
          lid[sw(i, r)] = INT_MAX;
        }
        __syncwarp();
        thr = -INFINITY;
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 2) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, 2);
}

// Unit rows in BF16, zero-padded to KD columns and to `rows_pad` rows.
__global__ void to_unit_bf16_kernel(const float* __restrict__ x, int64_t n, int d, int64_t rows_pad,
                                    __nv_bfloat16* __restrict__ out) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < rows_pad; i += nw) {
    float ss = 0.0f;
    if (i < n)
      for (int j = lane; j < d; j += 32) ss = fmaf(x[i * d + j], x[i * d + j], ss);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const float inv = ss > 0.0f ? rsqrtf(ss) : 0.0f;
    for (int j = lane; j < KD; j += 32) {
      float v = (i < n && j < d) ? x[i * d + j] * inv : 0.0f;
      out[i * KD + j] = __float2bfloat16_rn(v);
    }
  }
}

// Unit rows as E4M3 codes of (x / |x|) * kE4M3Scale, KD bytes a row, zero padded.
__global__ void to_unit_e4m3_kernel(const float* __restrict__ x, int64_t n, int d, int64_t rows_pad,
                                    uint8_t* __restrict__ out) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < rows_pad; i += nw) {
    float ss = 0.0f;
    if (i < n)
      for (int j = lane; j < d; j += 32) ss = fmaf(x[i * d + j], x[i * d + j], ss);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const float inv = ss > 0.0f ? rsqrtf(ss) * kE4M3Scale : 0.0f;
    for (int j = lane; j < KD; j += 32) {
      const float v = (i < n && j < d) ? x[i * d + j] * inv : 0.0f;
      out[i * KD + j] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
    }
  }
}

void to_unit_e4m3(const float* x, int64_t n, int d, int64_t rows_pad, uint8_t* out, cudaStream_t s) {
  int blocks = (int)std::min<int64_t>((rows_pad * 32 + 255) / 256, (int64_t)num_sms() * 16);
  to_unit_e4m3_kernel<<<std::max(blocks, 1), 256, 0, s>>>(x, n, d, rows_pad, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void to_unit_bf16(const float* x, int64_t n, int d, int64_t rows_pad, uint16_t* out, cudaStream_t s) {
  int64_t warps = rows_pad;
  int blocks = (int)std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)num_sms() * 16);
  to_unit_bf16_kernel<<<std::max(blocks, 1), 256, 0, s>>>(x, n, d, rows_pad, reinterpret_cast<__nv_bfloat16*>(out));
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    LSHG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) throw Error(LSHG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// Rows of KD bf16 (256 B); boxes of box_cols (<= 64) columns x box_rows rows with 128-byte
// swizzle.
CUtensorMap make_map(const void* base, int64_t rows, int box_rows, int box_cols) {
  LSHG_REQUIRE(((uintptr_t)base & 15) == 0, "TMA base must be 16-byte aligned");
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)KD, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)KD * 2};
  LSHG_REQUIRE(box_rows >= 1 && box_rows <= 256, "TMA box rows must be in [1, 256]");
  LSHG_REQUIRE(box_cols >= 8 && box_cols <= KHALF && box_cols % 8 == 0, "TMA box columns must be 8..64, multiple of 8");
  cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(LSHG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

CUtensorMap make_map_e4m3(const void* base, int64_t rows, int box_rows) {
  LSHG_REQUIRE(((uintptr_t)base & 15) == 0, "TMA base must be 16-byte aligned");
  LSHG_REQUIRE(box_rows >= 1 && box_rows <= 256, "TMA box rows must be in [1, 256]");
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)KD, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)KD};
  cuuint32_t box[2] = {(cuuint32_t)KD, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(LSHG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

CUtensorMap make_map_bytes(const void* base, int64_t rows, int kp, int box_rows) {
  LSHG_REQUIRE(((uintptr_t)base & 15) == 0 && kp % 16 == 0 && kp >= 128, "TMA: 16-byte base and row stride");
  LSHG_REQUIRE(box_rows >= 1 && box_rows <= 256, "TMA box rows must be in [1, 256]");
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kp};
  cuuint32_t box[2] = {128u, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(LSHG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

namespace {

template <int STAGES, int CT>
void run_list_kernel(const CUtensorMap& ma, const CUtensorMap& mb, const int* rows_dev, int64_t n, int NT, int d,
                     int grid, uint64_t* part, int* err, cudaStream_t s) {
  constexpr TcLayout L = tc_layout(STAGES, CT);
  auto kern = tc_list_kernel<STAGES, CT>;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L.total));
  kern<<<grid, NTHREADS, L.total, s>>>(ma, mb, rows_dev, n, NT, tc_ksteps(d), part, err);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

}  // namespace
}  // namespace tc

void tc_prepare(Index& I, cudaStream_t s) {
  using namespace tc;
  LSHG_REQUIRE(I.dist == DIST_ANGULAR, "tensor-core scan: angular distance only");
  LSHG_REQUIRE(I.d <= KD, "tensor-core scan: dimension must be <= 128");
  I.dp = KD;
  const int64_t npad = (int64_t)ceil_div(I.n, FILTER_TN) * FILTER_TN;  // whole filter tiles
  I.xbf.alloc((size_t)npad * KD, s);
  to_unit_bf16(I.x.ptr, I.n, I.d, npad, I.xbf.ptr, s);
  if (I.p.implementation == 9) {  // E4M3 operands for the filter (BF16 stays for the fallback)
    I.xf8.alloc((size_t)npad * KD, s);
    to_unit_e4m3(I.x.ptr, I.n, I.d, npad, I.xf8.ptr, s);
  }
  derive_tc(I, s);
}

void derive_tc(Index& I, cudaStream_t s) {
  if (I.p.opt.fp64_recheck == 0) return;
  I.xnorm64.alloc((size_t)I.n, s);
  launch_row_norms_fp64(I.x.ptr, I.n, I.d, I.xnorm64.ptr, s);
}

void launch_tc_scan(Index& I, const float* q, int nq, int k, lshg_point* out, cudaStream_t s,
                    const RerankBounds* extra) {
  using namespace tc;
  if (nq <= 0) return;
  LSHG_REQUIRE(k <= 128, "tensor-core scan: k must be <= 128");
  // candidates re-ranked a query: at least twice k up to k = 64 (BF16 or E4M3 scores can
  // swap near-equal neighbours at the boundary); 128 (the list kernel's maximum) beyond
  const bool e4m3 = I.p.implementation == 9;
  // E4M3 scores (3 mantissa bits) swap more near neighbours than BF16 ones: 128 candidates
  // at every k keep recall@32 above 0.99 (64 gave 0.985)
  const int CT = (k <= 32 && !e4m3) ? 64 : 128;
  int* err = I.error_word(s);
  const int64_t qpad = (int64_t)ceil_div(nq, BM) * BM;
  const int QT = (int)(qpad / BM);
  FilterPlan plan = plan_filter(I.n, CT);
  // test hook: LSHG_TC_FORCE_FALLBACK=1 sends every query through the list kernel, so
  // tests can compare the two selection paths on the same inputs
  if (const char* e = getenv("LSHG_TC_FORCE_FALLBACK"); e && e[0] == '1') plan.cap = 0;
  const int NT = ceil_div(I.n, BN);  // 128-row tiles of the list kernel
  LSHG_REQUIRE((int64_t)QT * NT < (int64_t)INT_MAX, "tensor-core scan: problem too large");
  DevBuf<uint16_t> qbf((size_t)qpad * KD, s);
  to_unit_bf16(q, nq, I.d, qpad, qbf.ptr, s);
  const CUtensorMap ma = make_map(qbf.ptr, qpad);
  const int64_t npad = (int64_t)ceil_div(I.n, FILTER_TN) * FILTER_TN;
  const CUtensorMap mb = make_map(I.xbf.ptr, npad);                    // list kernel: 128-row boxes
  const CUtensorMap mb256 = make_map(I.xbf.ptr, npad, FILTER_TN);      // filter: 256-row boxes
  // the filter's second 64-column half only up to the last K step (columns 64..16*ksteps)
  const int hi_cols = std::max(8, std::min(KHALF, 16 * tc_ksteps(I.d) - KHALF));
  const CUtensorMap mb256hi = make_map(I.xbf.ptr, npad, FILTER_TN, hi_cols);
  DevBuf<uint8_t> qf8;
  CUtensorMap ma8{}, mb8{};
  if (e4m3) {
    qf8.alloc((size_t)qpad * KD, s);
    to_unit_e4m3(q, nq, I.d, qpad, qf8.ptr, s);
    ma8 = make_map_e4m3(qf8.ptr, qpad, BM);
    mb8 = make_map_e4m3(I.xf8.ptr, npad, FILTER_TN);
  }

  // 1-2. thresholds and survivors
  DevBuf<float> tau((size_t)nq, s);
  DevBuf<int> cnt((size_t)nq + 1 + nq, s);  // [0, nq): survivors; [nq]: overflow count; then the list
  int* ovf = cnt.ptr + nq;
  LSHG_CUDA(cudaMemsetAsync(cnt.ptr, 0, (size_t)(nq + 1) * sizeof(int), s));
  DevBuf<uint64_t> cand((size_t)nq * plan.cap, s);
  if (e4m3)
    launch_filter_scan(ma8, mb8, mb8, hi_cols, plan, nq, I.n, I.d, QT, CT, tau.ptr, cnt.ptr, cand.ptr, err, true,
                       s);
  else
    launch_filter_scan(ma, mb256, mb256hi, hi_cols, plan, nq, I.n, I.d, QT, CT, tau.ptr, cnt.ptr, cand.ptr, err,
                       false, s);

  // 3. top-CT of the survivors
  DevBuf<uint64_t> best((size_t)nq * CT, s);
  // a query needs min(CT, n) survivors: fewer means its sampled threshold was too high
  launch_cand_select(cnt.ptr, cand.ptr, nq, plan.cap, (int)std::min<int64_t>(CT, I.n), CT, best.ptr, ovf, s);

  // 4. fallback for queries with more survivors than slots (massive ties) or fewer than CT
  //    (a sampled threshold above the query's CT-th best score)
  if ((int64_t)plan.cap < I.n || plan.rank < CT) {
    ProfScope _ps("tc_fallback", s);
    const int G = num_sms();
    DevBuf<uint16_t> qg((size_t)qpad * KD, s);
    launch_gather_rows(qbf.ptr, ovf, nq, qg.ptr, s);
    const CUtensorMap mg = make_map(qg.ptr, qpad);
    DevBuf<uint64_t> part((size_t)BM * (G + 2 * QT) * CT, s);
    if (CT == 64) run_list_kernel<3, 64>(mg, mb, ovf, I.n, NT, I.d, G, part.ptr, err, s);
    else run_list_kernel<1, 128>(mg, mb, ovf, I.n, NT, I.d, G, part.ptr, err, s);
    launch_merge_fallback(part.ptr, ovf, nq, NT, G, CT, best.ptr, s);
  }

  // 5. exact FP32 re-rank with the reference's angular formula
  DevBuf<float> qn((size_t)nq, s);
  launch_row_norms(q, nq, I.d, qn.ptr, s);
  launch_rerank(best.ptr, nq, CT, I.x.ptr, I.n, I.d, I.xnorm.ptr, q, qn.ptr, DIST_ANGULAR, k, out, s, err,
                I.p.opt.fp64_recheck != 0, I.xnorm64.ptr, extra);
}

}  // namespace lshg
