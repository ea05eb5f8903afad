// (K,L) LSH bucket tables and bucket-gather query (lshFramework.cuh:102-280).
//
// Build (same three steps as the reference): per-table key histogram; exclusive scan into
// absolute offsets where table t's region starts at t*N (buildHashBucketIndexes,
// :115-124 -- done here by one CTA per table instead of one serial thread); scatter of
// point ids with atomic cursors (:126-140).  Order inside a bucket is the atomic order,
// as in the reference; nothing downstream depends on it and exports sort it.
//
// Query (scan, :142-252 + removeDuplicates, :255-280): a CTA per query gathers the ids
// of its L buckets (bucket t ends at the next key's offset, or at the table's end for
// the last key, :183-184), drops repeats (the reference keeps repeats in its queue and
// removes adjacent equal ids after sorting), scores each distinct candidate exactly or by
// sketch, keeps the best C by (distance, id), and for sketched scoring re-ranks them
// exactly (candidateSetScan, :236-238) before writing the first k.  Fewer than k distinct
// candidates leave (-1, INT_MAX) entries.  Exact scoring with staged rows runs as two
// kernels: lsh_walk_kernel drops repeats in a shared-memory id set and lists each
// query's distinct ids, lsh_score_kernel scores the lists with rows staged in shared
// memory by bulk copies (staged_key).  Sketched scoring, and queries whose lists
// overflow, run the fused lsh_query_kernel, which drops repeats with a per-CTA bitmap.
#include "common.cuh"
#include "distance.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "profile.h"
#include "select.cuh"
#include "tc_ptx.cuh"

namespace lshg {

namespace {

constexpr int kQThreads = 256;
constexpr int kQBuf = 2 * kQThreads;
constexpr int kMaxTables = 256;
constexpr int kUnroll = 8;                    // bucket entries a thread loads per round
constexpr int kRound = kUnroll * kQThreads;   // entries walked per round
constexpr int kScoreAt = 1024;                // score the distinct list once it holds this many
constexpr int kListCap = kScoreAt + kRound;   // a round adds at most kRound ids
constexpr int kStageRows = 16;                // rows a warp stages per bulk-copy batch
constexpr int kStageMaxBytes = 136 * 1024;    // staging area limit (d up to 268 at 16 rows x 8 warps)
constexpr int kWalkCtasPerSm = 4;             // bucket-walk CTAs an SM (split path; 48 KB id set each)
constexpr int kWalkSlots = 12288;             // slots of a walk CTA's shared id set
constexpr int kSplitCap = 6144;               // distinct candidates a query listed by the walk
static_assert(3 * (kSplitCap + kRound) <= 2 * kWalkSlots, "walk id set: load factor at most 2/3");
static_assert(kWalkSlots % 4 == 0, "walk id set: cleared with 16-byte stores");
constexpr int kScoreCtasPerSm = 3;            // scoring CTAs an SM (register budget: 80 a thread)
constexpr int kQueryCtasPerSm = 3;            // resident fused-kernel CTAs an SM (register budget;
                                              // d = 128 staging, 66 KB a CTA, allows three)

__global__ void lsh_hist_kernel(const uint16_t* __restrict__ keys, int64_t n, int tables, int S, int* counts) {
  int64_t total = n * tables;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int t = (int)(i % tables);
    atomicAdd(&counts[(int64_t)t * S + keys[i]], 1);
  }
}

// One CTA per table: counts -> absolute exclusive offsets (table base t*n).
__global__ void lsh_scan_kernel(int* offsets, int S, int64_t n) {
  __shared__ int part[1024];
  const int t = blockIdx.x;
  int* row = offsets + (int64_t)t * S;
  const int per = (S + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per;
  int local = 0;
  for (int i = 0; i < per; ++i) if (b + i < S) local += row[b + i];
  part[threadIdx.x] = local;
  __syncthreads();
  for (int off = 1; off < (int)blockDim.x; off <<= 1) {
    int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = (int)(t * n) + (threadIdx.x ? part[threadIdx.x - 1] : 0);
  for (int i = 0; i < per; ++i) {
    if (b + i < S) {
      int c = row[b + i];
      row[b + i] = run;
      run += c;
    }
  }
}

__global__ void lsh_scatter_kernel(const uint16_t* __restrict__ keys, int64_t n, int tables, int S, int* cursors,
                                   int* __restrict__ buckets) {
  int64_t total = n * tables;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t p = i / tables;
    int t = (int)(i - p * tables);
    int pos = atomicAdd(&cursors[(int64_t)t * S + keys[i]], 1);
    buckets[pos] = (int)p;
  }
}

template <int DIST>
__device__ __forceinline__ float sketch_distance(const LshQueryArgs& a, int id, const uint32_t* qsk, const float* qsf) {
  if (a.sketch_kind == 6) {
    const float* r = a.xsf + (int64_t)id * a.sdim;
    float acc = 0.0f;
    for (int j = 0; j < a.sdim; ++j) {
      float df = __fsub_rn(qsf[j], r[j]);
      acc = __fmaf_rn(df, df, acc);
    }
    return acc;
  }
  const uint32_t* r = a.xs + (int64_t)id * a.wp;
  int acc = 0;
  if (a.sketch_kind == OP_BYTE_JACCARD) {
    for (int w = 0; w < a.wp; ++w) {
      uint32_t z = r[w] ^ qsk[w];
      uint32_t t = (z & 0x7f7f7f7fu) + 0x7f7f7f7fu;
      acc += __popc(~(t | z | 0x7f7f7f7fu));
    }
    return __fsub_rn(1.0f, __fdiv_rn((float)acc, (float)a.sbytes));
  }
  for (int w = 0; w < a.wp; ++w) acc += __popc(r[w] ^ qsk[w]);
  if (a.sketch_kind == OP_HAMMING) return (float)acc;
  return __fsub_rn(1.0f, __fdiv_rn((float)(32 * a.words - acc), (float)(32 * a.words)));
}



// Bounded wait on a staging barrier; on timeout raises error 3 (when err is given).
__device__ __forceinline__ bool stage_wait(uint32_t bar, uint32_t parity, int* err) {
  if (tc::mbar_try(bar, parity)) return true;
  const uint64_t t0 = tc::global_ns();
  while (!tc::mbar_try_sleep(bar, parity, 20000u)) {
    if (tc::global_ns() - t0 > tc::kWaitNs) {
      if (err) atomicExch(err, 3);
      return false;
    }
  }
  return true;
}

// Key of lane's candidate `id` (-1: none), warp-collective.  Rows are fetched by bulk
// copies into the warp's staging slots, kStageRows lanes at a time (a 16-byte lane load
// per row element would cap the gather near 2 TB/s: 32 scattered lines an instruction),
// then each lane runs its row's chain from shared memory in the same order as
// exact_distance.  If a copy wait times out, the warp stops staging (ok = false) and
// reads rows directly from then on; `pending` keeps the parity left incomplete.
template <int DIST>
__device__ __forceinline__ uint64_t staged_key(const LshQueryArgs& a, int id, const float* qr, float qn,
                                               unsigned char* stage, uint32_t bar, uint32_t& phase, bool& ok,
                                               uint32_t& pending) {
  const int lane = threadIdx.x & 31;
  const uint32_t rowb = (uint32_t)a.d * 4u, slot = stage_slot_bytes(a.d);
  const float xn = (DIST == DIST_ANGULAR && id >= 0) ? a.xnorm[id] : 1.0f;
  float dist = 0.0f;
#pragma unroll 1
  for (int b = 0; b < 32 / kStageRows; ++b) {
    const bool mine = id >= 0 && (lane / kStageRows) == b;
    const unsigned m = __ballot_sync(0xffffffffu, mine);
    if (!m) continue;
    unsigned char* dst = stage + (uint32_t)(lane % kStageRows) * slot;
    if (ok) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier slot reads first
      if (lane == 0) tc::mbar_expect_tx(bar, (uint32_t)__popc(m) * rowb);
      __syncwarp();
      if (mine) tc::bulk_load(tc::smem_u32(dst), a.x + (int64_t)id * a.d, rowb, bar);
      ok = __all_sync(0xffffffffu, stage_wait(bar, phase, a.err));
      if (!ok) pending = phase;
      phase ^= 1u;
    }
    if (mine) {
      dist = ok ? exact_distance_v4<DIST, true>(reinterpret_cast<const float4*>(dst),
                                                reinterpret_cast<const float4*>(qr), a.d >> 2, qn, xn)
                : exact_distance_v4<DIST, false>(reinterpret_cast<const float4*>(a.x + (int64_t)id * a.d),
                                                 reinterpret_cast<const float4*>(qr), a.d >> 2, qn, xn);
    }
    __syncwarp();
  }
  return id >= 0 ? make_key(dist, id) : kEmptyKey;
}

// Table of flat bucket-entry index idx: the t with pref[t] <= idx < pref[t+1].
__device__ __forceinline__ int entry_table(const int* pref, int tables, int idx) {
  int lo = 0, hi = tables;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (pref[mid] <= idx) lo = mid; else hi = mid;
  }
  return lo;
}

// A CTA answers the queries it takes off the batch counter a.qctr.  Per query: (1) the bucket
// entries are walked kUnroll per thread per round, deduplicated, and distinct ids appended
// to a shared list; (2) whenever the list holds kScoreAt ids (and after the last round)
// they are scored, one thread per candidate, and offered to the top-C queue.  Scoring
// order does not matter: keys (distance, id) are unique, so the kept set is the same.
template <int DIST>
__global__ void __launch_bounds__(kQThreads, kQueryCtasPerSm) lsh_query_kernel(LshQueryArgs a, lshg_point* __restrict__ out) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int NW = kQThreads / 32;
  const uint32_t stage_slot = stage_slot_bytes(a.d);
  const uint32_t stage_bytes = a.stage ? (uint32_t)(NW * kStageRows) * stage_slot : 0u;
  uint64_t* kept = reinterpret_cast<uint64_t*>(smem + stage_bytes);
  uint64_t* buf = kept + a.C;
  uint64_t* rk = buf + kQBuf;  // re-rank keys [C]
  // the distinct-id list lives in global memory (L2): kept out of shared memory it lets
  // three CTAs share an SM
  int* list = a.lists + (int64_t)blockIdx.x * kListCap;
  float* qr = reinterpret_cast<float*>(rk + a.C);
  const int dpad = (a.d + 3) & ~3;
  float* qsf = qr + dpad;
  uint32_t* qsk = reinterpret_cast<uint32_t*>(qsf + (a.sketch_kind == 6 ? a.sdim : 0));
  __shared__ int bstart[kMaxTables], pref[kMaxTables + 1];
  __shared__ int cnt_s;
  __shared__ int rcnt[3];  // ids appended per round, cycled: round r uses rcnt[r % 3]
  __shared__ uint64_t thr_s;
  TopCShared S{kept, buf, &cnt_s, &thr_s, a.C, kQBuf};
  __shared__ __align__(8) uint64_t stage_bar[NW];
  uint32_t* bitmap = a.bitmaps + (int64_t)blockIdx.x * ((a.n + 31) / 32);
  const int tid = threadIdx.x, lane = tid & 31;
  unsigned char* stage_w = smem + (uint32_t)((tid >> 5) * kStageRows) * stage_slot;
  const uint32_t bar_w = tc::smem_u32(&stage_bar[tid >> 5]);
  uint32_t sphase = 0, spending = 0;
  bool sok = true;  // warp-uniform
  if (a.stage) {
    if (tid < NW) tc::mbar_init(tc::smem_u32(&stage_bar[tid]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const int nloop = a.qlist ? a.qlist[0] : a.nq;
  bool bitmap_zero = !a.bitmap_dirty;  // uniform
  __shared__ int qslot[2];  // alternate slots: thread 0 fills the next before all read the last
  for (int it = 0;; ++it) {
    if (tid == 0) qslot[it & 1] = atomicAdd(a.qctr, 1);  // queries come off the batch counter
    __syncthreads();
    const int ii = qslot[it & 1];
    if (ii >= nloop) break;
    if (!bitmap_zero) {  // nobody zeroed the bitmap: do it before the CTA's first query
      for (int w = tid; w < (a.n + 31) / 32; w += kQThreads) bitmap[w] = 0u;
      __syncthreads();
      bitmap_zero = true;
    }
    const int qi = a.qlist ? a.qlist[1 + ii] : ii;
    for (int j = tid; j < dpad; j += kQThreads) qr[j] = j < a.d ? a.q[(int64_t)qi * a.d + j] : 0.0f;
    if (a.sketched) {
      if (a.sketch_kind == 6) {
        for (int j = tid; j < a.sdim; j += kQThreads) qsf[j] = a.qsf[(int64_t)qi * a.sdim + j];
      } else {
        for (int j = tid; j < a.wp; j += kQThreads) qsk[j] = a.qs[(int64_t)qi * a.wp + j];
      }
    }
    for (int t = tid; t < a.tables; t += kQThreads) {
      const int key = a.qkeys[(int64_t)qi * a.tables + t];
      int st = 0, en = 0;  // a key outside the table addresses no bucket
      if (key < a.tableSize) {
        st = a.offsets[(int64_t)t * a.tableSize + key];
        en = (key >= a.tableSize - 1) ? (int)(t * a.n + a.n) : a.offsets[(int64_t)t * a.tableSize + key + 1];
      }
      bstart[t] = st;
      pref[t + 1] = en - st;
    }
    topc_init(S, 1);
    if (tid == 0) rcnt[0] = rcnt[1] = rcnt[2] = 0;
    __syncthreads();
    if (tid == 0) {
      pref[0] = 0;
      for (int t = 0; t < a.tables; ++t) pref[t + 1] += pref[t];
    }
    __syncthreads();
    const float qn = (DIST == DIST_ANGULAR) ? a.qnorm[qi] : 1.0f;
    const int total = pref[a.tables];
    uint64_t thr = kEmptyKey;
    int distinct = 0;
    int lbase = 0;  // ids in the list before this round (uniform)
    for (int base = 0, r = 0; base < total; base += kRound, ++r) {
      // rcnt[(r+1) % 3] was last read right after round r-2's barrier, so every thread
      // is done with it once thread 0 has passed round r-1's barrier
      if (tid == 0) rcnt[(r + 1) % 3] = 0;
      int ids[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const int idx = base + u * kQThreads + tid;
        ids[u] = -1;
        if (idx < total) {
          const int t = entry_table(pref, a.tables, idx);
          ids[u] = a.buckets[bstart[t] + (idx - pref[t])];
        }
      }
      // Dedupe on the CTA's bitmap (one bit a base point): the thread whose atomicOr sets
      // an id's bit reports it new, so every distinct id is listed exactly once.  Every
      // atomic of the round is issued before any result is used, so the round costs one
      // L2 round trip, not kUnroll of them.  (A shared-memory id set in front of the bitmap
      // measured slower once rows were staged: its 32 KB cost resident CTAs.)
      uint32_t old[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u)
        old[u] = ids[u] >= 0 ? atomicOr(&bitmap[ids[u] >> 5], 1u << (ids[u] & 31)) : ~0u;
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {  // append the new ids: one shared atomic a warp
        const bool fresh = !(old[u] & (1u << (ids[u] & 31)));
        const unsigned m = __ballot_sync(0xffffffffu, fresh);
        if (m) {
          const int leader = __ffs(m) - 1;
          int wbase = 0;
          if (lane == leader) wbase = atomicAdd(&rcnt[r % 3], __popc(m));
          wbase = __shfl_sync(0xffffffffu, wbase, leader);
          if (fresh) list[lbase + wbase + __popc(m & ((1u << lane) - 1u))] = ids[u];
        }
      }
      __syncthreads();
      const int nl = lbase + rcnt[r % 3];  // uniform: rcnt[r % 3] is not written again before round r+3
      if (nl < kScoreAt && base + kRound < total) {
        lbase = nl;
        continue;
      }
      for (int i0 = 0; i0 < nl; i0 += kQThreads) {
        const int i = i0 + tid;
        if (a.stage) {  // uniform: every lane takes part in the warp's copies
          const uint64_t key = staged_key<DIST>(a, i < nl ? list[i] : -1, qr, qn, stage_w, bar_w, sphase, sok,
                                                spending);
          if (i < nl) topc_push(S, 0, key, thr);
        } else if (i < nl) {
          const int id = list[i];
          float dist;
          if (a.sketched) {
            dist = sketch_distance<DIST>(a, id, qsk, qsf);
          } else {
            const float xn = DIST == DIST_ANGULAR ? a.xnorm[id] : 1.0f;
            dist = a.vec4 ? exact_distance_v4<DIST>(reinterpret_cast<const float4*>(a.x + (int64_t)id * a.d),
                                                     reinterpret_cast<const float4*>(qr), a.d >> 2, qn, xn)
                          : exact_distance<DIST>(a.x + (int64_t)id * a.d, qr, a.d, qn, xn);
          }
          topc_push(S, 0, make_key(dist, id), thr);
        }
        // until the kept list is full every key is pushed: fold as soon as it can be
        // filled, so the first fold sorts at most one sub-round's keys
        topc_flush<true>(S, 1, thr == kEmptyKey ? a.C - 1 : kQBuf - kQThreads);
        thr = thr_s;
      }
      distinct += nl;
      lbase = 0;  // the list is reused: topc_flush's last barrier follows every read of it
    }
    topc_flush<true>(S, 1, 0);
    if (a.stats && tid == 0) {
      atomicAdd(a.stats, (unsigned long long)total);
      atomicAdd(a.stats + 1, (unsigned long long)distinct);
    }
    for (int idx = tid; idx < total; idx += kQThreads) {  // clear the bitmap words this query set
      const int t = entry_table(pref, a.tables, idx);
      const int id = a.buckets[bstart[t] + (idx - pref[t])];
      bitmap[id >> 5] = 0u;
    }
    const uint64_t* fin = kept;
    if (a.sketched) {
      for (int i = tid; i < a.C; i += kQThreads) {
        const uint64_t kin = kept[i];
        uint64_t ko = kEmptyKey;
        if (kin != kEmptyKey) {
          const int id = key_id(kin);
          ko = make_key(exact_distance<DIST>(a.x + (int64_t)id * a.d, qr, a.d, qn,
                                             DIST == DIST_ANGULAR ? a.xnorm[id] : 1.0f), id);
        }
        rk[i] = ko;
      }
      __syncthreads();
      block_bitonic_sort(rk, a.C);
      fin = rk;
    }
    for (int i = tid; i < a.k; i += kQThreads) {
      const uint64_t kk = i < a.C ? fin[i] : kEmptyKey;
      lshg_point pt;
      if (kk == kEmptyKey) { pt.ID = -1; pt.distance = kEmptyDistance; }
      else { pt.ID = key_id(kk); pt.distance = key_dist(kk); }
      out[(int64_t)qi * a.k + i] = pt;
    }
    __syncthreads();
  }
  if (a.stage && !sok) stage_wait(bar_w, spending, nullptr);  // a timed-out copy may still land
}

// Bucket bounds of query qi into bstart[t] (first entry of table t's bucket) and pref
// (pref[0] = 0, pref[t + 1] = entries of tables 0..t), by one warp: 32 tables a pass,
// prefix sums by shuffles.
__device__ __forceinline__ void bucket_bounds_warp(const LshQueryArgs& a, int qi, int* bstart, int* pref,
                                                   int lane) {
  int carry = 0;
  for (int t0 = 0; t0 < a.tables; t0 += 32) {
    const int t = t0 + lane;
    int st = 0, len = 0;  // a key outside the table addresses no bucket
    if (t < a.tables) {
      const int key = a.qkeys[(int64_t)qi * a.tables + t];
      if (key < a.tableSize) {
        st = a.offsets[(int64_t)t * a.tableSize + key];
        const int en = (key >= a.tableSize - 1) ? (int)(t * a.n + a.n)
                                                : a.offsets[(int64_t)t * a.tableSize + key + 1];
        len = en - st;
      }
    }
    int v = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    if (t < a.tables) {
      bstart[t] = st;
      pref[t + 1] = carry + v;
    }
    carry += __shfl_sync(0xffffffffu, v, 31);
  }
  if (lane == 0) pref[0] = 0;
}

// Open-addressing set of point ids in shared memory (kWalkSlots slots, -1 = empty, linear
// probing from a Fibonacci hash mapped onto the slots by a multiply-shift).  True when id
// was absent.  The walk inserts at most cap + kRound ids a query, at most 2/3 of
// kWalkSlots, so a free slot is always found; the probe count is bounded all the same.
__device__ __forceinline__ bool seen_insert(int* seen, int id) {
  uint32_t h = (uint32_t)(((uint64_t)((uint32_t)id * 2654435769u) * (uint32_t)kWalkSlots) >> 32);
  for (int p = 0; p < kWalkSlots; ++p) {
    const int prev = atomicCAS(&seen[h], -1, id);
    if (prev == -1) return true;
    if (prev == id) return false;
    h = h + 1 == (uint32_t)kWalkSlots ? 0u : h + 1;
  }
  return false;
}

__device__ __forceinline__ void seen_clear(int* seen, int tid) {
  for (int i = tid; i < kWalkSlots / 4; i += kQThreads) reinterpret_cast<int4*>(seen)[i] = make_int4(-1, -1, -1, -1);
}

// Split path, step 1 (exact scoring with staged rows): walk each query's buckets, drop
// repeats in the CTA's shared-memory id set and write the distinct ids to
// cand[q][0..cap); ccnt[q] = distinct count (a query with more than cap is listed in ovf
// for the fused kernel, and its walk stops there).  No scoring state and no global
// atomics on the entries: one barrier a round, and the set is cleared with 16-byte shared
// stores.  CTAs take queries off the batch counter *qctr (zero at launch), so the batch's
// uneven queries spread evenly over them.
__global__ void __launch_bounds__(kQThreads, kWalkCtasPerSm)
    lsh_walk_kernel(LshQueryArgs a, int* __restrict__ cand, int cap, int* __restrict__ ccnt, int* __restrict__ ovf,
                    int* __restrict__ qctr) {
  extern __shared__ __align__(16) int seen[];  // kWalkSlots ids
  __shared__ int bstart[kMaxTables], pref[kMaxTables + 1];
  __shared__ int wcnt, qcur;
  const int tid = threadIdx.x, lane = tid & 31;
  seen_clear(seen, tid);
  for (;;) {
    // warp 0 takes the next query and loads its bucket bounds; the previous query's last
    // reads of qcur/bstart/pref/wcnt precede its closing barrier
    if (tid < 32) {
      int q = 0;
      if (lane == 0) q = atomicAdd(qctr, 1);
      q = __shfl_sync(0xffffffffu, q, 0);
      if (q < a.nq) bucket_bounds_warp(a, q, bstart, pref, lane);
      if (lane == 0) {
        qcur = q;
        wcnt = 0;
      }
    }
    __syncthreads();
    const int qi = qcur;
    if (qi >= a.nq) break;
    const int total = pref[a.tables];
    int* dst = cand + (int64_t)qi * cap;
    for (int base = 0; base < total; base += kRound) {
      // a query past cap goes to the fused kernel anyway: stop walking it (the OR makes the
      // decision uniform; wcnt only grows, so a stale read only delays it a round)
      if (base > 0 && __syncthreads_or(wcnt > cap)) break;
      // a warp takes kUnroll * 32 consecutive entries, a lane every 32nd: its table index
      // only moves forward, so one search a round and a bucket-end compare an entry
      int ids[kUnroll];
      {
        const int i0 = base + (tid >> 5) * (kUnroll * 32) + lane;
        int t = i0 < total ? entry_table(pref, a.tables, i0) : 0;
        int tend = pref[t + 1], off = bstart[t] - pref[t];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
          const int idx = i0 + u * 32;
          ids[u] = -1;
          if (idx < total) {
            while (idx >= tend) {  // ends: idx < total = pref[tables]
              ++t;
              tend = pref[t + 1];
              off = bstart[t] - pref[t];
            }
            ids[u] = a.buckets[off + idx];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const bool fresh = ids[u] >= 0 && seen_insert(seen, ids[u]);
        const unsigned m = __ballot_sync(0xffffffffu, fresh);
        if (m) {
          const int leader = __ffs(m) - 1;
          int wbase = 0;
          if (lane == leader) wbase = atomicAdd(&wcnt, __popc(m));
          wbase = __shfl_sync(0xffffffffu, wbase, leader);
          const int pos = wbase + __popc(m & ((1u << lane) - 1u));
          if (fresh && pos < cap) dst[pos] = ids[u];
        }
      }
    }
    __syncthreads();  // every insert of the query is done: wcnt is final, the set may be cleared
    seen_clear(seen, tid);
    if (tid == 0) {
      const int distinct = wcnt;
      ccnt[qi] = distinct;
      if (distinct > cap) ovf[1 + atomicAdd(ovf, 1)] = qi;  // the fused kernel counts it
      else if (a.stats) {
        atomicAdd(a.stats, (unsigned long long)total);
        atomicAdd(a.stats + 1, (unsigned long long)distinct);
      }
    }
  }
}

// Split path, step 2: score each listed query's distinct candidates (rows staged by bulk
// copies, staged_key) into its top-C and write the first k.  Queries whose lists
// overflowed are left to the fused kernel.  Queries come off the batch counter *qctr.
template <int DIST>
__global__ void __launch_bounds__(kQThreads, kScoreCtasPerSm)
    lsh_score_kernel(LshQueryArgs a, const int* __restrict__ cand, int cap, const int* __restrict__ ccnt,
                     lshg_point* __restrict__ out, int* __restrict__ qctr) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int NW = kQThreads / 32;
  const uint32_t stage_slot = stage_slot_bytes(a.d);
  const uint32_t stage_bytes = (uint32_t)(NW * kStageRows) * stage_slot;
  uint64_t* kept = reinterpret_cast<uint64_t*>(smem + stage_bytes);
  uint64_t* buf = kept + a.C;
  float* qr = reinterpret_cast<float*>(buf + kQBuf);
  const int dpad = (a.d + 3) & ~3;
  __shared__ int cnt_s;
  __shared__ uint64_t thr_s;
  __shared__ __align__(8) uint64_t stage_bar[NW];
  TopCShared S{kept, buf, &cnt_s, &thr_s, a.C, kQBuf};
  const int tid = threadIdx.x;
  unsigned char* stage_w = smem + (uint32_t)((tid >> 5) * kStageRows) * stage_slot;
  const uint32_t bar_w = tc::smem_u32(&stage_bar[tid >> 5]);
  uint32_t sphase = 0, spending = 0;
  bool sok = true;  // warp-uniform
  if (tid < NW) tc::mbar_init(tc::smem_u32(&stage_bar[tid]), 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  __shared__ int qslot[2];  // alternate slots: thread 0 fills the next before all read the last
  for (int it = 0;; ++it) {
    if (tid == 0) qslot[it & 1] = atomicAdd(qctr, 1);  // queries come off the batch counter
    __syncthreads();
    const int qi = qslot[it & 1];
    if (qi >= a.nq) break;
    const int c = ccnt[qi];
    if (c > cap) continue;  // uniform: the fused kernel answers this query
    for (int j = tid; j < dpad; j += kQThreads) qr[j] = j < a.d ? a.q[(int64_t)qi * a.d + j] : 0.0f;
    topc_init(S, 1);
    __syncthreads();
    const float qn = (DIST == DIST_ANGULAR) ? a.qnorm[qi] : 1.0f;
    const int* lst = cand + (int64_t)qi * cap;
    uint64_t thr = kEmptyKey;
    for (int i0 = 0; i0 < c; i0 += kQThreads) {
      const int i = i0 + tid;
      const uint64_t key = staged_key<DIST>(a, i < c ? lst[i] : -1, qr, qn, stage_w, bar_w, sphase, sok, spending);
      // until the list is full every key is pushed: fold as soon as it can be filled; later
      // fold only when the buffer could not take another sub-round (one barrier otherwise)
      const int limit = thr == kEmptyKey ? a.C - 1 : kQBuf - kQThreads;
      bool over = false;
      if (i < c && key < thr) {
        const int pos = atomicAdd(&cnt_s, 1);
        buf[pos] = key;
        over = pos >= limit;
      }
      if (__syncthreads_or(over)) {
        topc_flush<true>(S, 1, limit);
        thr = thr_s;
      }
    }
    topc_flush<true>(S, 1, 0);
    for (int i = tid; i < a.k; i += kQThreads) {
      const uint64_t kk = i < a.C ? kept[i] : kEmptyKey;
      lshg_point pt;
      if (kk == kEmptyKey) { pt.ID = -1; pt.distance = kEmptyDistance; }
      else { pt.ID = key_id(kk); pt.distance = key_dist(kk); }
      out[(int64_t)qi * a.k + i] = pt;
    }
    __syncthreads();
  }
  if (!sok) stage_wait(bar_w, spending, nullptr);  // a timed-out copy may still land
}

}  // namespace

void launch_lsh_build(const uint16_t* keys, int64_t n, int tables, int tableSize, int* offsets, int* buckets,
                      int* cursors, cudaStream_t s) {
  LSHG_REQUIRE(n > 0 && tables > 0 && tables <= kMaxTables, "LSH: bad table count");
  LSHG_REQUIRE(n * tables < (int64_t)INT_MAX, "LSH: N * tables must fit in int32");
  size_t cells = (size_t)tables * tableSize;
  LSHG_CUDA(cudaMemsetAsync(offsets, 0, cells * sizeof(int), s));
  int64_t total = n * tables;
  int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  lsh_hist_kernel<<<blocks, 256, 0, s>>>(keys, n, tables, tableSize, offsets);
  count_launch();
  LSHG_CHECK_LAUNCH();
  lsh_scan_kernel<<<tables, 1024, 0, s>>>(offsets, tableSize, n);
  count_launch();
  LSHG_CHECK_LAUNCH();
  LSHG_CUDA(cudaMemcpyAsync(cursors, offsets, cells * sizeof(int), cudaMemcpyDeviceToDevice, s));
  lsh_scatter_kernel<<<blocks, 256, 0, s>>>(keys, n, tables, tableSize, cursors, buckets);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

static size_t lsh_stage_bytes(int d) { return (size_t)(kQThreads / 32) * kStageRows * stage_slot_bytes(d); }

size_t lsh_query_smem(const LshQueryArgs& a) {
  return (a.stage ? lsh_stage_bytes(a.d) : 0) + (size_t)(2 * a.C + kQBuf) * 8 +
         (size_t)((a.d + 3) & ~3) * 4 + (size_t)(a.sketch_kind == 6 ? a.sdim : 0) * 4 + (size_t)a.wp * 4 + 16;
}

template <int DV>
static int lsh_ctas_per_sm(size_t smem) {
  LSHG_CUDA(cudaFuncSetAttribute(lsh_query_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per = 0;
  LSHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lsh_query_kernel<DV>, kQThreads, smem));
  return per;
}

// Distinct-candidate slots a query on the split path: at most kSplitCap, and no more than
// 1 GiB of lists for the batch (0 = the batch takes the fused kernel).
static int split_cap(int nq) {
  const int64_t by_mem = ((int64_t)1 << 30) / (4 * (int64_t)std::max(nq, 1));
  const int cap = (int)std::min<int64_t>(kSplitCap, by_mem / 256 * 256);
  return cap >= 1024 ? cap : 0;
}

void lsh_query_plan(LshQueryArgs& a, int max_grid) {
  a.stage = (a.vec4 && !a.sketched && lsh_stage_bytes(a.d) <= (size_t)kStageMaxBytes) ? 1 : 0;
  const size_t smem = lsh_query_smem(a);
  int per = 1;
  if (smem <= 200 * 1024) {
    switch (a.dist) {
      case DIST_ANGULAR: per = lsh_ctas_per_sm<DIST_ANGULAR>(smem); break;
      case DIST_JACCARD: per = lsh_ctas_per_sm<DIST_JACCARD>(smem); break;
      default: per = lsh_ctas_per_sm<DIST_EUCLID>(smem); break;
    }
  }
  a.grid = std::max(1, std::min(std::min(max_grid, a.nq), num_sms() * std::max(1, per)));
  a.split_cap = a.stage ? split_cap(a.nq) : 0;
  a.walk_grid = 0;
  if (a.split_cap > 0) {
    constexpr int wsmem = kWalkSlots * 4;
    LSHG_CUDA(cudaFuncSetAttribute(lsh_walk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, wsmem));
    int wper = 0;
    LSHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&wper, lsh_walk_kernel, kQThreads, wsmem));
    a.walk_grid = std::max(1, std::min(a.nq, num_sms() * std::max(1, wper)));
  }
}

template <int DV>
static void launch_split(const LshQueryArgs& a, int cap, size_t fused_smem, lshg_point* out, cudaStream_t s) {
  // ctl: query counters of the walk [0], the scoring [1] and the fused kernel [2]; [3] the
  // overflow count, then the overflowing queries (the fused kernel's query list starts at [3])
  DevBuf<int> cand((size_t)a.nq * cap, s), ccnt((size_t)a.nq, s), ctl((size_t)a.nq + 4, s);
  LSHG_CUDA(cudaMemsetAsync(ctl.ptr, 0, 4 * sizeof(int), s));
  int* ovf = ctl.ptr + 3;
  lsh_walk_kernel<<<a.walk_grid, kQThreads, kWalkSlots * 4, s>>>(a, cand.ptr, cap, ccnt.ptr, ovf, ctl.ptr);
  count_launch();
  LSHG_CHECK_LAUNCH();
  const size_t ssmem = lsh_stage_bytes(a.d) + (size_t)(a.C + kQBuf) * 8 + (size_t)((a.d + 3) & ~3) * 4 + 16;
  LSHG_CUDA(cudaFuncSetAttribute(lsh_score_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssmem));
  int per = 0;
  LSHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lsh_score_kernel<DV>, kQThreads, ssmem));
  const int sgrid = std::max(1, std::min(a.nq, num_sms() * std::max(1, per)));
  lsh_score_kernel<DV><<<sgrid, kQThreads, ssmem, s>>>(a, cand.ptr, cap, ccnt.ptr, out, ctl.ptr + 1);
  count_launch();
  LSHG_CHECK_LAUNCH();
  LshQueryArgs f = a;  // queries with more than cap distinct candidates: the fused kernel
  f.qlist = ovf;
  f.bitmap_dirty = 1;
  f.qctr = ctl.ptr + 2;
  DevBuf<int> lists((size_t)a.grid * kListCap, s);
  f.lists = lists.ptr;
  LSHG_CUDA(cudaFuncSetAttribute(lsh_query_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_smem));
  lsh_query_kernel<DV><<<a.grid, kQThreads, fused_smem, s>>>(f, out);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

void launch_lsh_query(const LshQueryArgs& a, lshg_point* out, cudaStream_t s) {
  if (a.nq <= 0) return;
  LSHG_REQUIRE(a.tables <= kMaxTables, "LSH: too many tables");
  LSHG_REQUIRE(a.C >= 32 && (a.C & (a.C - 1)) == 0 && a.C >= a.k, "LSH: bad candidate count");
  LSHG_REQUIRE(!a.vec4 || (a.d % 4 == 0 && (reinterpret_cast<uintptr_t>(a.x) & 15) == 0),
               "LSH: vector row loads need 16-byte rows");
  size_t smem = lsh_query_smem(a);
  LSHG_REQUIRE(smem <= 200 * 1024, "LSH: candidate set too large for shared memory");
  ProfScope _ps("lsh_query", s);
  const int cap = a.split_cap;
  if (cap > 0) {  // exact scoring with staged rows: walk, then score (overflow: fused)
    switch (a.dist) {
      case DIST_ANGULAR: launch_split<DIST_ANGULAR>(a, cap, smem, out, s); break;
      case DIST_JACCARD: launch_split<DIST_JACCARD>(a, cap, smem, out, s); break;
      case DIST_EUCLID: launch_split<DIST_EUCLID>(a, cap, smem, out, s); break;
      default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "LSH: invalid distance function");
    }
    return;
  }
  DevBuf<int> lists((size_t)a.grid * kListCap, s), qctr(1, s);
  LSHG_CUDA(cudaMemsetAsync(qctr.ptr, 0, sizeof(int), s));
  LshQueryArgs f = a;
  f.lists = lists.ptr;
  f.qctr = qctr.ptr;
#define LSHG_LQ(DV)                                                                                        \
  do {                                                                                                     \
    LSHG_CUDA(cudaFuncSetAttribute(lsh_query_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    lsh_query_kernel<DV><<<a.grid, kQThreads, smem, s>>>(f, out);                                          \
  } while (0)
  switch (a.dist) {
    case DIST_ANGULAR: LSHG_LQ(DIST_ANGULAR); break;
    case DIST_JACCARD: LSHG_LQ(DIST_JACCARD); break;
    case DIST_EUCLID: LSHG_LQ(DIST_EUCLID); break;
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "LSH: invalid distance function");
  }
#undef LSHG_LQ
  count_launch();
  LSHG_CHECK_LAUNCH();
}

int lsh_query_grid(int nq) { return std::max(1, std::min(nq, num_sms() * kQueryCtasPerSm)); }

}  // namespace lshg
