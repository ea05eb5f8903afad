// (K,L) LSH bucket tables and bucket-gather query (lshFramework.cuh:102-280).
//
// Build (same three steps as the reference): per-table key histogram; exclusive scan into
// absolute offsets where table t's region starts at t*N (buildHashBucketIndexes,
// :115-124 -- done here by one CTA per table instead of one serial thread); scatter of
// point ids with atomic cursors (:126-140).  Order inside a bucket is the atomic order,
// as in the reference; nothing downstream depends on it and exports sort it.
//
// Query (scan, :142-252 + removeDuplicates, :255-280): one CTA per query gathers the
// ids of its L buckets (bucket t ends at the next key's offset, or at the table's end
// for the last key, :183-184), drops repeats with a shared-memory id set backed by a
// per-CTA bitmap (the reference keeps repeats in its queue and removes adjacent equal
// ids after sorting), scores each distinct candidate exactly or by sketch, keeps the
// best C by (distance, id), and for sketched scoring re-ranks them exactly
// (candidateSetScan, :236-238) before writing the first k.  Fewer than k distinct
// candidates leave (-1, INT_MAX) entries.
#include "common.cuh"
#include "distance.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "profile.h"
#include "select.cuh"

namespace lshg {

namespace {

constexpr int kQThreads = 256;
constexpr int kQBuf = 2 * kQThreads;
constexpr int kMaxTables = 256;
constexpr int kHashBits = 13;                 // shared dedupe set: 8192 ids (32 KB)
constexpr int kHashSlots = 1 << kHashBits;
constexpr int kProbe = 32;                    // linear-probe limit before the global bitmap
constexpr int kUnroll = 4;                    // bucket entries a thread loads per round
constexpr int kRound = kUnroll * kQThreads;   // entries walked per round
constexpr int kScoreAt = 1024;                // score the distinct list once it holds this many
constexpr int kListCap = kScoreAt + kRound;   // a round adds at most kRound ids

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

// Dedupe of one query's bucket entries: a shared-memory open-addressing set of ids
// (linear probing, at most kProbe slots, filled monotonically within the query), and the
// CTA's global bitmap for ids whose probe run is full.  An id found in its probe run is
// never sent to the bitmap, and an id whose run is full can no longer enter the set, so
// every distinct id is reported new exactly once.
__device__ __forceinline__ bool dedupe_new(int* hash, uint32_t* bitmap, int id, int* bm_used) {
  const uint32_t h = ((uint32_t)id * 0x9E3779B1u) >> (32 - kHashBits);
  for (int p = 0; p < kProbe; ++p) {
    int* slot = hash + ((h + p) & (kHashSlots - 1));
    const int v = *reinterpret_cast<volatile int*>(slot);
    if (v == id) return false;
    if (v == -1) {
      const int old = atomicCAS(slot, -1, id);
      if (old == -1) return true;
      if (old == id) return false;
    }
  }
  *bm_used = 1;
  const uint32_t bit = 1u << (id & 31);
  return !(atomicOr(&bitmap[id >> 5], bit) & bit);
}

// Exact distance of a 16-byte-aligned row held as d4 float4s: the same operations in the
// same order as exact_distance, with the row fetched eight float4s at a time.
template <int DIST>
__device__ __forceinline__ float exact_distance_v4(const float4* __restrict__ xr, const float4* qr, int d4, float qn,
                                                   float xn) {
  float acc = 0.0f, mx = 0.0f;
  for (int j0 = 0; j0 < d4; j0 += 8) {
    float4 xv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) xv[u] = j0 + u < d4 ? __ldg(xr + j0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      if (j0 + u >= d4) break;
      const float4 qv = qr[j0 + u];
      const float xs[4] = {xv[u].x, xv[u].y, xv[u].z, xv[u].w};
      const float qs[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (DIST == DIST_ANGULAR) {
          acc = __fmaf_rn(qs[e], xs[e], acc);
        } else if (DIST == DIST_JACCARD) {
          acc = __fadd_rn(acc, fminf(xs[e], qs[e]));
          mx = __fadd_rn(mx, fmaxf(xs[e], qs[e]));
        } else {
          const float df = __fsub_rn(qs[e], xs[e]);
          acc = __fmaf_rn(df, df, acc);
        }
      }
    }
  }
  if (DIST == DIST_ANGULAR) return __fsub_rn(1.0f, __fdiv_rn(acc, __fmul_rn(qn, xn)));
  if (DIST == DIST_JACCARD) return __fsub_rn(1.0f, __fdiv_rn(acc, mx));
  return DIST == DIST_EUCLID ? __fsqrt_rn(acc) : acc;
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

// One CTA answers queries qi = blockIdx.x, +gridDim.x, ...  Per query: (1) the bucket
// entries are walked kUnroll per thread per round, deduplicated, and distinct ids appended
// to a shared list; (2) whenever the list holds kScoreAt ids (and after the last round)
// they are scored, one thread per candidate, and offered to the top-C queue.  Scoring
// order does not matter: keys (distance, id) are unique, so the kept set is the same.
template <int DIST>
__global__ void __launch_bounds__(kQThreads, 4) lsh_query_kernel(LshQueryArgs a, lshg_point* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* kept = reinterpret_cast<uint64_t*>(smem);
  uint64_t* buf = kept + a.C;
  uint64_t* rk = buf + kQBuf;  // re-rank keys [C]
  int* hash = reinterpret_cast<int*>(rk + a.C);
  int* list = hash + kHashSlots;
  float* qr = reinterpret_cast<float*>(list + kListCap);
  const int dpad = (a.d + 3) & ~3;
  float* qsf = qr + dpad;
  uint32_t* qsk = reinterpret_cast<uint32_t*>(qsf + (a.sketch_kind == 6 ? a.sdim : 0));
  __shared__ int bstart[kMaxTables], pref[kMaxTables + 1];
  __shared__ int cnt_s, bm_used_s;
  __shared__ int rcnt[3];  // ids appended per round, cycled: round r uses rcnt[r % 3]
  __shared__ uint64_t thr_s;
  TopCShared S{kept, buf, &cnt_s, &thr_s, a.C, kQBuf};
  uint32_t* bitmap = a.bitmaps + (int64_t)blockIdx.x * ((a.n + 31) / 32);
  const int tid = threadIdx.x;

  for (int qi = blockIdx.x; qi < a.nq; qi += gridDim.x) {
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
    for (int i = tid; i < kHashSlots; i += kQThreads) hash[i] = -1;
    topc_init(S, 1);
    if (tid == 0) {
      rcnt[0] = rcnt[1] = rcnt[2] = 0;
      bm_used_s = 0;
    }
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
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        if (ids[u] >= 0 && dedupe_new(hash, bitmap, ids[u], &bm_used_s))
          list[lbase + atomicAdd(&rcnt[r % 3], 1)] = ids[u];
      }
      __syncthreads();
      const int nl = lbase + rcnt[r % 3];  // uniform: rcnt[r % 3] is not written again before round r+3
      if (nl < kScoreAt && base + kRound < total) {
        lbase = nl;
        continue;
      }
      for (int i0 = 0; i0 < nl; i0 += kQThreads) {
        const int i = i0 + tid;
        if (i < nl) {
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
        topc_flush(S, 1, kQBuf - kQThreads);
        thr = thr_s;
      }
      distinct += nl;
      lbase = 0;  // the list is reused: topc_flush's last barrier follows every read of it
    }
    topc_flush(S, 1, 0);
    if (a.stats && tid == 0) {
      atomicAdd(a.stats, (unsigned long long)total);
      atomicAdd(a.stats + 1, (unsigned long long)distinct);
    }
    if (bm_used_s) {  // clear the bitmap words this query set (rare: a probe run was full)
      for (int idx = tid; idx < total; idx += kQThreads) {
        const int t = entry_table(pref, a.tables, idx);
        const int id = a.buckets[bstart[t] + (idx - pref[t])];
        bitmap[id >> 5] = 0u;
      }
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

size_t lsh_query_smem(const LshQueryArgs& a) {
  return (size_t)(2 * a.C + kQBuf) * 8 + (size_t)(kHashSlots + kListCap) * 4 + (size_t)((a.d + 3) & ~3) * 4 +
         (size_t)(a.sketch_kind == 6 ? a.sdim : 0) * 4 + (size_t)a.wp * 4 + 16;
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
#define LSHG_LQ(DV)                                                                                        \
  do {                                                                                                     \
    LSHG_CUDA(cudaFuncSetAttribute(lsh_query_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    lsh_query_kernel<DV><<<a.grid, kQThreads, smem, s>>>(a, out);                                          \
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

int lsh_query_grid(int nq) { return std::max(1, std::min(nq, num_sms() * 4)); }

}  // namespace lshg
