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
// for the last key, :183-184), drops repeats with a per-CTA bitmap (the reference keeps
// repeats in its queue and removes adjacent equal ids after sorting), scores each
// distinct candidate exactly or by sketch, keeps the best C by (distance, id), and for
// sketched scoring re-ranks them exactly (candidateSetScan, :236-238) before writing
// the first k.  Fewer than k distinct candidates leave (-1, INT_MAX) entries.
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

template <int DIST>
__global__ void __launch_bounds__(kQThreads) lsh_query_kernel(LshQueryArgs a, lshg_point* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* kept = reinterpret_cast<uint64_t*>(smem);
  uint64_t* buf = kept + a.C;
  uint64_t* rk = buf + kQBuf;  // re-rank keys [C]
  float* qr = reinterpret_cast<float*>(rk + a.C);
  float* qsf = qr + a.d;
  uint32_t* qsk = reinterpret_cast<uint32_t*>(qsf + (a.sketch_kind == 6 ? a.sdim : 0));
  __shared__ int bstart[kMaxTables], pref[kMaxTables + 1];
  __shared__ int cnt_s;
  __shared__ uint64_t thr_s;
  TopCShared S{kept, buf, &cnt_s, &thr_s, a.C, kQBuf};
  uint32_t* bitmap = a.bitmaps + (int64_t)blockIdx.x * ((a.n + 31) / 32);

  for (int qi = blockIdx.x; qi < a.nq; qi += gridDim.x) {
    for (int j = threadIdx.x; j < a.d; j += blockDim.x) qr[j] = a.q[(int64_t)qi * a.d + j];
    if (a.sketched) {
      if (a.sketch_kind == 6) {
        for (int j = threadIdx.x; j < a.sdim; j += blockDim.x) qsf[j] = a.qsf[(int64_t)qi * a.sdim + j];
      } else {
        for (int j = threadIdx.x; j < a.wp; j += blockDim.x) qsk[j] = a.qs[(int64_t)qi * a.wp + j];
      }
    }
    for (int t = threadIdx.x; t < a.tables; t += blockDim.x) {
      int key = a.qkeys[(int64_t)qi * a.tables + t];
      int st = 0, en = 0;  // a key outside the table addresses no bucket
      if (key < a.tableSize) {
        st = a.offsets[(int64_t)t * a.tableSize + key];
        en = (key >= a.tableSize - 1) ? (int)(t * a.n + a.n) : a.offsets[(int64_t)t * a.tableSize + key + 1];
      }
      bstart[t] = st;
      pref[t + 1] = en - st;
    }
    topc_init(S, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      pref[0] = 0;
      for (int t = 0; t < a.tables; ++t) pref[t + 1] += pref[t];
    }
    __syncthreads();
    const float qn = (DIST == DIST_ANGULAR) ? a.qnorm[qi] : 1.0f;
    const int total = pref[a.tables];
    uint64_t thr = kEmptyKey;
    for (int base = 0; base < total; base += blockDim.x) {
      int idx = base + threadIdx.x;
      if (idx < total) {
        int lo = 0, hi = a.tables;  // find t with pref[t] <= idx < pref[t+1]
        while (hi - lo > 1) {
          int mid = (lo + hi) >> 1;
          if (pref[mid] <= idx) lo = mid; else hi = mid;
        }
        int id = a.buckets[bstart[lo] + (idx - pref[lo])];
        uint32_t bit = 1u << (id & 31);
        uint32_t old = atomicOr(&bitmap[id >> 5], bit);
        if (!(old & bit)) {
          float dist = a.sketched ? sketch_distance<DIST>(a, id, qsk, qsf)
                                  : exact_distance<DIST>(a.x + (int64_t)id * a.d, qr, a.d, qn,
                                                         DIST == DIST_ANGULAR ? a.xnorm[id] : 1.0f);
          topc_push(S, 0, make_key(dist, id), thr);
        }
      }
      topc_flush(S, 1, kQBuf - kQThreads);
      thr = thr_s;
    }
    topc_flush(S, 1, 0);
    // clear this query's bitmap words
    for (int base = 0; base < total; base += blockDim.x) {
      int idx = base + threadIdx.x;
      if (idx < total) {
        int lo = 0, hi = a.tables;
        while (hi - lo > 1) {
          int mid = (lo + hi) >> 1;
          if (pref[mid] <= idx) lo = mid; else hi = mid;
        }
        int id = a.buckets[bstart[lo] + (idx - pref[lo])];
        bitmap[id >> 5] = 0u;
      }
    }
    const uint64_t* fin = kept;
    if (a.sketched) {
      for (int i = threadIdx.x; i < a.C; i += blockDim.x) {
        uint64_t kin = kept[i];
        uint64_t ko = kEmptyKey;
        if (kin != kEmptyKey) {
          int id = key_id(kin);
          ko = make_key(exact_distance<DIST>(a.x + (int64_t)id * a.d, qr, a.d, qn,
                                             DIST == DIST_ANGULAR ? a.xnorm[id] : 1.0f), id);
        }
        rk[i] = ko;
      }
      __syncthreads();
      block_bitonic_sort(rk, a.C);
      fin = rk;
    }
    for (int i = threadIdx.x; i < a.k; i += blockDim.x) {
      uint64_t kk = i < a.C ? fin[i] : kEmptyKey;
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
  return (size_t)(2 * a.C + kQBuf) * 8 + (size_t)a.d * 4 + (size_t)(a.sketch_kind == 6 ? a.sdim : 0) * 4 +
         (size_t)a.wp * 4 + 16;
}

void launch_lsh_query(const LshQueryArgs& a, lshg_point* out, cudaStream_t s) {
  if (a.nq <= 0) return;
  LSHG_REQUIRE(a.tables <= kMaxTables, "LSH: too many tables");
  LSHG_REQUIRE(a.C >= 32 && (a.C & (a.C - 1)) == 0 && a.C >= a.k, "LSH: bad candidate count");
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
