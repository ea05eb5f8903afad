// Index build and query: the reference's host pipelines (linearScans, kernel.cu:27-55;
// runLsh, lshFramework.cuh:313-460; runSimHashLinearScan, simHash.cu:61-144;
// runWeightedMinHashLinearScan, weightedMinHash.cuh:345-429; runSimHashJLLinearScan,
// simHashJL.cuh:287-330; runMemOptimizedLinearScan, memOptimizedLinearScan.cu:129-191)
// re-expressed as one stream-ordered build that keeps base, sketches, keys and buckets
// resident, and a query that only processes the query batch.
//
// The in-place preprocessing the reference applies to data and queries together
// (normalisation, the Jaccard min shift) is recorded as a list of operations and
// replayed on every query batch, with statistics taken from the base (and, for the
// reference-compatible entry points, from the query batch it is built with).
#include <algorithm>
#include <cstring>

#include "host_rng.h"
#include "index.h"
#include "launch_count.h"
#include "tc_filter.h"

namespace lshg {

// Batches from this many queries up take the tensor-core sketch scan by default (a
// 128-query tile is the MMA's M; below this most of it would be padding).
constexpr int kTcSketchMinQueries = 64;

int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

void tile_sketches(Index& I, cudaStream_t s) {
  const int64_t tiles = (I.n + 127) / 128;
  I.xst.alloc((size_t)tiles * 128 * I.wp, s);
  launch_tile_sketches(I.xs.ptr, I.n, I.wp, I.xst.ptr, s);
  if (I.sk_kind == 4 && I.p.opt.sketch_scan != 1) {  // bit-sliced copy for the threshold-filter scan
    const int wsl = byte_slice_words(I.wp);
    DevBuf<uint32_t> sl((size_t)I.n * wsl, s);
    launch_slice_bytes(I.xs.ptr, I.n, I.wp, I.n, 0x00, sl.ptr, s);
    I.xsl.alloc((size_t)tiles * 128 * wsl, s);
    launch_tile_sketches(sl.ptr, I.n, wsl, I.xsl.ptr, s);
  }
  if (I.sk_kind == 10) {  // CWS: codes against the base's range of t, bit-sliced for the filter scan
    I.cws = cws_plan_codes(I.xs.ptr, I.n, I.cws_S, I.d, s);
    if (I.cws.pl && I.p.opt.sketch_scan != 1) {
      cws_build_dict(I.xs.ptr, I.n, I.cws_S, I.cws, I.cws_rank, s);
      const int wsl = I.cws_S / 32 * I.cws.pl;
      DevBuf<uint32_t> sl((size_t)I.n * wsl, s);
      launch_cws_slice(I.xs.ptr, I.n, I.cws_S, I.d, I.cws, false, sl.ptr, s);
      I.xsl.alloc((size_t)tiles * 128 * wsl, s);
      launch_tile_sketches(sl.ptr, I.n, wsl, I.xsl.ptr, s);
    }
  }
  if ((I.sk_kind == 3 || I.sk_kind == 5) && I.words <= 32 && I.p.opt.sketch_scan != 1) {
    const int64_t rows = (I.n + 255) / 256 * 256;
    I.xse.alloc((size_t)rows * 128 * tc::hamming_chunks(I.words), s);
    tc::launch_expand_bits(I.xs.ptr, I.n, I.wp, I.words, rows, I.xse.ptr, s);
  }
}

void launch_pack_bytes(const uint8_t* in, int64_t n, int sbytes, uint32_t* out, int wp, uint8_t pad, cudaStream_t s);
size_t wmh_state_bytes();
size_t lsh_query_smem(const LshQueryArgs& a);
int lsh_query_grid(int nq);
void lsh_query_plan(LshQueryArgs& a, int max_grid);
void launch_tc_scan(Index& idx, const float* q, int nq, int k, lshg_point* out, cudaStream_t s,
                    const RerankBounds* extra);
void tc_prepare(Index& idx, cudaStream_t s);

namespace {

template <typename T>
void upload(DevBuf<T>& b, const T* h, size_t count, cudaStream_t s) {
  b.alloc(count, s);
  if (count) LSHG_CUDA(cudaMemcpyAsync(b.ptr, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
}

void apply_op(const PrepOp& op, float* x, int64_t n, int d, cudaStream_t s) {
  if (n <= 0 || !x) return;
  if (op.kind == PrepOp::NORMALIZE) {
    launch_normalize(x, n, d, s);
  } else {
    launch_shift_abs(x, n, d, op.dminv->ptr, s);
  }
}

void apply_ops(const std::vector<PrepOp>& ops, float* x, int64_t n, int d, cudaStream_t s) {
  for (const auto& op : ops) apply_op(op, x, n, d, s);
}

// Record-and-apply helpers: the op is applied to the base and the companion.
void do_normalize(std::vector<PrepOp>& ops, float* x, int64_t n, float* comp, int nc, int d, cudaStream_t s) {
  PrepOp op{PrepOp::NORMALIZE, {}, nullptr};
  apply_op(op, x, n, d, s);
  apply_op(op, comp, nc, d, s);
  ops.push_back(op);
}

// transformData (processingUtils.cuh:12-46): shift every dimension by |min floor|,
// min taken over base and companion, starting from 0.
void do_shift(std::vector<PrepOp>& ops, float* x, int64_t n, float* comp, int nc, int d, cudaStream_t s) {
  std::vector<int> zero(d, 0);
  DevBuf<int> m;
  upload(m, zero.data(), d, s);
  launch_min_floor(x, n, d, m.ptr, s);
  if (comp && nc > 0) launch_min_floor(comp, nc, d, m.ptr, s);
  PrepOp op{PrepOp::SHIFT, std::vector<int>(d), nullptr};
  LSHG_CUDA(cudaMemcpyAsync(op.minv.data(), m.ptr, d * sizeof(int), cudaMemcpyDeviceToHost, s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  op.dminv = std::make_shared<DevBuf<int>>();
  upload(*op.dminv, op.minv.data(), d, s);
  apply_op(op, x, n, d, s);
  apply_op(op, comp, nc, d, s);
  ops.push_back(op);
}

// minHashPreprocessing + setupMaps (weightedMinHash.cuh:202-213, :71-90, :299-309) and the
// sampler tables.  H seeds; onebit: words x hashBits layout.
void wmh_prepare(WmhState& w, std::vector<PrepOp>& ops, float* x, int64_t n, float* comp, int nc, int d, int H,
                 int onebit, int words, int hashBits, cudaStream_t s) {
  do_shift(ops, x, n, comp, nc, d, s);
  do_normalize(ops, x, n, comp, nc, d, s);
  std::vector<int> zero(d, 0), bounds(d);
  DevBuf<int> mb;
  upload(mb, zero.data(), d, s);
  launch_max_ceil(x, n, d, mb.ptr, s);
  if (comp && nc > 0) launch_max_ceil(comp, nc, d, mb.ptr, s);
  LSHG_CUDA(cudaMemcpyAsync(bounds.data(), mb.ptr, d * sizeof(int), cudaMemcpyDeviceToHost, s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  int64_t M = 0;
  w.h_start.assign(d, 0);
  for (int i = 0; i < d; ++i) {
    w.h_start[i] = (int)M;
    M += std::max(0, bounds[i]);
  }
  LSHG_REQUIRE(M >= 1 && M < (1 << 24), "weighted MinHash: bad index-map size (all-zero or unnormalised data)");
  w.h_map.assign((size_t)M, 0);
  for (int i = 0; i < d; ++i)
    for (int j = w.h_start[i]; j < w.h_start[i] + std::max(0, bounds[i]); ++j) w.h_map[j] = i;
  w.M = (int)M;
  w.H = H;
  w.onebit = onebit;
  w.words = words;
  w.hashBits = hashBits;
  w.T = 1024;
  std::vector<int> seeds(H);
  for (int h = 0; h < H; ++h) seeds[h] = h * 1234 + 92138;  // createSeedArr, weightedMinHash.cuh:252-262
  std::vector<uint8_t> bm(255);
  random_bools(255, bm.data());  // generateRandomBoolVectors(255), weightedMinHash.cuh:231-250
  w.bitmapLen = 255;
  upload(w.start, w.h_start.data(), d, s);
  upload(w.map, w.h_map.data(), w.h_map.size(), s);
  upload(w.seeds, seeds.data(), H, s);
  upload(w.bitmap, bm.data(), bm.size(), s);
  w.rtab.alloc((size_t)w.T * H, s);
  w.states.alloc(wmh_state_bytes() * H, s);
  launch_wmh_tables(w.seeds.ptr, H, w.T, w.M, w.rtab.ptr, w.states.ptr, s);
  w.used = true;
}

void wmh_run(const WmhState& w, const float* x, int64_t n, int d, uint8_t* out8, uint32_t* out32, int* err,
             cudaStream_t s) {
  launch_wmh_sketch(x, n, d, w.start.ptr, w.map.ptr, w.M, w.rtab.ptr, w.states.ptr, w.H, w.T, w.onebit, w.words,
                    w.hashBits, w.bitmap.ptr, w.bitmapLen, out8, out32, err, s);
}

int log_dim(int d) {  // crossPolyTope.cuh:95-104
  int p = 1;
  while (p < d) p *= 2;
  return p;
}

void check_err_flag(int* err_dev, cudaStream_t s) {
  int e = 0;
  LSHG_CUDA(cudaMemcpyAsync(&e, err_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  if (e) throw Error(LSHG_ERR_SAMPLER_LIMIT, "weighted MinHash sampler exceeded its draw limit (zero or NaN input?)");
}

// Sketches of `rows` vectors (base or queries) for the index's sketch kind.  For packed
// kinds the result has rows of wp words; byte sketches pad with `padbyte`.
void make_sketch(const Index& idx, const float* v, int64_t rows, uint8_t padbyte, DevBuf<uint32_t>* packed,
                 DevBuf<float>* fl, int* err, cudaStream_t s) {
  const int d = idx.d;
  switch (idx.sk_kind) {
    case 3: {
      DevBuf<uint32_t> raw(rows * idx.words, s);
      if (idx.sk_split.ptr)  // tensor cores, bit-identical (exact recheck of the near-zero signs)
        tc::launch_tc_signs(v, rows, d, idx.sk_split.ptr, idx.sk_pnorm.ptr, idx.sk_planes.ptr, idx.words * 32,
                            idx.words, raw.ptr, err, s);
      else
        launch_project(v, rows, d, idx.sk_planes.ptr, idx.words * 32, 0, 32, idx.words, raw.ptr, nullptr, s);
      packed->alloc(rows * idx.wp, s);
      launch_pad_words(raw.ptr, rows, idx.words, packed->ptr, idx.wp, 0u, s);
      break;
    }
    case 4: {
      DevBuf<uint8_t> raw(rows * idx.sbytes, s);
      wmh_run(idx.wmh_sk, v, rows, d, raw.ptr, nullptr, err, s);
      packed->alloc(rows * idx.wp, s);
      launch_pack_bytes(raw.ptr, rows, idx.sbytes, packed->ptr, idx.wp, padbyte, s);
      break;
    }
    case 5: {
      DevBuf<uint32_t> raw(rows * idx.words, s);
      wmh_run(idx.wmh_sk, v, rows, d, nullptr, raw.ptr, err, s);
      packed->alloc(rows * idx.wp, s);
      launch_pad_words(raw.ptr, rows, idx.words, packed->ptr, idx.wp, 0u, s);
      break;
    }
    case 10: {
      packed->alloc(rows * idx.wp, s);
      launch_cws_sketch(v, rows, d, idx.cws_S, idx.cws_tab.ptr, packed->ptr, s);
      break;
    }
    case 6: {
      fl->alloc(rows * idx.sdim, s);
      launch_project(v, rows, d, idx.sk_planes.ptr, idx.sdim, 1, 32, 0, nullptr, fl->ptr, s);
      break;
    }
    default:
      break;
  }
}

void make_keys(const Index& idx, const float* v, int64_t rows, DevBuf<uint16_t>* keys, int* err, cudaStream_t s) {
  const int d = idx.d;
  keys->alloc(rows * idx.tables, s);
  switch (idx.key_kind) {
    case 3: {
      DevBuf<uint32_t> raw(rows * idx.tables, s);
      LSHG_CUDA(cudaMemsetAsync(raw.ptr, 0, raw.bytes(), s));
      launch_project(v, rows, d, idx.key_planes.ptr, idx.tables * idx.key_bits, 0, idx.key_bits, idx.tables, raw.ptr,
                     nullptr, s);
      launch_u32_to_u16(raw.ptr, rows * idx.tables, keys->ptr, s);
      break;
    }
    case 4: {
      DevBuf<uint8_t> raw(rows * idx.tables, s);
      wmh_run(idx.wmh_keys, v, rows, d, raw.ptr, nullptr, err, s);
      DevBuf<uint32_t> wide(rows * idx.tables, s);
      // widen u8 -> u16 through the packer: one byte per 32-bit word
      launch_pack_bytes(raw.ptr, rows * idx.tables, 1, wide.ptr, 1, 0, s);
      launch_u32_to_u16(wide.ptr, rows * idx.tables, keys->ptr, s);
      break;
    }
    case 5: {
      DevBuf<uint32_t> raw(rows * idx.tables, s);
      wmh_run(idx.wmh_keys, v, rows, d, nullptr, raw.ptr, err, s);
      launch_u32_to_u16(raw.ptr, rows * idx.tables, keys->ptr, s);
      break;
    }
    case 7:
      launch_crosspoly(v, rows, d, idx.cp_P, idx.tables, idx.cp_hashes, idx.cp_rounds, idx.cp_diag.ptr, keys->ptr, s);
      break;
    case 10: {  // CWS samples, K a table, hashed into bucketKeyBits bits
      const int S = idx.tables * idx.cp_hashes;
      DevBuf<uint32_t> smp((size_t)rows * S * 2, s);
      launch_cws_sketch(v, rows, d, S, idx.cws_key_tab.ptr, smp.ptr, s);
      launch_cws_keys(smp.ptr, rows, idx.tables, idx.cp_hashes, idx.key_bits, keys->ptr, s);
      break;
    }
    default:
      throw Error(LSHG_ERR_INVALID_ARGUMENT, "invalid keysImplementation");
  }
}

struct EventTimer {
  cudaEvent_t a, b;
  cudaStream_t s;
  explicit EventTimer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double ms() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float m = 0;
    cudaEventElapsedTime(&m, a, b);
    cudaEventRecord(a, s);
    return m;
  }
  ~EventTimer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

}  // namespace

int* Index::error_word(cudaStream_t s) {
  std::lock_guard<std::mutex> g(err_mu);
  auto it = err_words.find(s);
  if (it != err_words.end()) return it->second;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  LSHG_CUDA(cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone)
    throw Error(LSHG_ERR_INVALID_ARGUMENT,
                "first query of an index on this stream during a stream capture: run one query on the stream first");
  int* w = nullptr;
  LSHG_CUDA(cudaMalloc(&w, sizeof(int)));
  if (cudaMemsetAsync(w, 0, sizeof(int), s) != cudaSuccess) {
    cudaFree(w);
    LSHG_CUDA(cudaGetLastError());
  }
  err_words.emplace(s, w);
  return w;
}

void derive_simhash(Index& I, cudaStream_t s) {
  if (I.sk_kind != 3 || I.d > 128 || I.d < 1 || !I.sk_planes.ptr) return;
  const int P = I.words * 32;
  const int64_t ppad = (int64_t)(P + 255) / 256 * 256;
  I.sk_split.alloc((size_t)ppad * 3 * tc::signs_part_cols(I.d), s);
  I.sk_pnorm.alloc((size_t)ppad, s);
  tc::launch_split_bf16(I.sk_planes.ptr, P, I.d, ppad, 1, I.sk_split.ptr, I.sk_pnorm.ptr, s);
}

Index::~Index() {
  if (stream) cudaStreamSynchronize(stream);
  for (auto& kv : err_words) cudaFree(kv.second);  // cudaFree waits for work that may still write it
  x.release(); xnorm.release(); xt.release(); xs.release(); xse.release(); xsl.release(); xsf.release(); xsft.release();
  sk_planes.release(); sk_split.release(); sk_pnorm.release();
  keys.release(); offsets.release(); buckets.release(); key_planes.release(); cp_diag.release(); bitmaps.release();
  xbf.release(); xbf_scale.release(); xf8.release(); xnorm64.release(); xst.release(); qstats.release();
  cws_tab.release(); cws_rank.release(); cws_key_tab.release();
  for (auto* ops : {&ops_keys, &ops_sketch})
    for (auto& op : *ops)
      if (op.dminv) op.dminv->release();
  for (WmhState* w : {&wmh_sk, &wmh_keys}) {
    w->start.release(); w->map.release(); w->seeds.release(); w->rtab.release(); w->states.release(); w->bitmap.release();
  }
  if (stream) cudaStreamSynchronize(stream);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

std::unique_ptr<Index> build_index(const lshg_index_params& p, DevBuf<float>&& base, int64_t n, float* comp, int nc,
                                   cudaStream_t s, double* prep_ms, double* build_ms) {
  LSHG_REQUIRE(n >= 1 && p.d >= 1, "empty base or dimension");
  LSHG_REQUIRE(n < (int64_t)INT_MAX, "base too large for 32-bit ids");
  keep_pool_memory();
  auto idx = std::make_unique<Index>();
  Index& I = *idx;
  I.p = p;
  I.stream = s;
  cudaGetDevice(&I.device);
  I.n = n;
  I.d = p.d;
  I.x = std::move(base);
  const int d = p.d;
  const int impl = p.implementation == 1 ? 2 : p.implementation;
  const int tqs = p.opt.thread_queue_size > 0 ? p.opt.thread_queue_size : 128;
  int C = p.opt.candidates > 0 ? p.opt.candidates : 32 * tqs;
  I.C = std::min(4096, std::max(32, next_pow2(C)));
  DevBuf<int> err(1, s);
  LSHG_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), s));
  I.qstats.alloc(2, s);
  LSHG_CUDA(cudaMemsetAsync(I.qstats.ptr, 0, I.qstats.bytes(), s));
  EventTimer tm(s);
  double prep = 0, build = 0;
  float* X = I.x.ptr;

  LSHG_REQUIRE(impl == 2 || impl == 3 || impl == 4 || impl == 5 || impl == 6 || impl == 8 || impl == 9 || impl == 10,
               "Invalid implementation selected");
  LSHG_REQUIRE(p.framework == 0 || p.framework == 1, "framework must be 0 (linear scan) or 1 (LSH)");

  if (p.framework == 0) {
    switch (impl) {
      case 2:
      case 8:
      case 9:
        I.dist = p.distanceFunc;
        LSHG_REQUIRE(I.dist >= 1 && I.dist <= 3, "Invalid operation selected for distance function");
        if (I.dist == DIST_JACCARD) {  // memOptimizedLinearScan.cu:149-163
          do_shift(I.ops_sketch, X, n, comp, nc, d, s);
          do_normalize(I.ops_sketch, X, n, comp, nc, d, s);
        }
        break;
      case 3:
        I.dist = DIST_ANGULAR;  // simHash.cu:19
        break;
      case 4:
      case 5:
        I.dist = DIST_JACCARD;  // weightedMinHash.cuh:28
        break;
      case 10:  // the weighted MinHash preprocessing (processingUtils.cuh:12-67), then CWS samples
        I.dist = DIST_JACCARD;
        do_shift(I.ops_sketch, X, n, comp, nc, d, s);
        do_normalize(I.ops_sketch, X, n, comp, nc, d, s);
        break;
      case 6:
        I.dist = DIST_ANGULAR;  // candidateSetScan(..., 1), sketchedDistanceScanners.cuh:168
        do_normalize(I.ops_sketch, X, n, comp, nc, d, s);  // simHashJL.cuh:298
        break;
    }
  } else {
    I.dist = p.distanceFunc;
    LSHG_REQUIRE(I.dist >= 1 && I.dist <= 3, "Invalid operation selected for distance function");
    LSHG_REQUIRE(impl != 8 && impl != 9, "the tensor-core scan is a linear scan");
    LSHG_REQUIRE(impl != 10, "consistent weighted sampling is a linear-scan sketch");
    LSHG_REQUIRE(p.tables >= 1 && p.tables <= 256, "tables must be in [1, 256]");
    LSHG_REQUIRE(p.bucketKeyBits >= 1 && p.bucketKeyBits <= 24, "bucketKeyBits must be in [1, 24]");
    I.tables = p.tables;
    I.key_bits = p.bucketKeyBits;
    I.tableSize = 1 << p.bucketKeyBits;
    I.key_kind = p.keysImplementation;
    switch (I.key_kind) {
      case 3: {
        std::vector<float> R((size_t)p.tables * d * p.bucketKeyBits);
        random_normals((int64_t)R.size(), 1.0, R.data());
        upload(I.key_planes, R.data(), R.size(), s);
        break;
      }
      case 4:
        LSHG_REQUIRE(I.tableSize >= 256, "byte weighted-MinHash keys need bucketKeyBits >= 8");
        wmh_prepare(I.wmh_keys, I.ops_keys, X, n, comp, nc, d, p.tables, 0, 0, 0, s);
        break;
      case 5:
        LSHG_REQUIRE(p.bucketKeyBits <= 32, "one-bit weighted-MinHash keys need bucketKeyBits <= 32");
        wmh_prepare(I.wmh_keys, I.ops_keys, X, n, comp, nc, d, p.tables * p.bucketKeyBits, 1, p.tables,
                    p.bucketKeyBits, s);
        break;
      case 10: {  // consistent weighted sampling keys, K = cp_hashes samples a table
        LSHG_REQUIRE(p.bucketKeyBits <= 16, "CWS keys need bucketKeyBits <= 16");
        LSHG_REQUIRE(d <= 4096, "CWS keys: d must be <= 4096");
        I.cp_hashes = p.opt.cp_hashes > 0 ? p.opt.cp_hashes : 1;
        LSHG_REQUIRE(I.cp_hashes <= 16, "CWS keys: at most 16 samples a table");
        do_shift(I.ops_keys, X, n, comp, nc, d, s);  // the weighted MinHash preprocessing
        do_normalize(I.ops_keys, X, n, comp, nc, d, s);
        std::vector<float> tab;
        cws_tables(d, p.tables * I.cp_hashes, tab, kCwsKeySeed);
        upload(I.cws_key_tab, tab.data(), tab.size(), s);
        break;
      }
      case 7: {
        I.cp_P = log_dim(d);
        I.cp_hashes = p.opt.cp_hashes > 0 ? p.opt.cp_hashes : 1;
        I.cp_rounds = p.opt.cp_rounds > 0 ? p.opt.cp_rounds : 3;
        int64_t range = 1;
        for (int h = 0; h < I.cp_hashes; ++h) range *= 2 * I.cp_P;
        LSHG_REQUIRE(range <= 65536 && range <= I.tableSize,
                     "cross-polytope key range (2P)^hashes exceeds the table size or 16 bits");
        do_normalize(I.ops_keys, X, n, comp, nc, d, s);  // crossPolyTope.cuh:111
        std::vector<int32_t> D((size_t)I.cp_P * p.tables * I.cp_hashes * I.cp_rounds);
        random_plus_minus((int64_t)D.size(), D.data());
        upload(I.cp_diag, D.data(), D.size(), s);
        break;
      }
      default:
        throw Error(LSHG_ERR_INVALID_ARGUMENT, "Invalid implementation selected for LSH.");
    }
  }
  prep += tm.ms();

  // keys + buckets
  if (p.framework == 1) {
    make_keys(I, X, n, &I.keys, err.ptr, s);
    I.offsets.alloc((size_t)I.tables * I.tableSize, s);
    I.buckets.alloc((size_t)I.tables * n, s);
    DevBuf<int> cursors((size_t)I.tables * I.tableSize, s);
    launch_lsh_build(I.keys.ptr, n, I.tables, I.tableSize, I.offsets.ptr, I.buckets.ptr, cursors.ptr, s);
  }

  // sketches (generateHashes(isHashKeys = false), lshFramework.cuh:391)
  const bool want_sketch = (impl >= 3 && impl <= 6) || (p.framework == 0 && impl == 10);
  if (want_sketch) {
    LSHG_REQUIRE(p.sketchDim >= 1, "sketchDim must be >= 1");
    I.sk_kind = impl;
    switch (impl) {
      case 3: {
        I.words = p.sketchDim;
        LSHG_REQUIRE(I.words <= 64, "SimHash sketchDim must be <= 64 words");
        I.wp = (I.words + 3) / 4 * 4;
        std::vector<float> R((size_t)d * 32 * p.sketchDim);
        random_normals((int64_t)R.size(), 1.0, R.data());  // simHash.cu:73 / lshFramework.cuh:24-27
        upload(I.sk_planes, R.data(), R.size(), s);
        derive_simhash(I, s);
        break;
      }
      case 4:
        I.sbytes = p.sketchDim;
        I.words = (p.sketchDim + 3) / 4;
        I.wp = (I.words + 3) / 4 * 4;
        LSHG_REQUIRE(I.wp <= 64, "byte weighted-MinHash sketchDim must be <= 256");
        wmh_prepare(I.wmh_sk, I.ops_sketch, X, n, comp, nc, d, p.sketchDim, 0, 0, 0, s);
        break;
      case 5:
        I.words = p.sketchDim;
        I.wp = (I.words + 3) / 4 * 4;
        LSHG_REQUIRE(I.wp <= 64, "one-bit weighted-MinHash sketchDim must be <= 64 words");
        wmh_prepare(I.wmh_sk, I.ops_sketch, X, n, comp, nc, d, p.sketchDim * 32, 1, p.sketchDim, 32, s);
        break;
      case 10: {
        LSHG_REQUIRE(p.sketchDim >= 32 && p.sketchDim <= 256 && p.sketchDim % 32 == 0,
                     "CWS sketchDim (samples) must be a multiple of 32 in [32, 256]");
        LSHG_REQUIRE(d <= 4096, "CWS: d must be <= 4096");
        I.cws_S = p.sketchDim;
        I.words = 2 * p.sketchDim;
        I.wp = I.words;
        std::vector<float> tab;
        cws_tables(d, I.cws_S, tab);
        upload(I.cws_tab, tab.data(), tab.size(), s);
        break;
      }
      case 6: {
        I.sdim = p.sketchDim;
        if (p.framework == 1) do_normalize(I.ops_sketch, X, n, comp, nc, d, s);  // runGenericJL, simHashJL.cuh:254
        std::vector<float> R((size_t)p.sketchDim * d);
        random_normals((int64_t)R.size(), 1.0 / p.sketchDim, R.data());  // randomVectorGenerator.cpp:56-74
        upload(I.sk_planes, R.data(), R.size(), s);
        break;
      }
    }
    DevBuf<uint32_t> packed;
    DevBuf<float> fl;
    make_sketch(I, X, n, 0x00, &packed, &fl, err.ptr, s);
    if (impl == 6) {
      I.xsf = std::move(fl);
      I.xsft.alloc((size_t)ceil_div(n, 128) * 128 * I.sdim, s);
      launch_tile_transpose(I.xsf.ptr, n, I.sdim, I.xsft.ptr, s);
    } else {
      I.xs = std::move(packed);
      if (p.framework == 0) tile_sketches(I, s);
    }
  }

  // exact-distance arrays
  if (I.dist == DIST_ANGULAR) {
    I.xnorm.alloc(n, s);
    launch_row_norms(X, n, d, I.xnorm.ptr, s);
  }
  if (p.framework == 0 && impl == 2) {
    I.xt.alloc((size_t)ceil_div(n, 128) * 128 * d, s);
    launch_tile_transpose(X, n, d, I.xt.ptr, s);
  }
  if (p.framework == 0 && (impl == 8 || impl == 9)) tc_prepare(I, s);
  if (p.framework == 1) I.lsh_grid = lsh_query_grid(1 << 30);
  check_err_flag(err.ptr, s);
  build += tm.ms();
  if (prep_ms) *prep_ms = prep;
  if (build_ms) *build_ms = build;
  return idx;
}

void sketch_queries(Index& I, float* q, int nq, DevBuf<uint32_t>* qs, DevBuf<float>* qsf, DevBuf<uint16_t>* qkeys,
                    cudaStream_t s) {
  int* err = I.error_word(s);
  apply_ops(I.ops_keys, q, nq, I.d, s);
  if (I.p.framework == 1 && qkeys) make_keys(I, q, nq, qkeys, err, s);
  apply_ops(I.ops_sketch, q, nq, I.d, s);
  if (I.sk_kind) make_sketch(I, q, nq, 0xff, qs, qsf, err, s);
}

void check_device(const Index& I) {
  int dev = -1;
  LSHG_CUDA(cudaGetDevice(&dev));
  if (dev != I.device)
    throw Error(LSHG_ERR_INVALID_ARGUMENT, "the index lives on device " + std::to_string(I.device) +
                                               " but the calling thread's current device is " + std::to_string(dev));
}

void query_error(Index& I, cudaStream_t s) {
  int e = 0;
  int* w = I.error_word(s);
  LSHG_CUDA(cudaMemcpyAsync(&e, w, sizeof(int), cudaMemcpyDeviceToHost, s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  if (e) {
    LSHG_CUDA(cudaMemsetAsync(w, 0, sizeof(int), s));
    if (e == 2) throw Error(LSHG_ERR_TIMEOUT, "tensor-core scan: a pipeline wait timed out (kernel aborted)");
    if (e == 3) throw Error(LSHG_ERR_TIMEOUT, "a row-copy wait timed out (the rows were re-read directly)");
    throw Error(LSHG_ERR_SAMPLER_LIMIT, "weighted MinHash sampler exceeded its draw limit (zero or NaN query?)");
  }
}

void query_index(Index& I, float* q, int nq, int k, lshg_point* out, cudaStream_t s, const RerankBounds* extra) {
  LSHG_REQUIRE(k >= 1 && k <= 4096, "k must be in [1, 4096]");
  if (nq <= 0) return;
  const int impl = I.p.implementation == 1 ? 2 : I.p.implementation;
  DevBuf<uint32_t> qs;
  DevBuf<float> qsf;
  DevBuf<uint16_t> qkeys;
  sketch_queries(I, q, nq, &qs, &qsf, &qkeys, s);
  DevBuf<float> qnorm;
  if (I.dist == DIST_ANGULAR) {
    qnorm.alloc(nq, s);
    launch_row_norms(q, nq, I.d, qnorm.ptr, s);
  }
  const int kp = std::max(32, next_pow2(k));
  if (I.p.framework == 1) {
    LshQueryArgs a{};
    a.qkeys = qkeys.ptr;
    a.nq = nq;
    a.tables = I.tables;
    a.tableSize = I.tableSize;
    a.n = I.n;
    a.offsets = I.offsets.ptr;
    a.buckets = I.buckets.ptr;
    a.x = I.x.ptr;
    a.xnorm = I.xnorm.ptr;
    a.q = q;
    a.qnorm = qnorm.ptr;
    a.d = I.d;
    a.dist = I.dist;
    a.sketched = (I.p.runWithSketchedData && I.sk_kind) ? 1 : 0;
    a.sketch_kind = I.sk_kind;
    a.xs = I.xs.ptr;
    a.qs = qs.ptr;
    a.wp = I.wp;
    a.words = I.words;
    a.sbytes = I.sbytes;
    a.xsf = I.xsf.ptr;
    a.qsf = qsf.ptr;
    a.sdim = I.sdim;
    a.C = a.sketched ? std::max(I.C, kp) : kp;
    a.k = k;
    a.vec4 = (I.d % 4 == 0 && (reinterpret_cast<uintptr_t>(I.x.ptr) & 15) == 0) ? 1 : 0;
    lsh_query_plan(a, I.lsh_grid);  // staging choice and grid (resident CTAs)
    // per-call dedupe bitmaps of the fused kernel: concurrent queries on one index never
    // share them (on the split path the fused kernel only answers overflowing queries and
    // zeroes a bitmap itself when it gets one)
    DevBuf<uint32_t> bm((size_t)a.grid * ((I.n + 31) / 32), s);
    if (a.split_cap == 0) LSHG_CUDA(cudaMemsetAsync(bm.ptr, 0, bm.bytes(), s));
    a.bitmaps = bm.ptr;
    a.stats = I.qstats.ptr;
    a.err = I.error_word(s);
    launch_lsh_query(a, out, s);
    return;
  }
  if (impl == 8 || impl == 9) {
    launch_tc_scan(I, q, nq, k, out, s, extra);
    return;
  }
  if (impl == 2) {
    const int C = kp;
    int splits = scan_float_splits(I.n, nq, C);
    DevBuf<uint64_t> part((size_t)nq * splits * C, s);
    launch_scan_float(I.xt.ptr, I.n, I.d, I.xnorm.ptr, q, nq, qnorm.ptr, I.dist, C, splits, part.ptr, s);
    const uint64_t* keys = part.ptr;
    DevBuf<uint64_t> merged;
    if (splits > 1) {
      merged.alloc((size_t)nq * C, s);
      launch_merge_splits(part.ptr, nq, splits, C, merged.ptr, s);
      keys = merged.ptr;
    }
    launch_keys_to_points(keys, nq, C, k, out, s);
    return;
  }
  const int C = std::max(I.C, kp);
  DevBuf<uint64_t> part;
  int splits;
  if (impl == 10) {  // CWS: the exact top-C by (1 - matches / S, id), then the generalized-Jaccard re-rank
    part.alloc((size_t)nq * C, s);
    launch_cws_scan(I.cws.pl ? I.xsl.ptr : nullptr, I.xst.ptr, I.n, I.cws_S, I.d, I.cws, qs.ptr, nq, C, part.ptr,
                    I.error_word(s), s);
    launch_rerank(part.ptr, nq, C, I.x.ptr, I.n, I.d, I.xnorm.ptr, q, qnorm.ptr, I.dist, k, out, s, I.error_word(s),
                  I.p.opt.fp64_recheck > 0, nullptr, extra);
    return;
  }
  if (impl == 6) {
    splits = scan_float_splits(I.n, nq, C);
    part.alloc((size_t)nq * splits * C, s);
    launch_scan_float(I.xsft.ptr, I.n, I.sdim, nullptr, qsf.ptr, nq, nullptr, DIST_SQEUCLID, C, splits, part.ptr, s);
  } else {
    const int op = impl == 3 ? OP_HAMMING : (impl == 4 ? OP_BYTE_JACCARD : OP_ONEBIT_JACCARD);
    const int mode = I.p.opt.sketch_scan;
    if (I.xse.ptr && (mode == 2 || (mode == 0 && nq >= kTcSketchMinQueries)) && tc::plan_hamming(I.n, C).ok) {
      // tensor cores: the exact top-C by (sketch distance, id), then the same re-rank
      part.alloc((size_t)nq * C, s);
      tc::launch_tc_hamming(I.xse.ptr, I.n, I.xst.ptr, I.wp, I.words, qs.ptr, nq, op, C, part.ptr, I.error_word(s), s);
      launch_rerank(part.ptr, nq, C, I.x.ptr, I.n, I.d, I.xnorm.ptr, q, qnorm.ptr, I.dist, k, out, s, I.error_word(s),
                    I.p.opt.fp64_recheck > 0, nullptr, extra);
      return;
    }
    int fs = 0, fr = 0, fc = 0;
    if (I.xsl.ptr && C > 128 && (mode == 2 || (mode == 0 && nq >= kTcSketchMinQueries)) &&
        byte_filter_plan(I.n, C, &fs, &fr, &fc)) {
      // byte samples: bit-sliced threshold filter, the exact top-C, then the same re-rank
      part.alloc((size_t)nq * C, s);
      launch_byte_filter_scan(I.xsl.ptr, I.xst.ptr, I.n, I.wp, I.sbytes, qs.ptr, nq, C, part.ptr, I.error_word(s), s);
      launch_rerank(part.ptr, nq, C, I.x.ptr, I.n, I.d, I.xnorm.ptr, q, qnorm.ptr, I.dist, k, out, s, I.error_word(s),
                    I.p.opt.fp64_recheck > 0, nullptr, extra);
      return;
    }
    splits = scan_bits_splits(I.n, nq, C);
    part.alloc((size_t)nq * splits * C, s);
    launch_scan_bits(I.xst.ptr, I.n, I.wp, I.words, I.sbytes, qs.ptr, nq, op, C, splits, part.ptr, s);
  }
  const uint64_t* cand = part.ptr;
  DevBuf<uint64_t> merged;
  if (splits > 1) {
    merged.alloc((size_t)nq * C, s);
    launch_merge_splits(part.ptr, nq, splits, C, merged.ptr, s);
    cand = merged.ptr;
  }
  launch_rerank(cand, nq, C, I.x.ptr, I.n, I.d, I.xnorm.ptr, q, qnorm.ptr, I.dist, k, out, s, I.error_word(s),
                I.p.opt.fp64_recheck > 0, nullptr, extra);
}

}  // namespace lshg
