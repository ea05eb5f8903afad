// Resident index: the reference's pipelines (linearScans / runLsh) split into a build
// step that leaves every derived array in HBM and a query step that only touches the
// query batch.
#pragma once

#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace lshg {

// In-place transformation applied to the base (and replayed on queries), in the order
// the reference applies them to both arrays.
struct PrepOp {
  enum Kind { NORMALIZE = 0, SHIFT = 1 } kind;
  std::vector<int> minv;                 // SHIFT: per-dimension min of floor (shift is |minv|)
  std::shared_ptr<DevBuf<int>> dminv;    // device copy, so replay needs no host upload
};

// Weighted MinHash sampler state (weightedMinHash.cuh:345-468).
struct WmhState {
  bool used = false;
  int M = 0;
  int H = 0, T = 0;
  int onebit = 0, words = 0, hashBits = 0;
  DevBuf<int> start, map, seeds;
  DevBuf<float> rtab;
  DevBuf<unsigned char> states;
  DevBuf<uint8_t> bitmap;
  int bitmapLen = 255;
  std::vector<int> h_start, h_map;  // kept for export / persistence
};

struct Index {
  lshg_index_params p{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t n = 0;
  int d = 0;

  // base rows after preprocessing, magnitudes, and the 128-point tile layout
  DevBuf<float> x, xnorm, xt;
  int dist = DIST_ANGULAR;  // exact / re-rank distance
  int C = 0;                // candidate count for sketched scans

  std::vector<PrepOp> ops_keys;    // applied before keys are computed
  std::vector<PrepOp> ops_sketch;  // applied after keys, before sketches

  // sketches: kind 0 none, 3 SimHash, 4 byte WMH, 5 one-bit WMH, 6 JL, 10 CWS
  int sk_kind = 0;
  int words = 0, wp = 0, sbytes = 0, sdim = 0;
  DevBuf<uint32_t> xs;       // packed sketches, rows of wp words
  DevBuf<uint32_t> xst;      // linear scans: the same, tiled [ceil(N/128)][wp/4][128] x 16 B
  DevBuf<uint32_t> xsl;      // byte samples (kind 4) or CWS codes (kind 10) bit-sliced and tiled
                             // like xst, for the threshold-filter scan (derived, not stored)
  DevBuf<uint8_t> xse;       // tensor-core sketch scans: sketch bits as E4M3 +-1 rows,
                             // [ceil(n/256)*256][128 * ceil(words/4)] (derived, not stored)
  DevBuf<float> xsf, xsft;   // JL sketches [n][sdim] and their tile layout
  DevBuf<float> sk_planes;   // SimHash planes [32*sketchDim][d] or JL rows [sdim][d]
  DevBuf<uint16_t> sk_split; // SimHash planes split into BF16 [hi | lo | hi] rows for the
                             // tensor-core projection (d <= 128; derived, not stored)
  DevBuf<float> sk_pnorm;    // their norms, rows padded to 256
  WmhState wmh_sk;
  int cws_S = 0;             // CWS samples a vector; xs rows are S (index, t) int32 pairs
  DevBuf<float> cws_tab;     // CWS draw table [d][S][4]
  CwsCodes cws;              // CWS code plan (derived from xs at build and at load)
  DevBuf<uint8_t> cws_rank;  // CWS per-position code dictionaries (derived, not stored)

  // LSH
  int key_kind = 0;
  int tableSize = 0, tables = 0, key_bits = 0;
  DevBuf<uint16_t> keys;     // [n][tables]
  DevBuf<int> offsets, buckets;
  DevBuf<float> key_planes;  // SimHash key planes [tables*bits][d]
  DevBuf<int> cp_diag;       // [tables][hashes][rounds][P]
  DevBuf<float> cws_key_tab; // CWS keys (key kind 10): draw table [d][tables * cp_hashes][4]
  int cp_P = 0, cp_hashes = 1, cp_rounds = 3;
  WmhState wmh_keys;
  DevBuf<uint32_t> bitmaps;  // per-CTA dedupe bitmaps of the LSH query
  int lsh_grid = 0;

  // tensor-core exact scan (implementation 8)
  DevBuf<uint16_t> xbf;      // bf16 rows padded to dp
  DevBuf<float> xbf_scale;   // unused (kept for the file layout)
  DevBuf<uint8_t> xf8;       // E4M3 unit rows x kE4M3Scale, 128 bytes (implementation 9)
  DevBuf<double> xnorm64;    // base row norms in double for the FP64 re-check (derived, not stored)
  int dp = 0;

  // Device error words of the query path (a pipeline or row-copy wait that timed out,
  // the weighted-MinHash draw limit), one per stream that has run queries on this index:
  // the kernels of a batch raise the word of the stream they run on, and a sync on a
  // stream reports and clears only that stream's word.  Read by callers after the query
  // has completed, so the query itself never synchronises.
  std::mutex err_mu;
  std::map<cudaStream_t, int*> err_words;
  // The stream's word, created (zeroed on the stream) by its first query.  Creating one
  // inside a stream capture is refused: the first query on a stream must come before.
  int* error_word(cudaStream_t s);
  // query counters (LSH: bucket entries walked, distinct candidates scored), cumulative
  DevBuf<unsigned long long> qstats;

  ~Index();
};

// Build from a device copy of the base.  `companion` (optional, device, nq rows) are
// queries the reference would transform alongside the base: preprocessing statistics
// (Jaccard min shift, MinHash bounds) then cover base and companion, as in the
// reference.  The companion buffer is transformed in place.
std::unique_ptr<Index> build_index(const lshg_index_params& p, DevBuf<float>&& base, int64_t n, float* companion,
                                   int ncomp, cudaStream_t stream, double* prep_ms, double* build_ms);

// Answer nq device-resident queries (row-major, d floats) into device points.  The
// query buffer is transformed in place.  Stream-ordered with no host synchronisation
// and no pageable copies, so it can be recorded into a CUDA graph; callers check
// query_error() after the stream has completed.
// extra (optional, device memory): further places (< k) whose near-ties the FP64 re-check
// orders, for callers that answer requests of smaller k from this launch's first rows.
void query_index(Index& idx, float* q, int nq, int k, lshg_point* out, cudaStream_t stream,
                 const RerankBounds* extra = nullptr);
// Throws if a completed query on `stream` raised that stream's device error word (clears it).
void query_error(Index& idx, cudaStream_t stream);
// Throws LSHG_ERR_INVALID_ARGUMENT unless the calling thread's current device is the
// device the index was built or loaded on.
void check_device(const Index& idx);

// Sketch / key a device query batch (after replaying the preprocessing).
void sketch_queries(Index& idx, float* q, int nq, DevBuf<uint32_t>* qs, DevBuf<float>* qsf,
                    DevBuf<uint16_t>* qkeys, cudaStream_t stream);

int next_pow2(int v);

// Build idx.xst (the linear scans' tiled sketches) from idx.xs, and for Hamming / one-bit
// Jaccard sketches of at most 1024 bits idx.xse (their E4M3 rows for the tensor cores).
void tile_sketches(Index& idx, cudaStream_t stream);

// Arrays derived from stored ones at build and at load: the tensor-core scans' FP64 row norms,
// and the split SimHash planes of the tensor-core projection.
void derive_tc(Index& idx, cudaStream_t stream);
void derive_simhash(Index& idx, cudaStream_t stream);

// Persistence (persist.cpp): checksummed binary image of a built index.
void save_index(const Index& idx, const char* path);
std::unique_ptr<Index> load_index(const char* path);  // owns a new stream

}  // namespace lshg

// The C handle owns the index.
struct lshg_index {
  std::unique_ptr<lshg::Index> impl;
};
