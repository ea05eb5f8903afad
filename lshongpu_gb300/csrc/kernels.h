// Host-side launchers for every device kernel of the engine.  All pointers are device
// pointers; every launcher is asynchronous on `stream`.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace lshg {

// Distance-function codes of the reference (distanceFunctions.cuh:54-71) plus the
// squared Euclidean used on JL sketches (distanceFunctions.cuh:87-99).
enum DistFunc : int { DIST_ANGULAR = 1, DIST_JACCARD = 2, DIST_EUCLID = 3, DIST_SQEUCLID = 4 };

// Sketched-distance codes (runSketchedDistanceFunction, distanceFunctions.cuh:136-154).
enum BitOp : int { OP_HAMMING = 3, OP_BYTE_JACCARD = 4, OP_ONEBIT_JACCARD = 5 };

// ---- preprocess.cu ---------------------------------------------------------------
// sqrt(sequential fmaf sum of squares) per row, exactly as the reference computes
// magnitudes (distanceFunctions.cuh:31-36, processingUtils.cuh:55-60).
void launch_row_norms(const float* x, int64_t n, int d, float* norms, cudaStream_t s);
// In-place x /= norm (transformToUnitVectors, processingUtils.cuh:48-67).
void launch_normalize(float* x, int64_t n, int d, cudaStream_t s);
// Point-tile layout for the SIMT scans: xt[tile][j][128], zero padded.
void launch_tile_transpose(const float* x, int64_t n, int d, float* xt, cudaStream_t s);
// Jaccard shift (transformData, processingUtils.cuh:12-46): per-dim min of floor(x).
void launch_min_floor(const float* x, int64_t n, int d, int* minv, cudaStream_t s);
void launch_shift_abs(float* x, int64_t n, int d, const int* minv, cudaStream_t s);
// WMH bounds (weightedMinHash.cuh:41-69): per-dim max of ceil(x).
void launch_max_ceil(const float* x, int64_t n, int d, int* maxv, cudaStream_t s);
// Fill helpers.
void launch_fill_u32(uint32_t* p, int64_t n, uint32_t v, cudaStream_t s);
void launch_u32_to_u16(const uint32_t* in, int64_t n, uint16_t* out, cudaStream_t s);
void launch_u32_to_u8(const uint32_t* in, int64_t n, uint8_t* out, cudaStream_t s);
// Pad rows of `words` 32-bit words to `wp` words (pad value `pad`).
void launch_pad_words(const uint32_t* in, int64_t n, int words, uint32_t* out, int wp, uint32_t pad,
                      cudaStream_t s);

// ---- project.cu ------------------------------------------------------------------
// Projections with the reference's sequential FP32 FMA chain in dimension order.
// mode 0: sign bits (simHash.cuh:20-46): plane p = w*bits + b sets bit b of word w.
//         out32 must be zeroed when bits != 32.
// mode 1: floats (JL, simHashJL.cuh:34-51): out_f[i*planes + p].
void launch_project(const float* x, int64_t n, int d, const float* planes, int nplanes, int mode,
                    int bits, int words, uint32_t* out32, float* out_f, cudaStream_t s);
// Sign bits of 32-plane words as above, run only when *gate != 0 (read on the device: the
// blocks leave at once otherwise).
void launch_project_gated(const float* x, int64_t n, int d, const float* planes, int nplanes, int words,
                          uint32_t* out32, const int* gate, cudaStream_t s);

// ---- crosspoly.cu ----------------------------------------------------------------
// Cross-polytope keys (crossPolyTope.cuh:25-85) with `hashes` concatenated hashes per
// table (reference: 1).  diag: int[tables][hashes][rounds][P] of +-1.
void launch_crosspoly(const float* x, int64_t n, int d, int P, int tables, int hashes, int rounds,
                      const int* diag, uint16_t* keys, cudaStream_t s);

// ---- wmh.cu ----------------------------------------------------------------------
// Draw tables of the rejection sampler (weightedMinHash.cuh:109-166): for each seed,
// curand_init(seed, 0, 10000) then T draws r = M * curand_uniform.  Layout r[j*H + h];
// the XORWOW state after T draws is kept for continuation.
void launch_wmh_tables(const int* seeds, int H, int T, int M, float* r, void* states, cudaStream_t s);
// Samples: counter = number of red draws before the first green one.
//  onebit = 0: out8[i*H + h] = counter mod 256 (sketchDataOriginal)
//  onebit = 1: bit b of out32[i*words + w] = bitmap[counter] (sketchDataOneBit), with
//              seed index h = w*hashBits + b.
void launch_wmh_sketch(const float* x, int64_t n, int d, const int* start, const int* map, int M,
                       const float* r, const void* states, int H, int T, int onebit, int words,
                       int hashBits, const uint8_t* bitmap, int bitmapLen, uint8_t* out8,
                       uint32_t* out32, int* err, cudaStream_t s);

// ---- scan_float.cu ---------------------------------------------------------------
// Top-C keys per (query, split) over float vectors (exact scans and JL sketches).
// xt: tile layout of the base; q: row-major queries; norms only for DIST_ANGULAR.
// out: [nq][splits][C] ascending keys.  Returns the number of splits used.
int launch_scan_float(const float* xt, int64_t n, int d, const float* xnorm, const float* q, int nq,
                      const float* qnorm, int dist, int C, int splits, uint64_t* out, cudaStream_t s);
int scan_float_splits(int64_t n, int nq, int C);

// ---- scan_bits.cu ----------------------------------------------------------------
// Top-C keys per (query, split) over packed sketches: rows of wp 32-bit words
// (wp % 4 == 0) holding `words` real words (bytes for OP_BYTE_JACCARD: `sbytes` real).
// xst: sketches tiled by launch_tile_sketches ([ceil(n/128)][wp/4][128] 16-byte chunks).
int launch_scan_bits(const uint32_t* xst, int64_t n, int wp, int words, int sbytes, const uint32_t* qs,
                     int nq, int op, int C, int splits, uint64_t* out, cudaStream_t s);
// Rows of wp words ([n][wp], wp % 4 == 0) -> the scans' tiled layout: chunk c (16 bytes)
// of point t*128 + l at [t][c][l]; points past n are zero.
void launch_tile_sketches(const uint32_t* xs, int64_t n, int wp, uint32_t* xst, cudaStream_t s);
int scan_bits_splits(int64_t n, int nq, int C);

// ---- scan_filter.cu ---------------------------------------------------------------
// Byte weighted-MinHash samples bit-sliced: rows of byte_slice_words(wp) words (8 a group
// of 32 samples), bytes past 4 wp = pad.
int byte_slice_words(int wp);
void launch_slice_bytes(const uint32_t* xs, int64_t n, int wp, int64_t rows, uint8_t pad, uint32_t* out,
                        cudaStream_t s);
// Whether the threshold-filter scan can serve C candidates over n points.
bool byte_filter_plan(int64_t n, int C, int* stride, int* rank, int* cap);
// Exact top-C keys [nq][C] by (byte Jaccard sketch distance, id): xsl_t the sliced base
// tiled like the popcount scan's, xst the packed tiled base (listed rescans), qs packed
// query rows [nq][wp].
void launch_byte_filter_scan(const uint32_t* xsl_t, const uint32_t* xst, int64_t n, int wp, int sbytes,
                             const uint32_t* qs, int nq, int C, uint64_t* out, int* err, cudaStream_t s);

// Consistent weighted sampling (implementation 10, cws.cu): (index, t) samples of the
// generalized Jaccard similarity, their range-coded bit-sliced form, and the scan.
constexpr uint64_t kCwsSeed = 0x6C7368672D637773ull;     // sketch draws
constexpr uint64_t kCwsKeySeed = 0x6C7368672D6B6579ull;  // LSH key draws (independent of the sketch's)
struct CwsCodes {
  int tmin = 0, tmax = 0;  // range of t over the base's samples
  int kb = 0, tb = 0;      // code bits of the dimension index and of t - tmin
  int pl = 0;              // bit planes of the sliced codes (8 or 16); 0: codes need more than 16 bits
  int dict = 0;            // 1: codes are ranks in per-position dictionaries of the base's codes
  int rlog = 0;            // dictionary rows of 2^rlog bytes
  const uint8_t* rank = nullptr;  // dictionaries [S][2^rlog] (device; owned by the index)
};
// Draw table [d][S] of (r, 1/r, ln c, beta) as 4 floats.
void cws_tables(int d, int S, std::vector<float>& tab, uint64_t seed = kCwsSeed);
// LSH keys [rows][L] from samples [rows][L * K]: table t hashes samples t K .. t K + K - 1
// into `bits` bits.
void launch_cws_keys(const uint32_t* smp, int64_t rows, int L, int K, int bits, uint16_t* keys, cudaStream_t s);
// Samples of `rows` vectors: rows of S (index, t) int32 pairs (2 S words).
void launch_cws_sketch(const float* x, int64_t rows, int d, int S, const float* tab, uint32_t* out, cudaStream_t s);
// Code plan from the base's samples (synchronises the stream to read their range of t).
CwsCodes cws_plan_codes(const uint32_t* xs, int64_t n, int S, int d, cudaStream_t s);
// Per-position dictionaries of the base's 9..16-bit codes: on success (every position
// holds at most 255 codes) `rank` holds them and c switches to 8-plane dictionary codes.
bool cws_build_dict(const uint32_t* xs, int64_t n, int S, CwsCodes& c, DevBuf<uint8_t>& rank, cudaStream_t s);
// Samples -> codes bit-sliced into rows of (S / 32) * pl words (queries: padding never matches).
void launch_cws_slice(const uint32_t* smp, int64_t rows, int S, int d, const CwsCodes& c, bool query, uint32_t* out,
                      cudaStream_t s);
// Exact top-C by (1 - matches / S, id) of every query into out [nq][C].  xsl_t: the base's
// tiled sliced codes (nullptr when c.pl == 0); xst: its samples tiled [tile][S / 2][128].
void launch_cws_scan(const uint32_t* xsl_t, const uint32_t* xst, int64_t n, int S, int d, const CwsCodes& c,
                     const uint32_t* qs, int nq, int C, uint64_t* out, int* err, cudaStream_t s);

// ---- rerank.cu -------------------------------------------------------------------
// Merge per-split sorted lists into one sorted list of C keys per query.
void launch_merge_splits(const uint64_t* in, int nq, int splits, int C, uint64_t* out, cudaStream_t s);
// Places of the FP64 re-check besides k (requests of smaller k answered from the same
// launch); n <= 4.  Passed in device memory, so that a recorded launch can be replayed with
// other places.
struct RerankBounds {
  int n;
  int k[4];
};

// Exact re-rank of candidate keys (candidateSetScanner.cuh:10-32) and top-k output;
// fp64_recheck: re-score, in double precision, the run of candidates around the k-th
// place whose FP32 distances lie within the FP32 error bound of one another (among the
// first 128) and order that run by the FP64 distance.
void launch_rerank(const uint64_t* cand, int nq, int C, const float* x, int64_t n, int d,
                   const float* xnorm, const float* q, const float* qnorm, int dist, int k,
                   struct ::lshg_point_s* out, cudaStream_t s, int* err = nullptr, bool fp64_recheck = false,
                   const double* xn64 = nullptr, const RerankBounds* extra_dev = nullptr);
// Row norms in double precision (sum of squares in dimension order, then sqrt): the FP64
// re-check's base magnitudes.
void launch_row_norms_fp64(const float* x, int64_t n, int d, double* out, cudaStream_t s);
// The FP64 band of the re-rank: |FP32 distance - k-th| <= band_abs + band_rel * |k-th|.
void fp64_band(int dist, int d, float* band_abs, float* band_rel);
// Keys to result points (ID, distance); empty keys become (-1, INT_MAX).
void launch_keys_to_points(const uint64_t* keys, int nq, int C, int k, struct ::lshg_point_s* out,
                           cudaStream_t s);

// ---- lsh.cu ----------------------------------------------------------------------
// Bucket tables (lshFramework.cuh:102-140): counts -> absolute offsets -> ids.
// keys: [n][tables] (u16 or u8 widened to u16).  offsets: [tables][tableSize],
// buckets: [tables][n].
void launch_lsh_build(const uint16_t* keys, int64_t n, int tables, int tableSize, int* offsets,
                      int* buckets, int* cursors, cudaStream_t s);

struct LshQueryArgs {
  const uint16_t* qkeys;  // [nq][tables]
  int nq, tables, tableSize;
  int64_t n;
  const int* offsets;
  const int* buckets;
  // exact data
  const float* x;
  const float* xnorm;
  const float* q;
  const float* qnorm;
  int d;
  int dist;  // rerank / exact distance function
  // sketched data (optional)
  int sketched;  // 0: exact distances on candidates; 1: sketch distance then rerank
  int sketch_kind;  // 3 hamming, 4 byte, 5 onebit, 6 JL (float)
  const uint32_t* xs;
  const uint32_t* qs;
  int wp, words, sbytes;
  const float* xsf;  // JL sketches [n][sdim]
  const float* qsf;
  int sdim;
  int C;  // candidate count kept before re-rank (sketched) or pow2 >= k (exact)
  int k;
  uint32_t* bitmaps;  // per-CTA dedupe bitmaps of the fused kernel [grid][ceil(n/32)]: zero on
                      // entry and exit unless bitmap_dirty (the split path never zeroes them)
  int grid;
  int vec4;                   // rows are 16-byte aligned float4 runs (d % 4 == 0)
  unsigned long long* stats;  // optional: += bucket entries walked, distinct candidates
  int* err;                   // device error flag (3: a row-copy wait timed out)
  int stage;                  // set by lsh_query_plan: rows staged by bulk copies
  int walk_grid;              // set by lsh_query_plan: CTAs of the bucket-walk kernel (split path)
  int split_cap;              // set by lsh_query_plan: distinct ids a query the walk lists (0: fused path)
  int bitmap_dirty;           // internal: the fused kernel zeroes its bitmap before its first query
  int* qctr;                  // internal: the fused kernel's query counter (zero at launch)
  const int* qlist;           // internal: queries to answer ([0] = count, then indices); nullptr = all
  int* lists;                 // internal: the fused kernel's distinct-id lists, [grid][list capacity]
};
void launch_lsh_query(const LshQueryArgs& a, struct ::lshg_point_s* out, cudaStream_t s);

}  // namespace lshg
