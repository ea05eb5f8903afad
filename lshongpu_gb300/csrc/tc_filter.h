// Host-side interface of the tensor-core scan kernels (tc_filter.cu, tc_scan.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace lshg {
namespace tc {

constexpr int FILTER_TN = 256;    // base points a filter tile (UMMA N)
constexpr int MODE_GROUPMAX = 0;  // prepass: per-row group maxima of sampled tiles
constexpr int MODE_FILTER = 1;    // main pass: keep scores >= the row's threshold

// Subtracted from every threshold: the prepass and the main pass compute each score with
// the same instruction sequence, so this only guards against a last-bit difference.
constexpr float kTauMargin = 1e-6f;

// Parameters of the threshold prepass for a base of n points and CT candidates a query.
struct FilterPlan {
  int NT;   // 256-point base tiles
  int GW;   // group width of the prepass maxima (64 or 8; 0 = no prepass, keep every point)
  int S;    // prepass samples every S-th base tile
  int NS;   // sampled tiles
  int M;    // group maxima a query row
  int rank; // tau = the rank-th largest group maximum (CT, or fewer with sampling: see plan_filter)
  int cap;  // survivor slots a query
};

FilterPlan plan_filter(int64_t n, int CT);

// Prepass + threshold selection + filter pass: fills cnt[q] and cand[q][0..cap).
// mb: base tiles (256 rows x 64 columns boxes); mbhi: boxes of the second 64-column half
// trimmed to hi_cols columns (the K steps past the data dimension are never read).
// e4m3: operands are E4M3 codes (rows of 128 bytes; mb boxes of 256 rows x 128 bytes, mbhi
// unused); otherwise BF16 as above.
void launch_filter_scan(const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& mbhi, int hi_cols,
                        const FilterPlan& plan, int nq, int64_t n, int d, int QT, int CT, float* tau, int* cnt,
                        uint64_t* cand, int* err, bool e4m3, cudaStream_t s);

// tau[q] = a lower bound (within 1/65536 of the row's range) of the rank-th largest of the
// row's M group maxima, minus margin; -inf when the row holds fewer than rank maxima.
void launch_tau_select(const float* gmax, int nq, int M, int rank, float margin, float* tau, cudaStream_t s);

// Top-CT keys a query from its survivors (CT = 32, 64 or 128); queries with more survivors
// than cap or fewer than `need` are listed in ovf for the exact fallback.
void launch_cand_select(const int* cnt, const uint64_t* cand, int nq, int cap, int need, int CT, uint64_t* out,
                        int* ovf, cudaStream_t s);

// Tensor-core sketch scan (tc_hamming.cu): threshold plan for a base of n points and the
// top-C of each query.  ok = false: no prepass shape bounds C well (use the popcount scan).
struct HammingPlan {
  bool ok;
  int NT;    // 256-point base tiles
  int GW;    // prepass group width (64 or 8; 0 = no prepass, every point survives)
  int S;     // prepass samples every S-th tile
  int NS;    // sampled tiles
  int M;     // group maxima a query
  int rank;  // tau = the rank-th largest maximum
  int cap;   // survivor slots a query
};
HammingPlan plan_hamming(int64_t n, int C);
// 128-bit chunks of a sketch row of `words` words (rows of 128 * chunks E4M3 bytes).
int hamming_chunks(int words);
// Sketch rows [n][wp] (first `words` real) -> E4M3 +-1 rows [rows_pad][128 * chunks].
void launch_expand_bits(const uint32_t* xs, int64_t n, int wp, int words, int64_t rows_pad, uint8_t* out,
                        cudaStream_t s);
// Top-C keys [nq][C] of each query by (hamming asc, id asc); xse: the base's E4M3 rows
// (launch_expand_bits, rows padded to 256), xst: the tiled sketches (listed rescans), qs:
// query sketches [nq][wp].  op: OP_HAMMING or OP_ONEBIT_JACCARD.
void launch_tc_hamming(const uint8_t* xse, int64_t n, const uint32_t* xst, int wp, int words, const uint32_t* qs,
                       int nq, int op, int C, uint64_t* out, int* err, cudaStream_t s);
// Top-C keys [nq][C] of each query's survivors (keys make_key(-score, id), integer scores in
// [-bits, bits]): a warp sort for C <= 128, a histogram of the scores and a sort of the
// ties at the C-th score beyond; queries with fewer than `need` or more than `cap`
// survivors (or too many ties) are listed in ovf and their rows left for a rescan.
void launch_int_select(const int* cnt, const uint64_t* cand, int cap, int need, int C, int bits, int nq, uint64_t* out,
                       int* ovf, cudaStream_t s);

// Rows of kp bytes (a multiple of 16); boxes of 128 bytes x box_rows rows, 128-byte swizzle.
CUtensorMap make_map_bytes(const void* base, int64_t rows, int kp, int box_rows);

// SimHash sign bits on the tensor cores (tc_hamming.cu), bit-identical to project_kernel:
// a split-BF16 GEMM decides every sign outside a band around zero, the signs inside it are
// recomputed with the reference's FMA chain.  planes_split / pnorm: launch_split_bf16 of
// the planes (order 1, rows padded to 256) and their norms; out32 [n][words].
int signs_part_cols(int d);
void launch_split_bf16(const float* x, int64_t n, int d, int64_t rows_pad, int order, uint16_t* out, float* norms,
                       cudaStream_t s);
void launch_tc_signs(const float* x, int64_t n, int d, const uint16_t* planes_split, const float* pnorm,
                     const float* planes, int P, int words, uint32_t* out32, int* err, cudaStream_t s);

void launch_gather_rows(const uint16_t* src, const int* ovf, int nq, uint16_t* dst, cudaStream_t s);

void launch_merge_fallback(const uint64_t* part, const int* ovf, int nq, int NT, int grid, int CT, uint64_t* out,
                           cudaStream_t s);

// Work split of the per-row list kernel over `rows` gathered query rows: query tiles,
// tiles a CTA (stream-K), and partial-list slots a row.
struct ListGeometry {
  int QT, total, per, maxp;
};
__host__ __device__ inline ListGeometry tc_list_geometry(int rows, int NT, int grid) {
  ListGeometry g;
  g.QT = (rows + 127) / 128;
  g.total = g.QT * NT;
  g.per = g.total > 0 ? (g.total + grid - 1) / grid : 1;
  g.maxp = (NT + g.per - 1) / g.per + 1;
  return g;
}

}  // namespace tc
}  // namespace lshg
