// Sketched-distance linear scans over packed sketches with fused top-C selection.
//
// Replaces scanHammingDistance (sketchedDistanceScanners.cuh:14-100) and
// scanJaccardDistance (:194-274).  Distances are the reference's, as floats:
//   Hamming        sum popc(q ^ x)                                 (distanceFunctions.cuh:73-85)
//   one-bit WMH    1 - sum(32 - popc(q ^ x)) / (32 * words)         (:118-134)
//   byte WMH       1 - (#equal bytes) / sketchDim                   (:102-116)
// GB300 form: a CTA owns QB queries (sketches in shared memory) and a split of the
// base; each thread holds one point's sketch in registers and scores it against its half
// of the CTA's queries with XOR and popcount.  The base is read in the tiled layout
// (chunk c of point t*128 + l at [t][c][l], 16 bytes a chunk), so one warp load of a
// chunk is 512 contiguous bytes; read as rows, 32 lanes a row apart would touch 32 lines
// an instruction and the L1 data pipe, not the integer ALU, would bound the scan.  Candidates are filtered against each query's running threshold and
// folded into a per-query sorted top-C list (select.cuh).
#include "common.cuh"
#include "kernels.h"
#include "launch_count.h"
#include "profile.h"
#include "select.cuh"

namespace lshg {

namespace {

constexpr int kTile = 128;      // points per tile (one per thread of each half)
constexpr int kMaxChunks = 16;  // up to 64 words (2048 bits) per sketch

struct BitsSmem {
  size_t qs, kept, buf, thr, cnt, total;
};

__host__ __device__ inline size_t smem_take(size_t& off, size_t bytes) {
  off = (off + 15) / 16 * 16;
  size_t at = off;
  off += bytes;
  return at;
}

__host__ __device__ inline BitsSmem bits_layout(int wp, int QB, int C, int kBuf) {
  BitsSmem L;
  size_t off = 0;
  L.qs = smem_take(off, (size_t)QB * wp * 4);
  L.kept = smem_take(off, (size_t)QB * C * 8);
  L.buf = smem_take(off, (size_t)QB * kBuf * 8);
  L.thr = smem_take(off, (size_t)QB * 8);
  L.cnt = smem_take(off, (size_t)QB * 4);
  L.total = off;
  return L;
}

__device__ __forceinline__ int zero_bytes(uint32_t z) {
  uint32_t t = (z & 0x7f7f7f7fu) + 0x7f7f7f7fu;
  t = ~(t | z | 0x7f7f7f7fu);
  return __popc(t);
}

template <int OP>
__device__ __forceinline__ int word_score(uint32_t a, uint32_t b) {
  if (OP == OP_BYTE_JACCARD) return zero_bytes(a ^ b);
  return __popc(a ^ b);
}

// QB queries a CTA; each query's append buffer holds KBUF keys and the CTA checks the
// buffers every T tiles: a tile adds at most kTile keys to a query's buffer, so folding
// every buffer above KBUF - T * kTile at each check means no buffer can overflow between
// checks.  The check is one __syncthreads_or on "one of my appends landed above the
// limit" -- no block barrier in between.
// NC > 0: rows of exactly NC 128-bit chunks, loops fully unrolled without bounds tests;
// NC = 0: any row width up to kMaxChunks chunks (runtime bound).
// MINB: resident CTAs an SM the register budget is sized for.
template <int OP, int QB, int KBUF, int T, int NC, int MINB = 2>
__global__ void __launch_bounds__(256, MINB) scan_bits_kernel(const uint32_t* __restrict__ xst, int64_t n, int wp, int words,
                                                        int sbytes, const uint32_t* __restrict__ qs, int nq, int C,
                                                        int tiles_per_split, int splits, uint64_t* __restrict__ out,
                                                        const int* __restrict__ list) {
  static_assert(KBUF >= T * kTile, "append buffer must absorb T tiles");
  constexpr int kLimit = KBUF - T * kTile;
  extern __shared__ __align__(16) unsigned char smem[];
  const BitsSmem L = bits_layout(wp, QB, C, KBUF);
  uint32_t* qsm = reinterpret_cast<uint32_t*>(smem + L.qs);
  TopCShared S{reinterpret_cast<uint64_t*>(smem + L.kept), reinterpret_cast<uint64_t*>(smem + L.buf),
               reinterpret_cast<int*>(smem + L.cnt), reinterpret_cast<uint64_t*>(smem + L.thr), C, KBUF};

  // list (optional): scan only the queries list[1 .. list[0]]; slot i of the list is query
  // list[1 + i], and its result goes to that query's row
  const int nqe = list ? list[0] : nq;
  const int q0 = blockIdx.x * QB;
  if (q0 >= nqe) return;  // block-uniform, before any barrier
  const int split = blockIdx.y;
  const int ntiles = (int)((n + kTile - 1) / kTile);
  const int t_begin = split * tiles_per_split;
  const int t_end = min(ntiles, t_begin + tiles_per_split);
  constexpr int NCH = NC > 0 ? NC : kMaxChunks;
  const int nc = NC > 0 ? NC : (wp >> 2);

  for (int i = threadIdx.x; i < QB * wp; i += blockDim.x) {
    int qi = i / wp;
    const int64_t qrow = q0 + qi < nqe ? (list ? list[1 + q0 + qi] : q0 + qi) : 0;
    qsm[i] = (q0 + qi < nqe) ? qs[qrow * wp + (i - qi * wp)] : 0u;
  }
  topc_init(S, QB);
  __syncthreads();

  const int half = threadIdx.x >> 7;   // queries half, half+2, ...
  const int pl = threadIdx.x & 127;    // point within the tile
  constexpr int QPT = (QB + 1) / 2;    // queries per thread
  uint64_t thr[QPT];
#pragma unroll
  for (int a = 0; a < QPT; ++a) thr[a] = kEmptyKey;

  const float inv_div_f = (OP == OP_ONEBIT_JACCARD) ? (float)(32 * words) : (float)sbytes;
  bool over = false;  // one of this thread's appends since the last check landed above kLimit

  for (int tile = t_begin; tile < t_end; ++tile) {
    const int64_t p = (int64_t)tile * kTile + pl;
    const bool valid = p < n;
    uint4 xr[NCH];
    const uint4* col = reinterpret_cast<const uint4*>(xst) + (int64_t)tile * nc * kTile + pl;
#pragma unroll
    for (int c = 0; c < NCH; ++c) xr[c] = (NC > 0 || c < nc) ? __ldg(&col[c * kTile]) : make_uint4(0, 0, 0, 0);

    if (valid) {
#pragma unroll
      for (int a = 0; a < QPT; ++a) {
        const int qi = half + 2 * a;
        if (qi >= QB || q0 + qi >= nqe) continue;
        const uint4* qv = reinterpret_cast<const uint4*>(qsm + qi * wp);
        int acc = 0;
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
          if (NC > 0 || c < nc) {
            uint4 b = qv[c];
            acc += word_score<OP>(xr[c].x, b.x) + word_score<OP>(xr[c].y, b.y) + word_score<OP>(xr[c].z, b.z) +
                   word_score<OP>(xr[c].w, b.w);
          }
        }
        float dist;
        if (OP == OP_HAMMING) {
          dist = (float)acc;
        } else if (OP == OP_ONEBIT_JACCARD) {
          dist = __fsub_rn(1.0f, __fdiv_rn((float)(32 * words - acc), inv_div_f));
        } else {
          dist = __fsub_rn(1.0f, __fdiv_rn((float)acc, inv_div_f));
        }
        const uint64_t key = make_key(dist, (int)p);
        if (key < thr[a]) {
          const int pos = atomicAdd(&S.cnt[qi], 1);
          S.buf[(size_t)qi * KBUF + pos] = key;
          over |= pos >= kLimit;
        }
      }
    }
    if ((tile - t_begin) % T == T - 1 && tile + 1 < t_end) {  // uniform: same tile loop in every thread
      if (__syncthreads_or(over)) {
        topc_flush(S, QB, kLimit);
#pragma unroll
        for (int a = 0; a < QPT; ++a) {
          const int qi = half + 2 * a;
          if (qi < QB) thr[a] = S.thr[qi];
        }
      }
      over = false;
    }
  }
  topc_flush(S, QB, 0);

  for (int i = threadIdx.x; i < QB * C; i += blockDim.x) {
    int qi = i / C, c = i - qi * C;
    if (q0 + qi < nqe) {
      const int64_t qrow = list ? list[1 + q0 + qi] : q0 + qi;
      out[(qrow * splits + split) * C + c] = S.kept[(size_t)qi * C + c];
    }
  }
}

template <int OP, int QB, int KBUF, int T, int NC, int MINB = 2>
void launch_cfg(const uint32_t* xs, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq, int C,
                int splits, uint64_t* out, const int* list, cudaStream_t s) {
  ProfScope _ps(list ? "scan_bits_listed" : "scan_bits", s);
  size_t smem = bits_layout(wp, QB, C, KBUF).total;
  auto kern = scan_bits_kernel<OP, QB, KBUF, T, NC, MINB>;
  LSHG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int ntiles = ceil_div(n, kTile);
  int tps = ceil_div(ntiles, splits);
  dim3 grid(ceil_div(nq, QB), splits);
  kern<<<grid, 256, smem, s>>>(xs, n, wp, words, sbytes, qs, nq, C, tps, splits, out, list);
  count_launch();
  LSHG_CHECK_LAUNCH();
}

template <int OP, int NC>
void launch_op(const uint32_t* xs, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq, int C,
               int splits, uint64_t* out, const int* list, cudaStream_t s) {
  if (C <= 128) launch_cfg<OP, 16, 256, 1, NC, 3>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s);
  // up to 1024: 4 queries a block (49 KB at C = 1024) so that three CTAs share an SM and hide
  // one another's fold barriers; the base is streamed twice as often, which L2 absorbs
  else if (C <= 1024) launch_cfg<OP, 4, 512, 2, NC, 3>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s);
  else launch_cfg<OP, 2, 2048, 4, NC>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s);  // long folds: fewer
}

// Row width specialised for each sketch type's usual size (1024-bit SimHash = 8 chunks,
// 256 byte samples = 16 chunks, 256 one-bit samples = 2 chunks); other widths use the
// generic kernel.
template <int OP, int NC_FAST>
void launch_width(const uint32_t* xs, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq, int C,
                  int splits, uint64_t* out, const int* list, cudaStream_t s) {
  if (wp / 4 == NC_FAST) launch_op<OP, NC_FAST>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s);
  else launch_op<OP, 0>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s);
}

}  // namespace

int scan_bits_splits(int64_t n, int nq, int C) {
  // three CTAs an SM (two for C > 1024); for C <= 128 pick the split count whose grid fills whole waves best,
  // between the count giving ~1.5 CTAs a slot and 4x that (at most 64 splits, >= 4 tiles
  // a split)
  const int QB = C <= 128 ? 16 : (C <= 1024 ? 4 : 2);
  const int slots = num_sms() * (C > 1024 ? 2 : 3);
  const int qblocks = ceil_div(nq, QB);
  const int ntiles = ceil_div(n, kTile);
  const int maxs = std::max(1, std::min(ntiles / 4, 64));
  const int want = std::max(1, std::min(maxs, ceil_div((int64_t)num_sms() * 3, qblocks)));
  if (C > 128) return want;  // large lists: every extra split restarts them cold, which costs more than the tail
  int best = want;
  double best_eff = 0.0;
  for (int sp = want; sp <= std::min(maxs, 4 * want); ++sp) {
    const int64_t ctas = (int64_t)qblocks * sp;
    const double eff = (double)ctas / (double)(ceil_div(ctas, slots) * (int64_t)slots);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = sp;
    }
  }
  return best;
}

__global__ void tile_sketches_kernel(const uint4* __restrict__ xs, int64_t n, int nc, int64_t total,
                                     uint4* __restrict__ xst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = i % kTile, tc = i / kTile;   // i = (tile * nc + c) * kTile + l
    const int64_t c = tc % nc, t = tc / nc;
    const int64_t p = t * kTile + l;
    xst[i] = p < n ? xs[p * nc + c] : make_uint4(0, 0, 0, 0);
  }
}

void launch_tile_sketches(const uint32_t* xs, int64_t n, int wp, uint32_t* xst, cudaStream_t s) {
  LSHG_REQUIRE(wp % 4 == 0, "sketch rows must be a multiple of 4 words");
  const int nc = wp / 4;
  const int64_t total = (n + kTile - 1) / kTile * kTile * nc;
  if (total == 0) return;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
  tile_sketches_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const uint4*>(xs), n, nc, total,
                                              reinterpret_cast<uint4*>(xst));
  count_launch();
  LSHG_CHECK_LAUNCH();
}

namespace {
int scan_bits_dispatch(const uint32_t* xs, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq,
                       int op, int C, int splits, uint64_t* out, const int* list, cudaStream_t s) {
  if (nq <= 0) return splits;
  LSHG_REQUIRE(n > 0, "sketch scan: empty base");
  LSHG_REQUIRE(wp % 4 == 0 && wp / 4 <= kMaxChunks, "sketch scan: rows must be 4..64 words, multiple of 4");
  LSHG_REQUIRE(C >= 32 && C <= 4096 && (C & (C - 1)) == 0, "sketch scan: C must be a power of two in [32, 4096]");
  switch (op) {
    case OP_HAMMING: launch_width<OP_HAMMING, 8>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s); break;
    case OP_BYTE_JACCARD:
      launch_width<OP_BYTE_JACCARD, 16>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s);
      break;
    case OP_ONEBIT_JACCARD:
      launch_width<OP_ONEBIT_JACCARD, 2>(xs, n, wp, words, sbytes, qs, nq, C, splits, out, list, s);
      break;
    default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "sketch scan: invalid sketch type");
  }
  return splits;
}
}  // namespace

int launch_scan_bits(const uint32_t* xs, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq, int op,
                     int C, int splits, uint64_t* out, cudaStream_t s) {
  return scan_bits_dispatch(xs, n, wp, words, sbytes, qs, nq, op, C, splits, out, nullptr, s);
}

// The queries list[1 .. list[0]] (a device-side list, at most nq of them) scanned over
// the whole base, each result written to out[query][C]; blocks past the list's end exit.
int launch_scan_bits_listed(const uint32_t* xst, int64_t n, int wp, int words, int sbytes, const uint32_t* qs, int nq,
                            int op, int C, const int* list, uint64_t* out, cudaStream_t s) {
  return scan_bits_dispatch(xst, n, wp, words, sbytes, qs, nq, op, C, 1, out, list, s);
}

}  // namespace lshg
