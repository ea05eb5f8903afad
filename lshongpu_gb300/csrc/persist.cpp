// Index persistence: a built index (base, sketches, keys, buckets, sampler tables,
// random projections and the recorded preprocessing) written as one binary image with
// an FNV-1a 64 checksum, so a serving process can restart without rebuilding.  The
// reference rebuilds everything on every run.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "index.h"

using namespace lshg;

namespace {

constexpr char kMagic[8] = {'L', 'S', 'H', 'G', 'I', 'D', 'X', '2'};

struct Writer {
  FILE* f;
  uint64_t h = 1469598103934665603ull;
  void put(const void* p, size_t n) {
    const unsigned char* c = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
    if (n && fwrite(p, 1, n, f) != n) throw Error(LSHG_ERR_IO, "write failed");
  }
  template <typename T> void pod(const T& v) { put(&v, sizeof v); }
  template <typename T> void vec(const std::vector<T>& v) {
    uint64_t n = v.size();
    pod(n);
    put(v.data(), n * sizeof(T));
  }
  template <typename T> void dev(const DevBuf<T>& b, cudaStream_t s) {
    std::vector<T> hst(b.n);
    if (b.n) {
      LSHG_CUDA(cudaMemcpyAsync(hst.data(), b.ptr, b.bytes(), cudaMemcpyDeviceToHost, s));
      LSHG_CUDA(cudaStreamSynchronize(s));
    }
    vec(hst);
  }
};

struct Reader {
  FILE* f;
  uint64_t h = 1469598103934665603ull;
  void get(void* p, size_t n) {
    if (n && fread(p, 1, n, f) != n) throw Error(LSHG_ERR_IO, "truncated index file");
    const unsigned char* c = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  }
  template <typename T> void pod(T& v) { get(&v, sizeof v); }
  template <typename T> void vec(std::vector<T>& v) {
    uint64_t n = 0;
    pod(n);
    if (n > (1ull << 40) / sizeof(T)) throw Error(LSHG_ERR_IO, "corrupt index file");
    v.resize(n);
    get(v.data(), n * sizeof(T));
  }
  template <typename T> void dev(DevBuf<T>& b, cudaStream_t s) {
    std::vector<T> hst;
    vec(hst);
    b.alloc(hst.size(), s);
    if (!hst.empty()) {
      LSHG_CUDA(cudaMemcpyAsync(b.ptr, hst.data(), b.bytes(), cudaMemcpyHostToDevice, s));
      LSHG_CUDA(cudaStreamSynchronize(s));
    }
  }
};

template <typename IO, typename IdxT>
void scalars(IO& io, IdxT& I) {
  io.pod(I.p);
  io.pod(I.n);
  io.pod(I.d);
  io.pod(I.dist);
  io.pod(I.C);
  io.pod(I.sk_kind);
  io.pod(I.words);
  io.pod(I.wp);
  io.pod(I.sbytes);
  io.pod(I.sdim);
  io.pod(I.key_kind);
  io.pod(I.tableSize);
  io.pod(I.tables);
  io.pod(I.key_bits);
  io.pod(I.cp_P);
  io.pod(I.cp_hashes);
  io.pod(I.cp_rounds);
  io.pod(I.lsh_grid);
  io.pod(I.dp);
}

void write_ops(Writer& w, const std::vector<PrepOp>& ops) {
  uint64_t n = ops.size();
  w.pod(n);
  for (const auto& op : ops) {
    int k = op.kind;
    w.pod(k);
    w.vec(op.minv);
  }
}

void read_ops(Reader& r, std::vector<PrepOp>& ops, cudaStream_t s) {
  uint64_t n = 0;
  r.pod(n);
  if (n > 64) throw Error(LSHG_ERR_IO, "corrupt index file");
  ops.resize(n);
  for (auto& op : ops) {
    int k = 0;
    r.pod(k);
    op.kind = (PrepOp::Kind)k;
    r.vec(op.minv);
    if (op.kind == PrepOp::SHIFT) {
      op.dminv = std::make_shared<DevBuf<int>>(op.minv.size(), s);
      LSHG_CUDA(cudaMemcpyAsync(op.dminv->ptr, op.minv.data(), op.minv.size() * 4, cudaMemcpyHostToDevice, s));
    }
  }
}

template <typename IO>
void wmh_io(IO& io, WmhState& w, cudaStream_t s) {
  io.pod(w.used);
  io.pod(w.M);
  io.pod(w.H);
  io.pod(w.T);
  io.pod(w.onebit);
  io.pod(w.words);
  io.pod(w.hashBits);
  io.pod(w.bitmapLen);
  io.vec(w.h_start);
  io.vec(w.h_map);
  io.dev(w.start, s);
  io.dev(w.map, s);
  io.dev(w.seeds, s);
  io.dev(w.rtab, s);
  io.dev(w.states, s);
  io.dev(w.bitmap, s);
}

template <typename IO>
void buffers_io(IO& io, Index& I, cudaStream_t s) {
  io.dev(I.x, s);
  io.dev(I.xnorm, s);
  io.dev(I.xt, s);
  io.dev(I.xs, s);
  io.dev(I.xsf, s);
  io.dev(I.xsft, s);
  io.dev(I.sk_planes, s);
  io.dev(I.keys, s);
  io.dev(I.offsets, s);
  io.dev(I.buckets, s);
  io.dev(I.key_planes, s);
  io.dev(I.cp_diag, s);
  io.dev(I.xbf, s);
  io.dev(I.xbf_scale, s);
  io.dev(I.xf8, s);
  wmh_io(io, I.wmh_sk, s);
  wmh_io(io, I.wmh_keys, s);
}

}  // namespace

namespace lshg {

void save_index(const Index& idx, const char* path) {
  Index& I = const_cast<Index&>(idx);
  FILE* f = fopen(path, "wb");
  if (!f) throw Error(LSHG_ERR_IO, std::string("cannot open ") + path);
  try {
    Writer w{f};
    w.put(kMagic, 8);
    scalars(w, I);
    write_ops(w, I.ops_keys);
    write_ops(w, I.ops_sketch);
    buffers_io(w, I, I.stream);
    uint64_t sum = w.h;
    if (fwrite(&sum, 1, 8, f) != 8) throw Error(LSHG_ERR_IO, "write failed");
  } catch (...) {
    fclose(f);
    throw;
  }
  fclose(f);
}

std::unique_ptr<Index> load_index(const char* path, cudaStream_t s) {
  FILE* f = fopen(path, "rb");
  if (!f) throw Error(LSHG_ERR_IO, std::string("cannot open ") + path);
  auto idx = std::make_unique<Index>();
  Index& I = *idx;
  I.stream = s;
  cudaGetDevice(&I.device);
  try {
    Reader r{f};
    char magic[8];
    r.get(magic, 8);
    if (memcmp(magic, kMagic, 8) != 0) throw Error(LSHG_ERR_IO, "not an lshg index file");
    scalars(r, I);
    read_ops(r, I.ops_keys, s);
    read_ops(r, I.ops_sketch, s);
    buffers_io(r, I, s);
    if (I.p.framework == 0 && I.xs.n) tile_sketches(I, s);  // derived layout, not stored
    uint64_t want = r.h, got = 0;
    if (fread(&got, 1, 8, f) != 8 || got != want) throw Error(LSHG_ERR_IO, "index file checksum mismatch");
    if (I.cp_diag.n) {  // the cross-polytope kernel applies the diagonals as sign flips
      std::vector<int32_t> dg(I.cp_diag.n);
      LSHG_CUDA(cudaMemcpyAsync(dg.data(), I.cp_diag.ptr, I.cp_diag.bytes(), cudaMemcpyDeviceToHost, s));
      LSHG_CUDA(cudaStreamSynchronize(s));
      for (int32_t g : dg)
        if (g != 1 && g != -1) throw Error(LSHG_ERR_IO, "index file: cross-polytope diagonal entry is not +-1");
    }
  } catch (...) {
    fclose(f);
    throw;
  }
  fclose(f);
  I.qerr.alloc(1, s);
  LSHG_CUDA(cudaMemsetAsync(I.qerr.ptr, 0, sizeof(int), s));
  I.qstats.alloc(2, s);
  LSHG_CUDA(cudaMemsetAsync(I.qstats.ptr, 0, I.qstats.bytes(), s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  return idx;
}

}  // namespace lshg

extern "C" {

const char* lshg_last_error(void);

int lshg_index_save(lshg_index* idx, const char* path) {
  if (!idx || !idx->impl || !path) return LSHG_ERR_INVALID_ARGUMENT;
  try {
    save_index(*idx->impl, path);
    return LSHG_OK;
  } catch (const Error& e) {
    return e.status;
  }
}

int lshg_index_load(const char* path, lshg_index** out) {
  if (!path || !out) return LSHG_ERR_INVALID_ARGUMENT;
  try {
    cudaStream_t s;
    LSHG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    std::unique_ptr<Index> idx;
    try {
      idx = load_index(path, s);
    } catch (...) {
      cudaStreamDestroy(s);
      throw;
    }
    idx->own_stream = true;
    auto* h = new lshg_index();
    h->impl = std::move(idx);
    *out = h;
    return LSHG_OK;
  } catch (const Error& e) {
    return e.status;
  }
}

}  // extern "C"
