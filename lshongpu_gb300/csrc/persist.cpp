// Index persistence: a built index (base, sketches, keys, buckets, sampler tables,
// random projections and the recorded preprocessing) written as one binary image with
// an FNV-1a 64 checksum, so a serving process can restart without rebuilding.  The
// reference rebuilds everything on every run.
#include <climits>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "index.h"

using namespace lshg;

namespace lshg {
size_t wmh_state_bytes();
int lsh_query_grid(int nq);
void set_last_error(const char* msg);
}  // namespace lshg

namespace {

constexpr char kMagic[8] = {'L', 'S', 'H', 'G', 'I', 'D', 'X', '4'};

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

// Parses an image already in host memory whose checksum has been verified.  Device
// buffers are only staged here (element count and raw bytes); they are checked against the
// index's scalars and uploaded afterwards, so nothing of a damaged file reaches the GPU.
struct Reader {
  const unsigned char* p;
  size_t left;
  struct Staged {
    size_t count = 0;
    std::vector<unsigned char> raw;
    std::function<void(cudaStream_t)> upload;
  };
  std::map<const void*, Staged> staged;

  void get(void* dst, size_t n) {
    if (n > left) throw Error(LSHG_ERR_IO, "truncated index file");
    if (n) memcpy(dst, p, n);
    p += n;
    left -= n;
  }
  template <typename T> void pod(T& v) { get(&v, sizeof v); }
  template <typename T> void vec(std::vector<T>& v) {
    uint64_t n = 0;
    pod(n);
    if (n > left / sizeof(T)) throw Error(LSHG_ERR_IO, "corrupt index file");
    v.resize(n);
    get(v.data(), n * sizeof(T));
  }
  template <typename T> void dev(DevBuf<T>& b, cudaStream_t) {
    uint64_t n = 0;
    pod(n);
    if (n > left / sizeof(T)) throw Error(LSHG_ERR_IO, "corrupt index file");
    Staged& st = staged[&b];
    st.count = n;
    st.raw.resize(n * sizeof(T));
    get(st.raw.data(), st.raw.size());
    const std::vector<unsigned char>* raw = &st.raw;
    st.upload = [&b, raw, n](cudaStream_t s) {
      b.alloc(n, s);
      if (n) LSHG_CUDA(cudaMemcpyAsync(b.ptr, raw->data(), raw->size(), cudaMemcpyHostToDevice, s));
    };
  }
  size_t count(const void* b) const {
    auto it = staged.find(b);
    return it == staged.end() ? 0 : it->second.count;
  }
  template <typename T> const T* data(const DevBuf<T>& b) const {
    auto it = staged.find(&b);
    return it == staged.end() ? nullptr : reinterpret_cast<const T*>(it->second.raw.data());
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
  io.pod(I.cws_S);
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

void read_ops(Reader& r, std::vector<PrepOp>& ops) {
  uint64_t n = 0;
  r.pod(n);
  if (n > 64) throw Error(LSHG_ERR_IO, "corrupt index file");
  ops.resize(n);
  for (auto& op : ops) {
    int k = 0;
    r.pod(k);
    if (k != PrepOp::NORMALIZE && k != PrepOp::SHIFT) throw Error(LSHG_ERR_IO, "corrupt index file");
    op.kind = (PrepOp::Kind)k;
    r.vec(op.minv);
  }
}

void upload_ops(std::vector<PrepOp>& ops, cudaStream_t s) {
  for (auto& op : ops)
    if (op.kind == PrepOp::SHIFT) {
      op.dminv = std::make_shared<DevBuf<int>>(op.minv.size(), s);
      LSHG_CUDA(cudaMemcpyAsync(op.dminv->ptr, op.minv.data(), op.minv.size() * 4, cudaMemcpyHostToDevice, s));
    }
}

[[noreturn]] void bad(const char* what) {
  throw Error(LSHG_ERR_IO, std::string("index file: inconsistent ") + what);
}
void need(bool ok, const char* what) {
  if (!ok) bad(what);
}

// Sampler tables: sizes and the slot map, whose entries index the point's components.
void check_wmh(const Reader& r, const WmhState& w, int d, int H, int onebit, int words, int hashBits) {
  need(w.used && w.H == H && w.onebit == onebit && w.words == words && w.hashBits == hashBits, "sampler shape");
  need(w.M >= 1 && w.M < (1 << 24) && w.T >= 1 && w.T <= (1 << 16) && w.bitmapLen == 255, "sampler sizes");
  need(w.h_start.size() == (size_t)d && w.h_map.size() == (size_t)w.M, "sampler maps");
  for (int i = 0; i < d; ++i) need(w.h_start[i] >= 0 && w.h_start[i] <= w.M, "sampler start offsets");
  for (int v : w.h_map) need(v >= 0 && v < d, "sampler slot map");
  need(r.count(&w.start) == (size_t)d && r.count(&w.map) == (size_t)w.M, "sampler map buffers");
  need(memcmp(r.data(w.start), w.h_start.data(), (size_t)d * 4) == 0 &&
           memcmp(r.data(w.map), w.h_map.data(), (size_t)w.M * 4) == 0,
       "sampler map buffers");
  need(r.count(&w.seeds) == (size_t)H && r.count(&w.rtab) == (size_t)w.T * H &&
           r.count(&w.states) == wmh_state_bytes() * H && r.count(&w.bitmap) == (size_t)w.bitmapLen,
       "sampler tables");
}

void check_no_wmh(const Reader& r, const WmhState& w) {
  need(!w.used && !r.count(&w.start) && !r.count(&w.map) && !r.count(&w.seeds) && !r.count(&w.rtab) &&
           !r.count(&w.states) && !r.count(&w.bitmap),
       "sampler tables");
}

// Every buffer's length against the scalars it is indexed with, every required buffer
// present, and the bucket tables' offsets and ids in range: a kernel launched on a
// loaded index reads only within its buffers.
void check_loaded(const Reader& r, const Index& I) {
  const int64_t n = I.n;
  const int d = I.d;
  need(n >= 1 && n < (int64_t)INT_MAX && d >= 1 && d <= (1 << 16) && I.p.d == d, "base size");
  need(I.p.framework == 0 || I.p.framework == 1, "framework");
  const int impl = I.p.implementation == 1 ? 2 : I.p.implementation;
  need(impl == 2 || impl == 3 || impl == 4 || impl == 5 || impl == 6 || impl == 8 || impl == 9 || impl == 10,
       "implementation");
  need(impl != 10 || I.p.framework == 0, "implementation");
  need(I.dist >= 1 && I.dist <= 3, "distance function");
  need(I.C >= 32 && I.C <= 4096 && (I.C & (I.C - 1)) == 0, "candidate count");
  const size_t tiles = (size_t)ceil_div(n, 128);
  need(r.count(&I.x) == (size_t)n * d, "base rows");
  need(r.count(&I.xnorm) == (I.dist == DIST_ANGULAR ? (size_t)n : 0), "magnitudes");
  need(r.count(&I.xt) == (I.p.framework == 0 && impl == 2 ? tiles * 128 * d : 0), "base tiles");
  const bool sketched = (impl >= 3 && impl <= 6) || impl == 10;
  need(I.sk_kind == (sketched ? impl : 0), "sketch kind");
  size_t xs = 0, xsf = 0, xsft = 0, planes = 0;
  switch (I.sk_kind) {
    case 3:
      need(I.words >= 1 && I.words <= 64 && I.wp == (I.words + 3) / 4 * 4, "SimHash width");
      xs = (size_t)n * I.wp;
      planes = (size_t)d * 32 * I.words;
      break;
    case 4:
      need(I.sbytes >= 1 && I.sbytes <= 256 && I.words == (I.sbytes + 3) / 4 && I.wp == (I.words + 3) / 4 * 4,
           "sample width");
      xs = (size_t)n * I.wp;
      check_wmh(r, I.wmh_sk, d, I.sbytes, 0, 0, 0);
      break;
    case 5:
      need(I.words >= 1 && I.words <= 64 && I.wp == (I.words + 3) / 4 * 4, "sample width");
      xs = (size_t)n * I.wp;
      check_wmh(r, I.wmh_sk, d, I.words * 32, 1, I.words, 32);
      break;
    case 10:
      need(I.cws_S >= 32 && I.cws_S <= 256 && I.cws_S % 32 == 0 && I.words == 2 * I.cws_S && I.wp == I.words &&
               d <= 4096,
           "CWS width");
      xs = (size_t)n * I.wp;
      break;
    case 6:
      need(I.sdim >= 1 && I.sdim <= (1 << 16), "JL width");
      xsf = (size_t)n * I.sdim;
      xsft = tiles * 128 * I.sdim;
      planes = (size_t)I.sdim * d;
      break;
  }
  if (I.sk_kind != 4 && I.sk_kind != 5) check_no_wmh(r, I.wmh_sk);
  need(r.count(&I.cws_tab) == (I.sk_kind == 10 ? (size_t)d * I.cws_S * 4 : 0), "CWS draw table");
  need(r.count(&I.xs) == xs && r.count(&I.xsf) == xsf && r.count(&I.xsft) == xsft && r.count(&I.sk_planes) == planes,
       "sketch buffers");
  if (I.p.framework == 1) {
    need(impl != 8 && impl != 9, "implementation");
    need(I.tables >= 1 && I.tables <= 256 && I.key_bits >= 1 && I.key_bits <= 24 &&
             I.tableSize == (1 << I.key_bits),
         "table shape");
    const size_t L = I.tables, S = I.tableSize;
    need(r.count(&I.keys) == (size_t)n * L && r.count(&I.offsets) == L * S && r.count(&I.buckets) == L * n,
         "bucket tables");
    size_t kp = 0, diag = 0;
    switch (I.key_kind) {
      case 3:
        kp = L * d * I.key_bits;
        break;
      case 4:
        need(S >= 256, "table size");
        check_wmh(r, I.wmh_keys, d, I.tables, 0, 0, 0);
        break;
      case 5:
        check_wmh(r, I.wmh_keys, d, I.tables * I.key_bits, 1, I.tables, I.key_bits);
        break;
      case 10:
        need(I.key_bits <= 16 && I.cp_hashes >= 1 && I.cp_hashes <= 16 && d <= 4096, "CWS key shape");
        need(r.count(&I.cws_key_tab) == (size_t)d * L * I.cp_hashes * 4, "CWS key draw table");
        break;
      case 7: {
        int P = 1;
        while (P < d) P *= 2;
        need(I.cp_P == P && I.cp_hashes >= 1 && I.cp_hashes <= 16 && I.cp_rounds >= 1 && I.cp_rounds <= 16,
             "cross-polytope shape");
        int64_t range = 1;
        for (int h = 0; h < I.cp_hashes && range <= 65536; ++h) range *= 2 * P;
        need(range <= 65536 && range <= (int64_t)S, "cross-polytope key range");
        diag = (size_t)P * L * I.cp_hashes * I.cp_rounds;
        need(r.count(&I.cp_diag) == diag, "cross-polytope diagonals");
        const int32_t* dg = r.data(I.cp_diag);
        for (size_t i = 0; i < diag; ++i)  // the key kernel applies them as sign flips
          if (dg[i] != 1 && dg[i] != -1) throw Error(LSHG_ERR_IO, "index file: cross-polytope diagonal entry is not +-1");
        break;
      }
      default:
        bad("key kind");
    }
    if (I.key_kind != 4 && I.key_kind != 5) check_no_wmh(r, I.wmh_keys);
    if (I.key_kind != 10) need(!r.count(&I.cws_key_tab), "key buffers");
    need(r.count(&I.key_planes) == kp && r.count(&I.cp_diag) == diag, "key buffers");
    // offsets ascend within a table's region [t*n, t*n + n]; ids are row numbers
    const int32_t* off = r.data(I.offsets);
    const int32_t* bk = r.data(I.buckets);
    for (size_t t = 0; t < L; ++t) {
      int64_t prev = (int64_t)t * n;
      for (size_t k = 0; k < S; ++k) {
        const int64_t o = off[t * S + k];
        need(o >= prev && o <= (int64_t)(t + 1) * n, "bucket offsets");
        prev = o;
      }
    }
    for (size_t i = 0; i < L * (size_t)n; ++i) need(bk[i] >= 0 && bk[i] < n, "bucket ids");
  } else {
    need(I.key_kind == 0 && !r.count(&I.keys) && !r.count(&I.offsets) && !r.count(&I.buckets) &&
             !r.count(&I.key_planes) && !r.count(&I.cp_diag) && !r.count(&I.cws_key_tab),
         "bucket tables");
    check_no_wmh(r, I.wmh_keys);
  }
  if (impl == 8 || impl == 9) {
    need(I.p.framework == 0 && I.dist == DIST_ANGULAR && d <= 128 && I.dp == 128, "tensor-core layout");
    const size_t npad = (size_t)ceil_div(n, 256) * 256;
    need(r.count(&I.xbf) == npad * 128 && r.count(&I.xf8) == (impl == 9 ? npad * 128 : 0), "tensor-core rows");
  } else {
    need(!r.count(&I.xbf) && !r.count(&I.xf8), "tensor-core rows");
  }
  need(!r.count(&I.xbf_scale), "tensor-core scales");
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
  io.dev(I.cws_tab, s);
  io.dev(I.cws_key_tab, s);
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

std::unique_ptr<Index> load_index(const char* path) {
  // the whole file is read and its checksum compared before anything is parsed; no CUDA
  // call is made before the file has passed every check
  std::vector<unsigned char> img;
  {
    FILE* f = fopen(path, "rb");
    if (!f) throw Error(LSHG_ERR_IO, std::string("cannot open ") + path);
    unsigned char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof buf, f)) > 0) img.insert(img.end(), buf, buf + got);
    const bool err = ferror(f);
    fclose(f);
    if (err) throw Error(LSHG_ERR_IO, std::string("cannot read ") + path);
  }
  if (img.size() < sizeof kMagic + 8) throw Error(LSHG_ERR_IO, "truncated index file");
  const size_t body = img.size() - 8;
  uint64_t want = 1469598103934665603ull, got = 0;
  for (size_t i = 0; i < body; ++i) want = (want ^ img[i]) * 1099511628211ull;
  memcpy(&got, img.data() + body, 8);
  if (memcmp(img.data(), kMagic, 8) != 0) throw Error(LSHG_ERR_IO, "not an lshg index file");
  if (got != want) throw Error(LSHG_ERR_IO, "index file checksum mismatch");

  auto idx = std::make_unique<Index>();
  Index& I = *idx;
  Reader r{img.data() + 8, body - 8};
  scalars(r, I);
  read_ops(r, I.ops_keys);
  read_ops(r, I.ops_sketch);
  buffers_io(r, I, nullptr);  // staged in host memory only
  if (r.left != 0) throw Error(LSHG_ERR_IO, "corrupt index file (trailing bytes)");
  for (const auto* ops : {&I.ops_keys, &I.ops_sketch})
    for (const auto& op : *ops) need(op.kind == PrepOp::NORMALIZE || op.minv.size() == (size_t)I.d, "shift");
  check_loaded(r, I);

  // device work only from here on
  cudaStream_t s;
  LSHG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  I.stream = s;
  I.own_stream = true;
  cudaGetDevice(&I.device);
  I.p.opt.stream = nullptr;  // a stream handle of the process that saved the index
  if (I.p.framework == 1) I.lsh_grid = lsh_query_grid(1 << 30);  // this device's resident CTAs
  upload_ops(I.ops_keys, s);
  upload_ops(I.ops_sketch, s);
  for (auto& kv : r.staged) kv.second.upload(s);
  if (I.p.framework == 0 && I.xs.n) tile_sketches(I, s);  // derived layouts, not stored
  if (I.p.framework == 0 && (I.p.implementation == 8 || I.p.implementation == 9)) derive_tc(I, s);
  derive_simhash(I, s);
  I.qstats.alloc(2, s);
  LSHG_CUDA(cudaMemsetAsync(I.qstats.ptr, 0, I.qstats.bytes(), s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  return idx;
}

}  // namespace lshg

extern "C" {

int lshg_index_save(lshg_index* idx, const char* path) {
  if (!idx || !idx->impl || !path) return LSHG_ERR_INVALID_ARGUMENT;
  try {
    check_device(*idx->impl);
    save_index(*idx->impl, path);
    return LSHG_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  }
}

int lshg_index_load(const char* path, lshg_index** out) {
  if (!path || !out) return LSHG_ERR_INVALID_ARGUMENT;
  try {
    std::unique_ptr<Index> idx = load_index(path);
    auto* h = new lshg_index();
    h->impl = std::move(idx);
    *out = h;
    return LSHG_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  }
}

}  // extern "C"
