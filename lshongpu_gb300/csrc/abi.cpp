// extern "C" boundary of liblshg.so (declared in include/lshg.h).
//
// Every entry point catches exceptions and returns a status; the message is kept per
// thread for lshg_last_error.  The reference instead prints and exits on CUDA errors
// (cudaHelpers.cuh:8-15) and prints "Invalid implementation selected" for bad codes
// (kernel.cu:48-51).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <set>
#include <string>
#include <vector>

#include "host_rng.h"
#include "index.h"
#include "launch_count.h"

namespace lshg {
std::atomic<int64_t>& launch_counter() {
  static std::atomic<int64_t> c{0};
  return c;
}
}  // namespace lshg

using namespace lshg;

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace lshg {
// Lets entry points defined in other translation units report their message.
void set_last_error(const char* msg) { g_last_error = msg; }
}  // namespace lshg

namespace {

template <typename F>
int guarded(F&& f) {
  try {
    f();
    return LSHG_OK;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    g_last_error = "host out of memory";
    return LSHG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return LSHG_ERR_CUDA;
  }
}

void require_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    throw Error(LSHG_ERR_NO_DEVICE, "no CUDA device available");
  }
}

cudaStream_t pick_stream(const lshg_options* opt, bool* own) {
  if (opt && opt->stream) {
    *own = false;
    return (cudaStream_t)opt->stream;
  }
  cudaStream_t s;
  LSHG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *own = true;
  return s;
}

struct StreamGuard {
  cudaStream_t s;
  bool own;
  ~StreamGuard() {
    if (own && s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }
};

DevBuf<float> upload_floats(const float* h, size_t count, cudaStream_t s) {
  DevBuf<float> b(count, s);
  LSHG_CUDA(cudaMemcpyAsync(b.ptr, h, count * sizeof(float), cudaMemcpyHostToDevice, s));
  return b;
}

// Shared body of lshg_linear_scans / lshg_lsh: upload, build (statistics over data and
// queries, as the reference), query, download.
void run_reference_call(const lshg_index_params& p, int k, int N_query, int N_data, const float* data,
                        const float* queries, lshg_result* res) {
  LSHG_REQUIRE(res && res->results, "result buffer is NULL");
  LSHG_REQUIRE(data && queries, "data / queries are NULL");
  LSHG_REQUIRE(k >= 1 && N_query >= 0 && N_data >= 1 && p.d >= 1, "invalid sizes");
  require_device();
  bool own = false;
  cudaStream_t s = pick_stream(&p.opt, &own);
  StreamGuard g{s, own};
  auto t0 = std::chrono::steady_clock::now();
  DevBuf<float> base = upload_floats(data, (size_t)N_data * p.d, s);
  DevBuf<float> comp = upload_floats(queries, (size_t)N_query * p.d, s);
  DevBuf<float> q = upload_floats(queries, (size_t)N_query * p.d, s);
  double prep = 0, build = 0;
  auto idx = build_index(p, std::move(base), N_data, comp.ptr, N_query, s, &prep, &build);
  comp.release();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  DevBuf<lshg_point> out((size_t)N_query * k, s);
  query_index(*idx, q.ptr, N_query, k, out.ptr, s);
  cudaEventRecord(e1, s);
  LSHG_CUDA(cudaMemcpyAsync(res->results, out.ptr, (size_t)N_query * k * sizeof(lshg_point), cudaMemcpyDeviceToHost,
                            s));
  LSHG_CUDA(cudaStreamSynchronize(s));
  query_error(*idx, s);
  float scan = 0;
  cudaEventElapsedTime(&scan, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  (void)t0;
  res->preprocess_us = prep * 1e3;
  res->construction_us = build * 1e3;
  res->scan_us = scan * 1e3;
  res->preprocess_ms = (int64_t)prep;
  res->construction_ms = (int64_t)build;
  res->scan_ms = (int64_t)scan;
  res->recall = 0;
  res->avg_distance = 0;
}

}  // namespace

extern "C" {

const char* lshg_version(void) { return "lshg 0.1 (sm_103a)"; }
const char* lshg_last_error(void) { return g_last_error.c_str(); }
int lshg_calculate_k(int k) { return ((k - 1) / 32) * 32 + 32; }
int64_t lshg_launch_count(void) { return launch_counter().load(); }

void lshg_options_default(lshg_options* opt) {
  if (!opt) return;
  opt->thread_queue_size = 128;
  opt->candidates = 0;
  opt->cp_hashes = 1;
  opt->cp_rounds = 3;
  opt->stream = nullptr;
  opt->fp64_recheck = -1;
  opt->sketch_scan = 0;
}

int lshg_linear_scans_ex(int implementation, int k, int d, int N_query, int N_data, const float* data,
                         const float* queries, int sketchDim, int distanceFunc, const lshg_options* opt,
                         lshg_result* res) {
  return guarded([&] {
    lshg_index_params p{};
    p.implementation = implementation;
    p.distanceFunc = distanceFunc;
    p.sketchDim = sketchDim;
    p.d = d;
    p.framework = 0;
    if (opt) p.opt = *opt; else lshg_options_default(&p.opt);
    run_reference_call(p, k, N_query, N_data, data, queries, res);
  });
}

int lshg_linear_scans(int implementation, int k, int d, int N_query, int N_data, const float* data,
                      const float* queries, int sketchDim, int distanceFunc, lshg_result* res) {
  return lshg_linear_scans_ex(implementation, k, d, N_query, N_data, data, queries, sketchDim, distanceFunc, nullptr,
                              res);
}

int lshg_lsh_ex(int implementation, int keysImplementation, int k, int d, int N_query, int N_data, const float* data,
                const float* queries, int sketchDim, int distanceFunc, int bucketKeyBits, int tables,
                int runWithSketchedData, const lshg_options* opt, lshg_result* res) {
  return guarded([&] {
    lshg_index_params p{};
    p.implementation = implementation;
    p.distanceFunc = distanceFunc;
    p.sketchDim = sketchDim;
    p.d = d;
    p.framework = 1;
    p.keysImplementation = keysImplementation;
    p.bucketKeyBits = bucketKeyBits;
    p.tables = tables;
    p.runWithSketchedData = runWithSketchedData;
    if (opt) p.opt = *opt; else lshg_options_default(&p.opt);
    run_reference_call(p, k, N_query, N_data, data, queries, res);
  });
}

int lshg_lsh(int implementation, int keysImplementation, int k, int d, int N_query, int N_data, const float* data,
             const float* queries, int sketchDim, int distanceFunc, int bucketKeyBits, int tables,
             int runWithSketchedData, lshg_result* res) {
  return lshg_lsh_ex(implementation, keysImplementation, k, d, N_query, N_data, data, queries, sketchDim,
                     distanceFunc, bucketKeyBits, tables, runWithSketchedData, nullptr, res);
}

int lshg_random_normals(int64_t count, double stddev, float* out) {
  return guarded([&] {
    LSHG_REQUIRE(out && count >= 0, "invalid arguments");
    random_normals(count, stddev, out);
  });
}
int lshg_random_plus_minus(int64_t count, int32_t* out) {
  return guarded([&] {
    LSHG_REQUIRE(out && count >= 0, "invalid arguments");
    random_plus_minus(count, out);
  });
}
int lshg_random_bools(int64_t count, uint8_t* out) {
  return guarded([&] {
    LSHG_REQUIRE(out && count >= 0, "invalid arguments");
    random_bools(count, out);
  });
}

// ---- index -----------------------------------------------------------------------

int lshg_index_build(const lshg_index_params* p, const float* data, int64_t N_data, int data_on_device,
                     lshg_index** out) {
  return guarded([&] {
    LSHG_REQUIRE(p && data && out, "NULL argument");
    require_device();
    bool own = false;
    cudaStream_t s = pick_stream(&p->opt, &own);
    DevBuf<float> base((size_t)N_data * p->d, s);
    LSHG_CUDA(cudaMemcpyAsync(base.ptr, data, base.bytes(), data_on_device ? cudaMemcpyDeviceToDevice
                                                                           : cudaMemcpyHostToDevice, s));
    std::unique_ptr<Index> idx;
    try {
      idx = build_index(*p, std::move(base), N_data, nullptr, 0, s, nullptr, nullptr);
    } catch (...) {
      if (own) cudaStreamDestroy(s);
      throw;
    }
    idx->own_stream = own;
    LSHG_CUDA(cudaStreamSynchronize(s));
    lshg_index* h = new lshg_index();
    h->impl = std::move(idx);
    *out = h;
  });
}

int lshg_index_query(lshg_index* idx, const float* queries, int N_query, int k, lshg_point* results, int on_device,
                     void* stream) {
  return guarded([&] {
    LSHG_REQUIRE(idx && results && (queries || N_query == 0), "NULL argument");
    Index& I = *idx->impl;
    check_device(I);
    cudaStream_t s = stream ? (cudaStream_t)stream : I.stream;
    DevBuf<float> q((size_t)N_query * I.d, s);
    if (N_query)
      LSHG_CUDA(cudaMemcpyAsync(q.ptr, queries, q.bytes(), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                s));
    if (on_device) {
      query_index(I, q.ptr, N_query, k, results, s);
    } else {
      DevBuf<lshg_point> out((size_t)N_query * k, s);
      query_index(I, q.ptr, N_query, k, out.ptr, s);
      if (N_query)
        LSHG_CUDA(cudaMemcpyAsync(results, out.ptr, out.bytes(), cudaMemcpyDeviceToHost, s));
    }
    LSHG_CUDA(cudaStreamSynchronize(s));
    query_error(I, s);
  });
}

int lshg_index_query_async(lshg_index* idx, const float* queries, int N_query, int k, lshg_point* results,
                           int on_device, void* stream) {
  return guarded([&] {
    LSHG_REQUIRE(idx && results && (queries || N_query == 0), "NULL argument");
    Index& I = *idx->impl;
    check_device(I);
    cudaStream_t s = stream ? (cudaStream_t)stream : I.stream;
    // the pipelines preprocess queries in place: work on a stream-ordered copy
    DevBuf<float> q((size_t)N_query * I.d, s);
    if (N_query)
      LSHG_CUDA(cudaMemcpyAsync(q.ptr, queries, q.bytes(), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                s));
    if (on_device) {
      query_index(I, q.ptr, N_query, k, results, s);
    } else {
      DevBuf<lshg_point> out((size_t)N_query * k, s);
      query_index(I, q.ptr, N_query, k, out.ptr, s);
      if (N_query)
        LSHG_CUDA(cudaMemcpyAsync(results, out.ptr, out.bytes(), cudaMemcpyDeviceToHost, s));
    }
  });
}

int lshg_index_sync(lshg_index* idx, void* stream) {
  return guarded([&] {
    LSHG_REQUIRE(idx, "NULL argument");
    Index& I = *idx->impl;
    check_device(I);
    cudaStream_t s = stream ? (cudaStream_t)stream : I.stream;
    LSHG_CUDA(cudaStreamSynchronize(s));
    query_error(I, s);
  });
}

int lshg_index_free(lshg_index* idx) {
  return guarded([&] {
    if (!idx) return;
    // release on the index's device, whatever the calling thread's current device is
    int cur = -1;
    LSHG_CUDA(cudaGetDevice(&cur));
    const int dev = idx->impl ? idx->impl->device : cur;
    if (dev != cur) LSHG_CUDA(cudaSetDevice(dev));
    delete idx;
    if (dev != cur) LSHG_CUDA(cudaSetDevice(cur));
  });
}

int lshg_index_export(lshg_index* idx, int what, void* dst, size_t* bytes) {
  return guarded([&] {
    LSHG_REQUIRE(idx && bytes, "NULL argument");
    Index& I = *idx->impl;
    check_device(I);
    cudaStream_t s = I.stream;
    const void* src = nullptr;
    size_t nb = 0;
    switch (what) {
      case 0: src = I.x.ptr; nb = I.x.bytes(); break;
      case 1:
        if (I.sk_kind == 6) { src = I.xsf.ptr; nb = I.xsf.bytes(); }
        else if (I.sk_kind == 4) nb = (size_t)I.n * I.sbytes;
        else if (I.sk_kind) nb = (size_t)I.n * I.words * 4;
        break;
      case 2: src = I.keys.ptr; nb = I.keys.bytes(); break;
      case 3: src = I.offsets.ptr; nb = I.offsets.bytes(); break;
      case 4: src = I.buckets.ptr; nb = I.buckets.bytes(); break;
      case 5: src = I.qstats.ptr; nb = I.qstats.bytes(); break;
      case 6: nb = 6 * sizeof(int32_t); break;
      default: throw Error(LSHG_ERR_INVALID_ARGUMENT, "unknown export item");
    }
    *bytes = nb;
    if (!dst || nb == 0) return;
    if (what == 6) {  // CWS code plan (zeros for other sketch kinds)
      const int32_t plan[6] = {I.cws.tmin, I.cws.tmax, I.cws.kb, I.cws.tb, I.sk_kind == 10 ? I.cws.pl : 0,
                               I.cws.dict};
      memcpy(dst, plan, sizeof plan);
      return;
    }
    if (what == 1 && (I.sk_kind == 3 || I.sk_kind == 5 || I.sk_kind == 4 || I.sk_kind == 10)) {
      std::vector<uint32_t> rows((size_t)I.n * I.wp);
      LSHG_CUDA(cudaMemcpyAsync(rows.data(), I.xs.ptr, rows.size() * 4, cudaMemcpyDeviceToHost, s));
      LSHG_CUDA(cudaStreamSynchronize(s));
      if (I.sk_kind == 4) {
        uint8_t* o = (uint8_t*)dst;
        for (int64_t i = 0; i < I.n; ++i) memcpy(o + i * I.sbytes, &rows[(size_t)i * I.wp], I.sbytes);
      } else {
        uint32_t* o = (uint32_t*)dst;
        for (int64_t i = 0; i < I.n; ++i) memcpy(o + i * I.words, &rows[(size_t)i * I.wp], (size_t)I.words * 4);
      }
      return;
    }
    LSHG_CUDA(cudaMemcpyAsync(dst, src, nb, cudaMemcpyDeviceToHost, s));
    LSHG_CUDA(cudaStreamSynchronize(s));
    if (what == 4) {  // ascending ids within each bucket
      std::vector<int> off((size_t)I.tables * I.tableSize);
      LSHG_CUDA(cudaMemcpy(off.data(), I.offsets.ptr, off.size() * 4, cudaMemcpyDeviceToHost));
      int* b = (int*)dst;
      for (int t = 0; t < I.tables; ++t)
        for (int key = 0; key < I.tableSize; ++key) {
          int st = off[(size_t)t * I.tableSize + key];
          int en = key + 1 < I.tableSize ? off[(size_t)t * I.tableSize + key + 1] : (int)(t * I.n + I.n);
          std::sort(b + st, b + en);
        }
    }
  });
}

int lshg_index_sketch_queries(lshg_index* idx, const float* queries, int N_query, void* sketches, uint16_t* keys) {
  return guarded([&] {
    LSHG_REQUIRE(idx && queries, "NULL argument");
    Index& I = *idx->impl;
    check_device(I);
    cudaStream_t s = I.stream;
    DevBuf<float> q = upload_floats(queries, (size_t)N_query * I.d, s);
    DevBuf<uint32_t> qs;
    DevBuf<float> qsf;
    DevBuf<uint16_t> qk;
    sketch_queries(I, q.ptr, N_query, &qs, &qsf, keys ? &qk : nullptr, s);
    query_error(I, s);
    if (keys && I.p.framework == 1)
      LSHG_CUDA(cudaMemcpyAsync(keys, qk.ptr, qk.bytes(), cudaMemcpyDeviceToHost, s));
    if (sketches && I.sk_kind == 6)
      LSHG_CUDA(cudaMemcpyAsync(sketches, qsf.ptr, qsf.bytes(), cudaMemcpyDeviceToHost, s));
    std::vector<uint32_t> rows;
    if (sketches && I.sk_kind && I.sk_kind != 6) {
      rows.resize((size_t)N_query * I.wp);
      LSHG_CUDA(cudaMemcpyAsync(rows.data(), qs.ptr, rows.size() * 4, cudaMemcpyDeviceToHost, s));
    }
    LSHG_CUDA(cudaStreamSynchronize(s));
    if (!rows.empty()) {
      for (int i = 0; i < N_query; ++i) {
        if (I.sk_kind == 4) memcpy((uint8_t*)sketches + (size_t)i * I.sbytes, &rows[(size_t)i * I.wp], I.sbytes);
        else memcpy((uint32_t*)sketches + (size_t)i * I.words, &rows[(size_t)i * I.wp], (size_t)I.words * 4);
      }
    }
  });
}

// ---- sharding --------------------------------------------------------------------

int lshg_merge_topk(const lshg_point* lists, int shards, int N_query, int k_in, int k, lshg_point* out) {
  return guarded([&] {
    LSHG_REQUIRE(lists && out && shards >= 1 && k_in >= 1 && k >= 1, "invalid arguments");
    std::vector<uint64_t> keys;
    for (int q = 0; q < N_query; ++q) {
      keys.clear();
      for (int s = 0; s < shards; ++s)
        for (int i = 0; i < k_in; ++i) {
          const lshg_point& p = lists[((size_t)s * N_query + q) * k_in + i];
          if (p.ID >= 0) keys.push_back(make_key(p.distance, p.ID));
        }
      std::sort(keys.begin(), keys.end());
      int w = 0;
      int prev = -1;
      for (size_t i = 0; i < keys.size() && w < k; ++i) {
        int id = key_id(keys[i]);
        if (id == prev) continue;
        bool seen = false;  // same id from two shards with different distances
        for (int j = 0; j < w && !seen; ++j) seen = out[(size_t)q * k + j].ID == id;
        if (seen) continue;
        out[(size_t)q * k + w].ID = id;
        out[(size_t)q * k + w].distance = key_dist(keys[i]);
        ++w;
        prev = id;
      }
      for (; w < k; ++w) {
        out[(size_t)q * k + w].ID = -1;
        out[(size_t)q * k + w].distance = kEmptyDistance;
      }
    }
  });
}

// ---- validation (validation.cpp:129-208) ------------------------------------------

int lshg_validate(const lshg_point* truth, int truth_k, const lshg_point* results, int N_query, int k, int reportK,
                  float* recall, float* distance_ratio) {
  return guarded([&] {
    LSHG_REQUIRE(truth && results && recall && distance_ratio, "NULL argument");
    LSHG_REQUIRE(reportK >= 1 && reportK <= k && reportK <= truth_k, "reportK out of range");
    float total_recall = 0, total_ratio = 0;
    for (int q = 0; q < N_query; ++q) {
      // result set: first reportK entries, as a set by ID (readData, validation.cpp:39-60)
      std::set<int> ids;
      std::vector<std::pair<int, float>> uniq;
      for (int i = 0; i < reportK; ++i) {
        const lshg_point& p = results[(size_t)q * k + i];
        if (ids.insert(p.ID).second) uniq.push_back({p.ID, p.distance});
      }
      float rec = 0;
      float tdist = 0;
      for (int i = 0; i < reportK; ++i) {
        const lshg_point& t = truth[(size_t)q * truth_k + i];
        if (ids.count(t.ID)) rec += 1;
        tdist += t.distance;
      }
      float rdist = 0;
      std::sort(uniq.begin(), uniq.end());  // std::set iteration order (by ID)
      for (auto& u : uniq) rdist += u.second;
      total_recall += rec / reportK;
      total_ratio += rdist / tdist;
    }
    *recall = N_query ? total_recall / N_query : 0;
    *distance_ratio = N_query ? total_ratio / N_query : 0;
  });
}

// ---- reference text format (gloveparser.cu:9-86; DataParsing/Writer/writer.cpp) --
//
// A file is a line with n, a line with d, then a line a point: "<id> v v ... v " with a
// space after every value.  Values are read by the reference reader's rules, kept because
// existing files (and the ground truth computed from them) went through that reader:
//   * the first space-separated field of a line (the id) is skipped;
//   * a value is stored when the space after it is read: a field that ends its line or
//     the file is dropped, and two spaces in a row store a zero;
//   * in a value field only '0'-'9', '-' and '.' count, every other byte is skipped:
//       - a digit before any '.' replaces the value ("12.5" reads 2.5, "1e3" reads 3);
//       - every '.' and every digit after one advance a place count e, and such a digit c
//         adds c / 10^e, in double, to the float value ("1.2.3" reads 1.203);
//       - a '-' anywhere in the field negates the stored value; the sign is cleared only
//         when a value is stored, so the '-' of a dropped field at a line end carries over
//         to the next stored value.

namespace {

// Value of one field by the rules above; `neg` is set by a '-' and left set otherwise.
float field_value(const unsigned char* b, const unsigned char* e, bool& neg) {
  float v = 0.0f;
  int places = 0;  // 0: no '.' seen yet
  for (; b < e; ++b) {
    const unsigned c = *b;
    if (c >= '0' && c <= '9') {
      if (places == 0) {
        v = (float)(c - 48.0);
      } else {
        v = (float)(v + (c - 48.0) / std::pow(10.0, (double)places));
        ++places;
      }
    } else if (c == '-') {
      neg = true;
    } else if (c == '.') {
      ++places;
    }
  }
  return v;
}

}  // namespace

int lshg_parse_file(const char* path, int* n_out, int* d_out, float** out) {
  return guarded([&] {
    LSHG_REQUIRE(path && n_out && d_out && out, "NULL argument");
    FILE* fp = fopen(path, "r");
    if (!fp) throw Error(LSHG_ERR_IO, std::string("Error while opening file: ") + path);
    char nb[256], db[256];
    if (!fgets(nb, sizeof nb, fp) || !fgets(db, sizeof db, fp)) {
      fclose(fp);
      throw Error(LSHG_ERR_IO, "truncated header");
    }
    const int n = atoi(nb), d = atoi(db);
    if (n < 0 || d <= 0) {
      fclose(fp);
      throw Error(LSHG_ERR_IO, "bad header");
    }
    std::vector<unsigned char> text;
    unsigned char chunk[1 << 16];
    for (size_t got; (got = fread(chunk, 1, sizeof chunk, fp)) > 0;) text.insert(text.end(), chunk, chunk + got);
    fclose(fp);
    const size_t cap = (size_t)n * d;
    float* vals = (float*)calloc(cap + 1, sizeof(float));
    if (!vals) throw Error(LSHG_ERR_OUT_OF_MEMORY, "cannot allocate the dataset");
    const unsigned char* t = text.data();
    const unsigned char* end = t + text.size();
    size_t stored = 0;
    bool neg = false;
    for (const unsigned char* line = t; line < end;) {
      const unsigned char* eol = std::find(line, end, (unsigned char)'\n');
      const unsigned char* f = std::find(line, eol, (unsigned char)' ');  // end of the id
      while (f < eol) {
        const unsigned char* b = f + 1;
        f = std::find(b, eol, (unsigned char)' ');
        float v = field_value(b, f, neg);
        if (f == eol) break;  // no space after the field: dropped
        if (neg) v = -v;
        neg = false;
        if (stored < cap) vals[stored] = v;
        ++stored;
      }
      line = eol + 1;
    }
    *n_out = n;
    *d_out = d;
    *out = vals;
  });
}

int lshg_write_file(const char* path, const float* x, int n, int d) {
  return guarded([&] {
    LSHG_REQUIRE(path && (x || n == 0), "NULL argument");
    FILE* fp = fopen(path, "w");
    if (!fp) throw Error(LSHG_ERR_IO, std::string("cannot open ") + path);
    fprintf(fp, "%d\n%d\n", n, d);
    for (int i = 0; i < n; ++i) {
      fprintf(fp, "%d ", i);
      for (int j = 0; j < d; ++j) fprintf(fp, "%.6f ", x[(size_t)i * d + j]);
      fprintf(fp, "\n");
    }
    fclose(fp);
  });
}

void lshg_free(void* p) { free(p); }

int lshg_read_truth(const char* path, int* n_out, int* k_out, lshg_point** out) {
  return guarded([&] {
    LSHG_REQUIRE(path && n_out && k_out && out, "NULL argument");
    std::ifstream f(path);
    if (!f) throw Error(LSHG_ERR_IO, std::string("cannot open ") + path);
    int n = 0, k = 0;
    f >> n >> k;
    if (!f || n < 0 || k < 0) throw Error(LSHG_ERR_IO, "bad truth-file header");
    lshg_point* pts = (lshg_point*)malloc(sizeof(lshg_point) * ((size_t)n * k + 1));
    std::string qid;
    for (int q = 0; q < n; ++q) {
      f >> qid;
      for (int i = 0; i < k; ++i) {
        int id = 0;
        float dist = 0;
        f >> id >> dist;
        pts[(size_t)q * k + i].ID = id;
        pts[(size_t)q * k + i].distance = dist;
      }
    }
    if (!f) {
      free(pts);
      throw Error(LSHG_ERR_IO, "truncated truth file");
    }
    *n_out = n;
    *k_out = k;
    *out = pts;
  });
}

}  // extern "C"
