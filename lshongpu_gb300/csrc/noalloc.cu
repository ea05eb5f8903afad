// Allocation-free query entry point for the exact linear-scan index.
//
// Some callers cannot allocate device memory while they answer queries: a serving
// process whose free HBM is already owned by another allocator (a framework's caching
// allocator reserves it up front), or a latency-critical thread that must not enter the
// CUDA allocator at all (growing the stream-ordered pool can block).  For them,
// lshg_index_query_noalloc runs the same kernels as lshg_index_query for an exact
// angular index (implementation 2, linear scan) but takes every temporary -- query
// magnitudes, the per-split candidate lists and their merge -- from one file-scope
// device array of kNoAllocScratchBytes.  Nothing is allocated or freed on any call.
//
// Properties the caller must respect:
//  * the array exists once per GPU that loads this library and stays allocated until
//    the process exits;
//  * every call shares it, so calls that overlap on the GPU (different streams or
//    threads without ordering) race on it -- serialise them;
//  * it keeps the previous call's contents; nothing in it is read before being written
//    in the same call;
//  * the first call on each device looks the array's device address up
//    (cudaGetSymbolAddress, with that device current); make that first call before any
//    stream capture begins;
//  * the calling thread's current device must be the index's device (the call is
//    rejected with LSHG_ERR_INVALID_ARGUMENT otherwise), so the array used is the one on
//    the GPU that holds the index.
//  * batches whose temporaries exceed the array are rejected with
//    LSHG_ERR_INVALID_ARGUMENT.
#include <mutex>

#include "index.h"
#include "launch_count.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `dev`, which must be the calling thread's current
// device (the caller has checked that it is the index's device); looked up once per device.
void* scratch_for_device(int dev) {
  if (dev < 0 || dev >= kMaxDevices) throw lshg::Error(LSHG_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    LSHG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (!p) throw lshg::Error(LSHG_ERR_CUDA, "cudaGetSymbolAddress returned NULL for the query scratch");
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

}  // namespace

namespace lshg {
void set_last_error(const char* msg);
}

using namespace lshg;

extern "C" int lshg_index_query_noalloc(lshg_index* idx, const float* d_queries, int N_query, int k,
                                        lshg_point* d_results, void* stream) {
  try {
    if (!idx || !idx->impl || !d_results || (!d_queries && N_query > 0))
      throw Error(LSHG_ERR_INVALID_ARGUMENT, "NULL argument");
    Index& I = *idx->impl;
    check_device(I);  // the scratch array and the index's buffers are on the same GPU
    const int impl = I.p.implementation == 1 ? 2 : I.p.implementation;
    if (I.p.framework != 0 || impl != 2 || I.dist != DIST_ANGULAR)
      throw Error(LSHG_ERR_UNSUPPORTED, "the allocation-free query serves exact angular linear-scan indexes only");
    if (k < 1 || k > 4096) throw Error(LSHG_ERR_INVALID_ARGUMENT, "k must be in [1, 4096]");
    if (N_query <= 0) return LSHG_OK;
    cudaStream_t s = stream ? (cudaStream_t)stream : I.stream;
    const int C = std::max(32, next_pow2(k));
    const int splits = scan_float_splits(I.n, N_query, C);
    const size_t qn_bytes = align256((size_t)N_query * sizeof(float));
    const size_t part_bytes = align256((size_t)N_query * splits * C * sizeof(uint64_t));
    const size_t merged_bytes = splits > 1 ? align256((size_t)N_query * C * sizeof(uint64_t)) : 0;
    const size_t need = qn_bytes + part_bytes + merged_bytes;
    if (need > kNoAllocScratchBytes)
      throw Error(LSHG_ERR_INVALID_ARGUMENT,
                  "query batch needs " + std::to_string(need) + " bytes of temporaries; the allocation-free entry "
                  "point has " + std::to_string(kNoAllocScratchBytes) + " (use fewer queries or a smaller k)");
    unsigned char* base = static_cast<unsigned char*>(scratch_for_device(I.device));
    float* qnorm = reinterpret_cast<float*>(base);
    uint64_t* part = reinterpret_cast<uint64_t*>(base + qn_bytes);
    uint64_t* merged = reinterpret_cast<uint64_t*>(base + qn_bytes + part_bytes);
    launch_row_norms(d_queries, N_query, I.d, qnorm, s);
    launch_scan_float(I.xt.ptr, I.n, I.d, I.xnorm.ptr, d_queries, N_query, qnorm, DIST_ANGULAR, C, splits, part, s);
    const uint64_t* keys = part;
    if (splits > 1) {
      launch_merge_splits(part, N_query, splits, C, merged, s);
      keys = merged;
    }
    launch_keys_to_points(keys, N_query, C, k, d_results, s);
    return LSHG_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  }
}
