// Harness that runs the reference's own GPU kernels -- TEST INFRASTRUCTURE ONLY.
//
// oracle/build.py compiles the reference's unmodified LinearScan translation units to
// sm_103a cubins (oracle/_ref/ref_*.cubin) and records the mangled names of the kernels
// below (oracle/_ref/ref_kernels.txt).  This file loads those cubins with the CUDA driver
// API and launches the kernels with the reference's launch shapes and argument layouts,
// so tests can compare the engine with the reference GPU path bit for bit.
//
// Only kernels whose synchronisation is well defined for the inputs used are driven:
//   knn (memOptimizedLinearScan.cu:20-106)   with N_data a multiple of 32, so no lane
//                                            leaves the scan loop before the warp-wide
//                                            ballots (sketchedDistanceScanners.cuh:74);
//   simHash::sketch (simHash.cu:22-47), simHashJl::sketch (simHashJL.cuh:34-51),
//   crosspoly::generateHashCrossPoly (crossPolyTope.cuh:25-85): no synchronisation;
//   weightedMinHash::sketchDataOriginal / sketchDataOneBit (weightedMinHash.cuh:109-166):
//                                            callers first check on the CPU that every
//                                            sample ends within 4096 draws; the index map
//                                            gets one extra zero entry and the bit map is
//                                            padded to 65536 zero entries, so the reads
//                                            the reference makes past its arrays
//                                            (map[M], randomBitMap[counter >= 255]) stay
//                                            inside allocated memory.
// The LSH scan kernel (lshFramework.cuh:142-252) is not driven: its ballots run with
// lanes that have left their bucket loops, which is undefined on independent-thread-
// scheduling GPUs.
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

namespace {

// Layout of LaunchDTO<T> (launchDTO.h:5-25) for any pointer type T.
struct RefLaunchDTO {
  int implementation;
  int distanceFunc;
  float* data;
  float* queries;
  int N_data;
  int N_queries;
  int dimensions;
  void* sketchedData;
  void* sketchedQueries;
  int sketchedDataSize;
  int sketchedQueriesSize;
  int sketchDim;
  int k;
  int dataSize;
  int querySize;
  int resultSize;
  void* results;
};

struct RefPoint {
  int ID;
  float distance;
};

std::string g_err;
std::map<std::string, CUfunction> g_fn;
std::map<std::string, CUmodule> g_mod;
CUcontext g_ctx = nullptr;

#define RH(call)                                                   \
  do {                                                             \
    CUresult _r = (call);                                          \
    if (_r != CUDA_SUCCESS) {                                      \
      const char* s = nullptr;                                     \
      cuGetErrorString(_r, &s);                                    \
      g_err = std::string(#call) + ": " + (s ? s : "?");           \
      return 1;                                                    \
    }                                                              \
  } while (0)

// calculateThreadsLocal / calculateBlocksLocal (launchHelper.cuh:9-19)
int threads_local(int q) { return q * 32 < 1024 ? q * 32 : 1024; }
int blocks_local(int q) { return q * 32 < 1024 ? 1 : (q + 31) / 32; }

struct Dev {
  CUdeviceptr p = 0;
  ~Dev() {
    if (p) cuMemFree(p);
  }
};

int upload(Dev& d, const void* h, size_t bytes) {
  RH(cuMemAlloc(&d.p, bytes ? bytes : 4));
  if (bytes && h) RH(cuMemcpyHtoD(d.p, h, bytes));
  return 0;
}

int launch(const char* tag, int grid, int block, void** args) {
  auto it = g_fn.find(tag);
  if (it == g_fn.end()) {
    g_err = std::string("kernel not loaded: ") + tag;
    return 1;
  }
  RH(cuLaunchKernel(it->second, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr));
  RH(cuCtxSynchronize());
  return 0;
}

}  // namespace

extern "C" {

const char* rh_error(void) { return g_err.c_str(); }

// Load every cubin listed in <dir>/ref_kernels.txt ("tag cubin mangled-name" lines).
int rh_init(const char* dir) {
  RH(cuInit(0));
  CUdevice dev;
  RH(cuDeviceGet(&dev, 0));
  RH(cuDevicePrimaryCtxRetain(&g_ctx, dev));
  RH(cuCtxSetCurrent(g_ctx));
  std::ifstream f(std::string(dir) + "/ref_kernels.txt");
  if (!f) {
    g_err = "ref_kernels.txt not found";
    return 1;
  }
  std::string tag, cubin, name;
  while (f >> tag >> cubin >> name) {
    if (!g_mod.count(cubin)) {
      CUmodule m;
      RH(cuModuleLoad(&m, (std::string(dir) + "/" + cubin).c_str()));
      g_mod[cubin] = m;
    }
    CUfunction fn;
    RH(cuModuleGetFunction(&fn, g_mod[cubin], name.c_str()));
    g_fn[tag] = fn;
  }
  return 0;
}

// knn with the reference's shape: threads/2, blocks*2 (memOptimizedLinearScan.cu:131-136).
int rh_knn(const float* data, int n, const float* q, int nq, int d, int k, int func, int32_t* ids, float* dists,
           float* ms) {
  if (n % 32) {
    g_err = "N_data must be a multiple of 32";
    return 1;
  }
  RH(cuCtxSetCurrent(g_ctx));
  Dev dq, dd, dr;
  if (upload(dq, q, (size_t)nq * d * 4) || upload(dd, data, (size_t)n * d * 4) ||
      upload(dr, nullptr, (size_t)nq * k * sizeof(RefPoint)))
    return 1;
  int threads = threads_local(nq) / 2, blocks = blocks_local(nq) * 2;
  void* args[] = {&dq.p, &dd.p, &nq, &n, &d, &k, &dr.p, &func};
  CUevent a, b;
  RH(cuEventCreate(&a, CU_EVENT_DEFAULT));
  RH(cuEventCreate(&b, CU_EVENT_DEFAULT));
  RH(cuEventRecord(a, nullptr));
  if (launch("knn", blocks, threads, args)) return 1;
  RH(cuEventRecord(b, nullptr));
  RH(cuEventSynchronize(b));
  if (ms) RH(cuEventElapsedTime(ms, a, b));
  cuEventDestroy(a);
  cuEventDestroy(b);
  std::vector<RefPoint> out((size_t)nq * k);
  RH(cuMemcpyDtoH(out.data(), dr.p, out.size() * sizeof(RefPoint)));
  for (size_t i = 0; i < out.size(); ++i) {
    ids[i] = out[i].ID;
    dists[i] = out[i].distance;
  }
  return 0;
}

int rh_simhash(const float* x, int n, int launch_q, int d, const float* planes, int words, uint32_t* out) {
  RH(cuCtxSetCurrent(g_ctx));
  Dev dx, dp, dout;
  if (upload(dx, x, (size_t)n * d * 4) || upload(dp, planes, (size_t)words * 32 * d * 4) ||
      upload(dout, nullptr, (size_t)n * words * 4))
    return 1;
  void* args[] = {&dx.p, &dp.p, &n, &d, &words, &dout.p};
  if (launch("simhash_sketch", blocks_local(launch_q), threads_local(launch_q), args)) return 1;
  RH(cuMemcpyDtoH(out, dout.p, (size_t)n * words * 4));
  return 0;
}

int rh_jl(const float* x, int n, int launch_q, int d, const float* R, int sdim, float* out) {
  RH(cuCtxSetCurrent(g_ctx));
  Dev dx, dR, dout;
  if (upload(dx, x, (size_t)n * d * 4) || upload(dR, R, (size_t)sdim * d * 4) ||
      upload(dout, nullptr, (size_t)n * sdim * 4))
    return 1;
  RefLaunchDTO dto{};
  dto.dimensions = d;
  dto.sketchDim = sdim;
  void* args[] = {&dto, &dx.p, &dR.p, &n, &dout.p};
  if (launch("jl_sketch", blocks_local(launch_q), threads_local(launch_q), args)) return 1;
  RH(cuMemcpyDtoH(out, dout.p, (size_t)n * sdim * 4));
  return 0;
}

int rh_crosspoly(const float* x, int n, int launch_q, int d, int P, int tables, const int32_t* diag, uint16_t* keys) {
  RH(cuCtxSetCurrent(g_ctx));
  const int blocks = blocks_local(launch_q), threads = threads_local(launch_q);
  const size_t scratch = (size_t)blocks * threads * P * 4;
  Dev dx, dk, ddiag, dpart, dtmp;
  if (upload(dx, x, (size_t)n * d * 4) || upload(dk, nullptr, (size_t)n * tables * 2) ||
      upload(ddiag, diag, (size_t)P * tables * 3 * 4) || upload(dpart, nullptr, scratch) ||
      upload(dtmp, nullptr, scratch))
    return 1;
  RefLaunchDTO dto{};
  dto.dimensions = d;
  void* args[] = {&dto, &dx.p, &dk.p, &n, &tables, &ddiag.p, &dpart.p, &dtmp.p, &P};
  if (launch("crosspoly", blocks, threads, args)) return 1;
  RH(cuMemcpyDtoH(keys, dk.p, (size_t)n * tables * 2));
  return 0;
}

// Rejection-sampled MinHash on preprocessed rows x with the given start offsets / map.
// onebit = 0: out is u8 [n][H]; onebit = 1: out is u32 [n][words] (H = words*hashBits).
int rh_wmh(const float* x, int n, int launch_q, int d, const int32_t* start, const int32_t* map, int M, int H,
           int onebit, int words, int hashBits, const uint8_t* bitmap, int bitmap_len, void* out) {
  RH(cuCtxSetCurrent(g_ctx));
  std::vector<int32_t> seeds(H), mp(map, map + M);
  for (int h = 0; h < H; ++h) seeds[h] = h * 1234 + 92138;  // createSeedArr (weightedMinHash.cuh:252-262)
  mp.push_back(0);
  std::vector<uint8_t> bm(65536, 0);
  memcpy(bm.data(), bitmap, bitmap_len);
  const size_t out_bytes = onebit ? (size_t)n * words * 4 : (size_t)n * H;
  Dev dx, dstart, dmap, dseeds, dbm, dout;
  if (upload(dx, x, (size_t)n * d * 4) || upload(dstart, start, (size_t)d * 4) ||
      upload(dmap, mp.data(), mp.size() * 4) || upload(dseeds, seeds.data(), (size_t)H * 4) ||
      upload(dbm, bm.data(), bm.size()) || upload(dout, nullptr, out_bytes))
    return 1;
  RefLaunchDTO dto{};
  dto.dimensions = d;
  const int blocks = blocks_local(launch_q), threads = threads_local(launch_q);
  if (onebit) {
    void* args[] = {&dto, &dx.p, &n, &words, &hashBits, &dmap.p, &dstart.p, &M, &dseeds.p, &dbm.p, &dout.p};
    if (launch("wmh_onebit", blocks, threads, args)) return 1;
  } else {
    void* args[] = {&dto, &dx.p, &n, &H, &dmap.p, &dstart.p, &M, &dseeds.p, &dout.p};
    if (launch("wmh_byte", blocks, threads, args)) return 1;
  }
  RH(cuMemcpyDtoH(out, dout.p, out_bytes));
  return 0;
}

}  // extern "C"
