/*
 * lshg.h - C ABI of the GB300-native k-NN / LSH engine (liblshg.so).
 *
 * Drop-in boundary for the reference's launch surface (peturssonstefan/LSHonGPU):
 *   Result linearScans(int implementation, int k, int d, int N_query, int N_data,
 *                      float* data, float* queries, int sketchDim, int distanceFunc)
 *       -> LinearScan/kernel.cu:27
 *   Result LSH(int implementation, int keysImplementation, int k, int d, int N_query,
 *              int N_data, float* data, float* queries, int sketchDim, int distanceFunc,
 *              int bucketKeyBits, int tables, bool runWithSketchedData)
 *       -> LinearScan/kernel.cu:91 (which reaches runLsh<T,K>, lshFramework.cuh:313)
 * plus a resident-index API for serving, the host random generators the reference
 * uses for its projections, the validation of recall / distance ratio, and the
 * reference text dataset format.
 *
 * Conventions: plain pointers and sizes; host pointers unless a parameter says
 * otherwise; every function returns an lshg_status and never exits the process; the
 * device is the calling thread's current CUDA device and is never reset (the
 * reference calls cudaDeviceReset() after every pipeline, e.g. simHash.cu:141).
 *
 * Codes (kernel.cu:25, kernel.cu:65-85, distanceFunctions.cuh:54-71):
 *   implementation:      1 = exact (the reference's defunct impl 1 is served by the
 *                            exact scan), 2 = exact linear scan, 3 = SimHash,
 *                            4 = weighted MinHash (byte), 5 = one-bit weighted MinHash,
 *                            6 = Johnson-Lindenstrauss,
 *                            8 = tensor-core exact scan (BF16, no reference counterpart),
 *                            9 = the same with E4M3 (FP8) tensor-core scores; both
 *                                return exact FP32 distances of their candidates,
 *                            10 = consistent weighted sampling (Ioffe's ICWS; no
 *                                reference counterpart): sketchDim (index, t) samples,
 *                                a multiple of 32 up to 256, linear scan only, the
 *                                weighted MinHash preprocessing and generalized-Jaccard
 *                                re-rank
 *   keysImplementation:  3 = SimHash, 4 = WMH byte, 5 = one-bit WMH, 7 = cross-polytope,
 *                        10 = consistent weighted sampling (no reference counterpart:
 *                            lshg_options.cp_hashes samples a table hashed into
 *                            bucketKeyBits <= 16 bits, the weighted MinHash preprocessing)
 *   distanceFunc:        1 = angular, 2 = generalized Jaccard, 3 = Euclidean
 */
#ifndef LSHG_H_
#define LSHG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LSHG_ABI_VERSION 2

typedef enum {
  LSHG_OK = 0,
  LSHG_ERR_INVALID_ARGUMENT = 1, /* reference prints "Invalid implementation selected" (kernel.cu:48-51) */
  LSHG_ERR_CUDA = 2,             /* reference: CUDA_CHECK_RETURN -> exit(-1) (cudaHelpers.cuh:8-15) */
  LSHG_ERR_OUT_OF_MEMORY = 3,
  LSHG_ERR_NO_DEVICE = 4,
  LSHG_ERR_UNSUPPORTED = 5,
  LSHG_ERR_SAMPLER_LIMIT = 6, /* weighted-MinHash rejection sampler exceeded its draw limit */
  LSHG_ERR_BUSY = 7,          /* serving admission refused (queue full / not enough free HBM) */
  LSHG_ERR_TIMEOUT = 8,
  LSHG_ERR_IO = 9
} lshg_status;

/* Result element; mirrors struct Point {int ID; float distance;} (point.h:3-7). */
typedef struct lshg_point_s {
  int32_t ID;
  float distance;
} lshg_point;

/* Mirrors struct Result (resultDTO.h:5-32).  `results` is a caller-owned host buffer of
 * N_query * k points (the reference mallocs it inside; here the caller provides it). */
typedef struct lshg_result_s {
  lshg_point* results;
  int64_t preprocess_ms;   /* resultDTO.h:7  */
  int64_t construction_ms; /* resultDTO.h:8  */
  int64_t scan_ms;         /* resultDTO.h:9  */
  float recall;            /* resultDTO.h:10 (set by lshg_validate) */
  float avg_distance;      /* resultDTO.h:11 */
  double preprocess_us;    /* the same three timers with microsecond resolution */
  double construction_us;
  double scan_us;
} lshg_result;

/* Knobs the reference fixes at compile time (constants.cuh:3-11) or does not have. */
typedef struct lshg_options_s {
  int thread_queue_size; /* THREAD_QUEUE_SIZE (constants.cuh:6), default 128; the re-rank
                            candidate set is 32 * thread_queue_size (candidateSetScanner.cuh) */
  int candidates;        /* > 0 overrides 32 * thread_queue_size (rounded up to a power of 2) */
  int cp_hashes;         /* cross-polytope hashes concatenated per table key (reference: 1);
                            CWS keys (keysImplementation 10): samples hashed per table key */
  int cp_rounds;         /* cross-polytope rotation rounds (reference: 3, crossPolyTope.cuh:44) */
  void* stream;          /* cudaStream_t to run on, NULL = a library-owned stream */
  int fp64_recheck;      /* re-score, in double precision on the GPU, the re-ranked candidates
                            whose FP32 distance lies within the FP32 error bound of the k-th
                            one (the run of near-ties around the k-th place), and order them
                            by the FP64 distance (ties: lower index); so the top-k set is the
                            FP64 top-k of the candidates.  Returned distances stay FP32.  -1 (default) = on for the
                            tensor-core scans (8, 9), off elsewhere; 0 = off; 1 = on for every
                            re-ranked scan (3-6, 8, 9).  The exact scan (2) returns the
                            reference's FP32 order. */
  int sketch_scan;       /* Hamming / one-bit Jaccard sketch scans (3, 5) with rows of at most
                            1024 bits: 0 (default) = tensor cores for batches of 64 queries or
                            more, XOR/popcount otherwise; 1 = always XOR/popcount (and no E4M3
                            copy of the sketches is kept); 2 = tensor cores whenever the base
                            allows.  Both give the same candidates (ties: lower index). */
} lshg_options;

/* ---- library ---------------------------------------------------------------------- */
const char* lshg_version(void);
/* Message of the last error raised on the calling thread. */
const char* lshg_last_error(void);
/* calculateK (launchHelper.cuh:21-25): k rounded up to a multiple of 32. */
int lshg_calculate_k(int k);
void lshg_options_default(lshg_options* opt);
/* Number of kernel launches issued by the library so far (all threads). */
int64_t lshg_launch_count(void);
/* Benchmark aid: when enabled, every hot-path kernel launch is bracketed by CUDA events
 * on its own stream.  lshg_profile_report writes "name launches total_ms" lines for
 * the launches since the last report into buf and returns the size needed. */
int lshg_profile_enable(int on);
int lshg_profile_report(char* buf, int cap);

/* ---- reference launch surface ----------------------------------------------------- */
/* linearScans (kernel.cu:27).  `k` is the already-rounded k (calculateK); res->results
 * must hold N_query * k points, ascending distance per query (ties: lower index). */
int lshg_linear_scans(int implementation, int k, int d, int N_query, int N_data, const float* data,
                      const float* queries, int sketchDim, int distanceFunc, lshg_result* res);
int lshg_linear_scans_ex(int implementation, int k, int d, int N_query, int N_data, const float* data,
                         const float* queries, int sketchDim, int distanceFunc, const lshg_options* opt,
                         lshg_result* res);

/* LSH (kernel.cu:91) -> runLsh (lshFramework.cuh:313). */
int lshg_lsh(int implementation, int keysImplementation, int k, int d, int N_query, int N_data,
             const float* data, const float* queries, int sketchDim, int distanceFunc, int bucketKeyBits,
             int tables, int runWithSketchedData, lshg_result* res);
int lshg_lsh_ex(int implementation, int keysImplementation, int k, int d, int N_query, int N_data,
                const float* data, const float* queries, int sketchDim, int distanceFunc, int bucketKeyBits,
                int tables, int runWithSketchedData, const lshg_options* opt, lshg_result* res);

/* ---- host random generators (randomVectorGenerator.cpp, weightedMinHash.cuh) ------ */
/* generateRandomVectors (randomVectorGenerator.cpp:5-53): `count` draws of
 * normal_distribution<double>(0, stddev) from a default-seeded minstd_rand0, cast to
 * float.  stddev = 1 for SimHash; 1.0/sketchDim for JL (randomVectorGenerator.cpp:56-74). */
int lshg_random_normals(int64_t count, double stddev, float* out);
/* generateRandomOnePlusMinusVector (randomVectorGenerator.cpp:76-87). */
int lshg_random_plus_minus(int64_t count, int32_t* out);
/* generateRandomBoolVectors (weightedMinHash.cuh:231-250). */
int lshg_random_bools(int64_t count, uint8_t* out);

/* ---- resident index (serving use; no reference counterpart beyond runLsh) ---------- */
typedef struct lshg_index lshg_index;

typedef struct lshg_index_params_s {
  int implementation; /* as above */
  int distanceFunc;
  int sketchDim;
  int d;
  int framework; /* 0 = linear scan, 1 = (K,L) LSH */
  int keysImplementation;
  int bucketKeyBits;
  int tables;
  int runWithSketchedData;
  lshg_options opt;
} lshg_index_params;

/* Build an index over N_data points (host pointer unless data_on_device). */
int lshg_index_build(const lshg_index_params* p, const float* data, int64_t N_data, int data_on_device,
                     lshg_index** out);
/* Query: `queries` [N_query][d], `results` [N_query][k]; both host pointers unless
 * on_device.  stream: cudaStream_t or NULL (index stream).  Synchronous on return. */
int lshg_index_query(lshg_index* idx, const float* queries, int N_query, int k, lshg_point* results,
                     int on_device, void* stream);
int lshg_index_free(lshg_index* idx);
/* Stream-ordered query (no counterpart in the reference, which answers one synchronous
 * batch per run).  queries [N_query][d] and results [N_query][k] are device pointers
 * when on_device, else host pointers (page-locked for the copies to run asynchronously;
 * they must stay valid until the stream is synchronised).  The batch -- host-to-device
 * copy, query, device-to-host copy -- is enqueued on `stream` (NULL = index stream) and
 * the call returns without waiting, so a caller can keep several batches in flight on
 * one or more streams.  Argument errors are returned at once; errors found on the device
 * (a pipeline wait timed out, the MinHash sampler limit) are kept and reported by the
 * next lshg_index_sync or lshg_index_query on the index.  The query buffer is not
 * modified. */
int lshg_index_query_async(lshg_index* idx, const float* queries, int N_query, int k, lshg_point* results,
                           int on_device, void* stream);
/* Wait for every batch enqueued on `stream` (NULL = index stream) and report device
 * errors kept since the last report. */
int lshg_index_sync(lshg_index* idx, void* stream);
/* Allocation-free query (no counterpart in the reference).  For callers that cannot
 * allocate device memory while answering queries -- e.g. a server whose free HBM is
 * already held by another allocator, or a latency-critical thread that must not enter
 * the CUDA allocator.  Serves exact angular linear-scan indexes (implementation 2,
 * framework 0) only; d_queries [N_query][d] and d_results [N_query][k] are device
 * pointers.  All temporaries live in one 32 MiB device array per GPU that stays
 * allocated until the process exits; batches needing more are rejected with
 * LSHG_ERR_INVALID_ARGUMENT.  Calls that overlap on the GPU race on that array, so
 * serialise them.  The first call on a device looks up the array's address; make it
 * before any stream capture begins.  Asynchronous on `stream` (NULL = index stream). */
int lshg_index_query_noalloc(lshg_index* idx, const float* d_queries, int N_query, int k, lshg_point* d_results,
                             void* stream);

/* Export index internals to host memory for checks and persistence.  what:
 *  0 = base data after preprocessing (float [n][d])
 *  1 = sketches (u32 words [n][sketchDim] for 3/5, u8 [n][sketchDim] for 4, float for 6,
 *      int32 (index, t) pairs [n][sketchDim][2] for 10)
 *  2 = LSH keys (u16 [n][tables])
 *  3 = LSH bucket offsets (int32 [tables][tableSize], absolute into the bucket array)
 *  4 = LSH bucket ids (int32 [tables][n], ascending ids within each bucket)
 *  5 = query counters (uint64 [2], cumulative since the build or load: LSH bucket
 *      entries walked, distinct LSH candidates scored); read after the queries' streams
 *      have been synchronised
 *  6 = consistent-weighted-sampling code plan (int32 [6]: min and max t over the base's
 *      samples, code bits of the dimension index and of t, bit planes of the sliced codes
 *      -- 8 or 16, 0 when the codes need more than 16 bits and every scan is direct --,
 *      and 1 when the codes are ranks in per-position dictionaries of the base's codes)
 * If dst is NULL only *bytes is set. */
int lshg_index_export(lshg_index* idx, int what, void* dst, size_t* bytes);
/* Hash/sketch queries with the index's random vectors: sketches and keys as in export. */
int lshg_index_sketch_queries(lshg_index* idx, const float* queries, int N_query, void* sketches,
                              uint16_t* keys);
/* Persist / restore a built index (checksummed file). */
int lshg_index_save(lshg_index* idx, const char* path);
int lshg_index_load(const char* path, lshg_index** out);

/* ---- sharding helpers ------------------------------------------------------------- */
/* Merge `shards` per-shard top-k lists [shards][N_query][k_in] (IDs already global)
 * into [N_query][k] by (distance, ID), dropping duplicate IDs.  Host only. */
int lshg_merge_topk(const lshg_point* lists, int shards, int N_query, int k_in, int k, lshg_point* out);

/* ---- validation (validation.cpp:129-208) ------------------------------------------ */
/* recall@reportK = |truth top-reportK (by ID) in result first reportK| / reportK, and the
 * distance ratio sum(result) / sum(truth), averaged over queries. */
int lshg_validate(const lshg_point* truth, int truth_k, const lshg_point* results, int N_query, int k,
                  int reportK, float* recall, float* distance_ratio);

/* Read a GoldStandard truth file (goldstandard.cpp:123-134 writes it; validation.cpp:62-107
 * reads it): "n\nk\n" then per query "qid:" and k lines "id distance".  Returns a
 * malloc'ed lshg_point[n*k] (free with lshg_free). */
int lshg_read_truth(const char* path, int* n, int* k, lshg_point** out);

/* ---- reference text dataset format (gloveparser.cu:9-86, DataParsing/Writer) ------- */
/* parseFile: returns a malloc'ed float[n*d] (free with lshg_free). */
int lshg_parse_file(const char* path, int* n, int* d, float** out);
int lshg_write_file(const char* path, const float* x, int n, int d);
void lshg_free(void* p);

/* ---- serving loop ----------------------------------------------------------------- */
typedef struct lshg_server lshg_server;
typedef struct lshg_server_params_s {
  int max_batch;          /* largest coalesced launch (queries), default 4096 */
  int max_queue;          /* admission queue capacity (requests), default 65536 */
  int streams;            /* concurrent device streams, default 2 */
  int use_graphs;         /* capture launches in CUDA graphs per (index, k, batch class) */
  int64_t hbm_reserve_mb; /* admission keeps this much device memory free */
  int batch_window_us;    /* how long the batcher waits to fill a launch */
} lshg_server_params;
void lshg_server_params_default(lshg_server_params* p);
int lshg_server_create(const lshg_server_params* p, lshg_server** out);
/* Register a built index under `index_id` (the server does not take ownership). */
int lshg_server_add_index(lshg_server* s, int index_id, lshg_index* idx);
/* Submit one request (copies the queries).  *ticket identifies it for polling. */
int lshg_server_submit(lshg_server* s, int index_id, const float* queries, int N_query, int k,
                       int64_t* ticket);
/* Wait up to timeout_us for a ticket; copies N_query*k points into results.  Returns
 * LSHG_ERR_TIMEOUT if not done.  latency_us (optional) = submit-to-ready time. */
int lshg_server_wait(lshg_server* s, int64_t ticket, lshg_point* results, int64_t timeout_us,
                     double* latency_us);
/* Counters: completed requests, launches, graph replays, rejected submissions. */
int lshg_server_stats(lshg_server* s, int64_t* completed, int64_t* launches, int64_t* graph_replays,
                      int64_t* rejected);
int lshg_server_destroy(lshg_server* s);

#ifdef __cplusplus
}
#endif
#endif /* LSHG_H_ */
