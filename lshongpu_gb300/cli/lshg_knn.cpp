// lshg_knn: command-line drop-in for the reference's `knn` program
// (LinearScan/kernel.cu:119-196), on top of liblshg.so.
//
// Same 15 positional arguments:
//   1 data file   2 query file   3 truth file   4 validate (0/1)   5 write results (0/1)
//   6 k   7 implementation   8 sketchDim   9 distanceFunc   10 framework (0 linear, 1 LSH)
//   11 bucketKeyBits   12 tables   13 keysImplementation   14 runWithSketchedData
//   15 result file (one CSV line appended per run)
// Files use the reference text format (parseFile, gloveparser.cu:9-86); the truth file
// is GoldStandard's (goldstandard.cpp:123-134).  k is rounded up to a multiple of 32 as
// the reference does (calculateK); validation and the printed results use the first
// `k` (reportK) entries.  The CSV line has the reference's columns
// (resultWriter.cpp:43-55): implementation, keyImplementation, sketchDim, k,
// THREAD_QUEUE_SIZE, bucketKeyBits, tables, WITH_TQ_OR_BUFFER, preprocessTime,
// constructionTime, scanTime, recall, avgDistance.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lshg.h"

int main(int argc, char** argv) {
  if (argc < 16) {
    fprintf(stderr,
            "usage: %s data queries truth validate writeRes k implementation sketchDim distanceFunc framework "
            "bucketKeyBits tables keysImplementation runWithSketchedData resultFile\n",
            argv[0]);
    return 2;
  }
  const char* data_path = argv[1];
  const char* query_path = argv[2];
  const char* truth_path = argv[3];
  const int validate = atoi(argv[4]);
  const int write_res = atoi(argv[5]);
  const int reportK = atoi(argv[6]);
  const int implementation = atoi(argv[7]);
  const int sketchDim = atoi(argv[8]);
  const int distanceFunc = atoi(argv[9]);
  const int framework = atoi(argv[10]);
  const int bucketKeyBits = atoi(argv[11]);
  const int tables = atoi(argv[12]);
  const int keysImplementation = atoi(argv[13]);
  const int runWithSketchedData = atoi(argv[14]);
  const char* result_path = argv[15];
  const int k = lshg_calculate_k(reportK);

  int nq = 0, nd = 0, d = 0, d2 = 0;
  float* queries = nullptr;
  float* data = nullptr;
  if (lshg_parse_file(query_path, &nq, &d, &queries) || lshg_parse_file(data_path, &nd, &d2, &data)) {
    fprintf(stderr, "%s\n", lshg_last_error());
    return 1;
  }
  if (d != d2) {
    fprintf(stderr, "dimension mismatch: queries %d, data %d\n", d, d2);
    return 1;
  }
  printf("N_Query = %d \nN_Data = %d \nk is set to: %d\n", nq, nd, k);

  std::vector<lshg_point> results((size_t)nq * k);
  lshg_result res{};
  res.results = results.data();
  int st = framework == 0
               ? lshg_linear_scans(implementation, k, d, nq, nd, data, queries, sketchDim, distanceFunc, &res)
               : lshg_lsh(implementation, keysImplementation, k, d, nq, nd, data, queries, sketchDim, distanceFunc,
                          bucketKeyBits, tables, runWithSketchedData, &res);
  if (st != LSHG_OK) {
    fprintf(stderr, "lshg error %d: %s\n", st, lshg_last_error());
    lshg_free(queries);
    lshg_free(data);
    return 1;
  }
  printf("Time to preprocess: %lld \nTime to build: %lld \nTime to calculate distance on the GPU: %lld \n",
         (long long)res.preprocess_ms, (long long)res.construction_ms, (long long)res.scan_ms);

  if (validate) {
    int tn = 0, tk = 0;
    lshg_point* truth = nullptr;
    if (lshg_read_truth(truth_path, &tn, &tk, &truth) == LSHG_OK && tn == nq && tk >= reportK) {
      lshg_validate(truth, tk, results.data(), nq, k, reportK, &res.recall, &res.avg_distance);
      printf("Averge recall: %g\nTotal average: %g\n", res.recall, res.avg_distance);
    } else {
      fprintf(stderr, "validation skipped: %s\n", lshg_last_error());
    }
    lshg_free(truth);
  }
  if (write_res) {  // writeResult, resultWriter.cpp:7-20
    printf("%d\n%d\n", nq, reportK);
    for (int i = 0; i < nq; ++i) {
      printf("%d:\n", i);
      for (int j = 0; j < reportK; ++j) printf("%d %f\n", results[(size_t)i * k + j].ID, results[(size_t)i * k + j].distance);
    }
  }
  FILE* f = fopen(result_path, "a");
  if (f) {
    const int thread_queue_size = 128, with_tq_or_buffer = 0;
    fprintf(f, "%d,%d,%d,%d,%d,%d,%d,%d,%lld,%lld,%lld,%g,%g\n", implementation, keysImplementation, sketchDim, k,
            thread_queue_size, bucketKeyBits, tables, with_tq_or_buffer, (long long)res.preprocess_ms,
            (long long)res.construction_ms, (long long)res.scan_ms, res.recall, res.avg_distance);
    fclose(f);
  }
  lshg_free(queries);
  lshg_free(data);
  printf("Success. Program exiting. \n");
  return 0;
}
