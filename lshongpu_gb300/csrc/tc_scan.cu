// Tensor-core exact scan (implementation 8): placeholder until the tcgen05 kernel lands.
#include "index.h"

namespace lshg {

void tc_prepare(Index& idx, cudaStream_t s) {
  (void)idx;
  (void)s;
  throw Error(LSHG_ERR_UNSUPPORTED, "tensor-core scan not built yet");
}

void launch_tc_scan(Index& idx, const float* q, int nq, int k, lshg_point* out, cudaStream_t s) {
  (void)idx; (void)q; (void)nq; (void)k; (void)out; (void)s;
  throw Error(LSHG_ERR_UNSUPPORTED, "tensor-core scan not built yet");
}

}  // namespace lshg
