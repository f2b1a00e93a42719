// Split-precision Gram x1 x2^T / D on the tcgen05 tensor cores (sm_103a).
#include "ntg_common.cuh"

namespace ntg {
int gram_tc(cudaStream_t, const float*, const float*, int64_t, int64_t, int64_t, float*) {
  return fail(NTG_ERR_UNSUPPORTED, "ntg_gram: tensor-core path not built");
}
}  // namespace ntg
