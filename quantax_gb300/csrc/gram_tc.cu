// Tensor-core Gram paths (tcgen05). Placeholder until the tcgen05 kernel lands.
#include "qgx_common.cuh"

namespace qgx {
int gram_tc(const float*, int64_t, int64_t, int64_t, double*, int64_t, int, cudaStream_t) {
  return QGX_ERR_UNSUPPORTED;
}
}  // namespace qgx
