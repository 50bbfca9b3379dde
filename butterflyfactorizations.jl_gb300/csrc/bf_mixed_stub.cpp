// Entry points of the mixed-precision path that are not built yet.
#include "bf_surrogate.h"
using namespace bfg;
namespace bfg {
int surrogate_predict_gpu(const float*, const float*, float*, int64_t, cudaStream_t) {
  set_error("surrogate GPU inference not available in this build");
  return BF_ENOTSUP;
}
}  // namespace bfg
