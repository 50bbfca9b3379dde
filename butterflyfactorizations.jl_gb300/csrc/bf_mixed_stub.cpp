// Entry points of the mixed-precision path that are not built yet.
#include "bf_surrogate.h"
using namespace bfg;
namespace bfg {
int surrogate_predict_gpu(const float*, const float*, float*, int64_t, cudaStream_t) {
  set_error("surrogate GPU inference not available in this build");
  return BF_ENOTSUP;
}
}  // namespace bfg
extern "C" int bf_matvec_mixed(bf_op_t, int, int64_t, const double*, int64_t, double*, int64_t,
                               const double*, const double*, int, void*) {
  set_error("bf_matvec_mixed: not available in this build");
  return BF_ENOTSUP;
}
