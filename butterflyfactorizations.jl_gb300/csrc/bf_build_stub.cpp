// Placeholder entry points until the GPU construction and mixed path land.
#include "bf_internal.h"
using namespace bfg;
extern "C" {
int bf_build(bf_ctx_t, const double*, int64_t, const double*, int64_t, bf_tree_t, bf_tree_t,
             const int64_t*, const int64_t*, int64_t, double, double, const bf_build_opts*,
             bf_op_t* out) {
  if (out) *out = nullptr;
  set_error("bf_build: not available in this build");
  return BF_ENOTSUP;
}
int bf_matvec_mixed(bf_op_t, int, int64_t, const double*, int64_t, double*, int64_t,
                    const double*, const double*, int, void*) {
  set_error("bf_matvec_mixed: not available in this build");
  return BF_ENOTSUP;
}
}
