// Mixed-precision (tcgen05) logistic-regression target: not built yet.
#include "engine.h"

namespace gbm {
std::unique_ptr<Target> make_logreg_tc(gbm_context*, const void*, int, int64_t, int64_t,
                                       const float*, float) {
  return nullptr;
}
}  // namespace gbm
