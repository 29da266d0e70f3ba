// Mixed-precision instantiation of the batched interior-point kernel (cxg_ipm.cuh), large-root
// form: FP32 root factor with the double-float fallback.
#include "cxg_ipm.cuh"

namespace cxg {
CXG_IPM_FORM(, float, 256, 1)
}  // namespace cxg
