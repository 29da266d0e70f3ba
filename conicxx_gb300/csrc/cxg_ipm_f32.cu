// Mixed-precision instantiations of the interior-point kernels (cxg_ipm.cuh), large-root form:
// FP32 root factor with the double-float fallback, batched and whole-GPU.
#include "cxg_ipm.cuh"

namespace cxg {
CXG_IPM_FORM(, float, 256, 1)
CXG_IPM_GRID(, float)
}  // namespace cxg
