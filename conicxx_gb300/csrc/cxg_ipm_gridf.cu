// Mixed-precision (FP32 root factor, double-float fallback) instantiation of the whole-GPU form of the interior-point kernel (cxg_ipm.cuh): one
// large instance, cooperative launch, the root spread over every SM.
#include "cxg_ipm.cuh"

namespace cxg {
CXG_IPM_GRID(, float)
}  // namespace cxg
