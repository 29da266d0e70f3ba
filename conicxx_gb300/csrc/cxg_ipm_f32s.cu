// Mixed-precision instantiation of the interior-point kernel (cxg_ipm.cuh), small-root form
// (up to 64 threads, 8 resident CTAs per SM).
#include "cxg_ipm.cuh"

namespace cxg {
CXG_IPM_FORM(, float, 64, 8)
}  // namespace cxg
