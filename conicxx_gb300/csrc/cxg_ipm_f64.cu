// FP64 instantiations of the interior-point kernels (cxg_ipm.cuh), the adjoint kernel, and the
// host entry points that pick the FP32 or FP64 instantiation.
#include "cxg_ipm.cuh"

namespace cxg {

CXG_IPM_FORM(, double, 256, 1)
CXG_IPM_FORM(, double, 64, 8)
// instantiated in cxg_ipm_f32.cu, cxg_ipm_f32s.cu, cxg_ipm_gridf.cu and cxg_ipm_gridd.cu
CXG_IPM_FORM(extern, float, 256, 1)
CXG_IPM_FORM(extern, float, 64, 8)
CXG_IPM_GRID(extern, float)
CXG_IPM_GRID(extern, double)

size_t gridCtlBytes() { return sizeof(GridCtl); }

// the small-root form for blocks of up to 64 threads, the large-root form otherwise
template <typename FT>
static cudaError_t launchIpmFT(const LaunchArgs& a, int grid, int block, size_t smem, cudaStream_t stream) {
  return (block <= 64) ? launchIpmFormT<FT, 64, 8>(a, grid, block, smem, stream)
                       : launchIpmFormT<FT, 256, 1>(a, grid, block, smem, stream);
}
template <typename FT>
static cudaError_t ipmOccupancyFT(int* blocksPerSM, int block, size_t smem) {
  return (block <= 64) ? ipmOccupancyFormT<FT, 64, 8>(blocksPerSM, block, smem)
                       : ipmOccupancyFormT<FT, 256, 1>(blocksPerSM, block, smem);
}

cudaError_t launchIpm(const LaunchArgs& a, int grid, int block, size_t smem, bool fp32, cudaStream_t stream) {
  return fp32 ? launchIpmFT<float>(a, grid, block, smem, stream) : launchIpmFT<double>(a, grid, block, smem, stream);
}

cudaError_t ipmOccupancy(int* blocksPerSM, int block, size_t smem, bool fp32) {
  return fp32 ? ipmOccupancyFT<float>(blocksPerSM, block, smem) : ipmOccupancyFT<double>(blocksPerSM, block, smem);
}

cudaError_t launchIpmGrid(const LaunchArgs& a, GridCtl* g, int grid, size_t smem, bool fp32, cudaStream_t stream) {
  return fp32 ? launchIpmGridT<float>(a, g, grid, smem, stream) : launchIpmGridT<double>(a, g, grid, smem, stream);
}

cudaError_t ipmGridOccupancy(int* blocksPerSM, size_t smem, bool fp32) {
  return fp32 ? ipmGridOccupancyT<float>(blocksPerSM, smem) : ipmGridOccupancyT<double>(blocksPerSM, smem);
}

__global__ void __launch_bounds__(256) adjointKernel(LaunchArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int sInst;
  __shared__ int sRedi[4];
  __shared__ Ctx c;
  double* scratch = a.scratch + (int64_t)blockIdx.x * a.scratchStride;
  for (;;) {
    if (threadIdx.x == 0) sInst = atomicAdd(a.counter, 1);
    __syncthreads();
    const int slot = sInst;
    __syncthreads();
    if (slot >= a.count) break;
    const int inst = a.order[slot];
    if (threadIdx.x == 0) setupCtx(c, a, inst, smem, scratch, sRedi);
    __syncthreads();
    loadInstance(c, a);
    adjointInstance(c, a);
  }
}

cudaError_t launchAdjoint(const LaunchArgs& a, int grid, int block, size_t smem, cudaStream_t stream) {
  cudaError_t e = raiseDynSmem((const void*)adjointKernel, smem);
  if (e != cudaSuccess) return e;
  adjointKernel<<<grid, block, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace cxg
