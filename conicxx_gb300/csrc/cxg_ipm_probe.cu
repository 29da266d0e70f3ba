// Diagnostic entry of the dense root (cxg_dense_ldlt): the root LDL' and triangular solves of
// the interior-point kernels (cxg_ipm.cuh) on one given matrix, on one CTA or on the whole GPU.
#include <algorithm>
#include <cstring>
#include <vector>

#include "cxg_ipm.cuh"

// ------------------------------------------------------------------------------------------
// diagnostic: the dense root LDL' and solve of the IPM kernel on one given matrix (one CTA)
// ------------------------------------------------------------------------------------------
namespace cxg {

template <typename T>
__global__ void __launch_bounds__(256) denseProbeKernel(int nr, int nx, const double* K, const double* b,
                                                         DevSettings st, double* Lout, double* Dout, double* xout,
                                                         long long* cyc, int* flags) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ Ctx c;
  __shared__ double scArea[160];
  T* M = reinterpret_cast<T*>(smem);
  const int Tn = rootTiles(nr);
  const int64_t rs = rootSize(nr);
  T* y = M + rs;
  if (threadIdx.x == 0) {
    c.nr = nr;
    c.n = nx;
    c.red = scArea;
    c.sc = scArea + 128;
  }
  for (int64_t t = threadIdx.x; t < rs; t += blockDim.x) M[t] = (T)0;
  __syncthreads();
  for (int i = nr + (int)threadIdx.x; i < Tn * kTile; i += blockDim.x) M[rootIdx(nr, i, i)] = (T)1;
  for (int t = threadIdx.x; t < nr * nr; t += blockDim.x) {
    const int i = t % nr, j = t / nr;
    if (i >= j) M[rootIdx(nr, i, j)] = (T)K[t];
  }
  __syncthreads();
  int fail = 0, wrong = 0;
  double mind = 0.0;
  const long long t0 = clock64();
  denseLdlt<T>(c, M, st, fail, wrong, mind);
  const long long t1 = clock64();
  for (int t = threadIdx.x; t < nr * nr; t += blockDim.x) {
    const int i = t % nr, j = t / nr;
    Lout[t] = (i > j) ? (double)M[rootIdx(nr, i, j)] : ((i == j) ? 1.0 : 0.0);
  }
  for (int i = threadIdx.x; i < nr; i += blockDim.x) Dout[i] = (double)M[rootIdx(nr, i, i)];
  for (int i = threadIdx.x; i < Tn * kTile; i += blockDim.x) y[i] = (i < nr) ? (T)b[i] : (T)0;
  __syncthreads();
  const long long t2 = clock64();
  denseSolve<T>(c, M, y);
  const long long t3 = clock64();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) xout[i] = (double)y[i];
  if (threadIdx.x == 0) {
    cyc[0] = t1 - t0;
    cyc[1] = t3 - t2;
    flags[0] = fail;
    flags[1] = wrong;
  }
}

template <typename T>
static cudaError_t probeLaunch(int nr, int nx, const double* K, const double* b, const DevSettings& st, int threads,
                               double* L, double* D, double* x, long long* cyc, int* flags) {
  const size_t smem = (size_t)(rootSize(nr) + (int64_t)rootTiles(nr) * kTile) * sizeof(T);
  cudaError_t e = cudaFuncSetAttribute(denseProbeKernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  denseProbeKernel<T><<<1, threads, smem>>>(nr, nx, K, b, st, L, D, x, cyc, flags);
  return cudaGetLastError();
}

// Whole-GPU form of the probe: the root in global memory, factored and solved by gridLdlt /
// gridSolve on every SM (cooperative launch). cyc holds nanoseconds (device global timer).
template <typename T>
__global__ void __launch_bounds__(256, 1) denseProbeGridKernel(int nr, int nx, const double* K, const double* b,
                                                               DevSettings st, T* M, T* y, GridCtl* g, double* Lout,
                                                               double* Dout, double* xout, long long* cyc,
                                                               int* flags, unsigned char* slices) {
  __shared__ PivotStats sPs;
  extern __shared__ __align__(16) unsigned char stageSmem[];
  T* stage = reinterpret_cast<T*>(stageSmem);
  const int Tn = rootTiles(nr);
  const int64_t rs = rootSize(nr);
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
  const int64_t nn = (int64_t)nr * nr;
  if (threadIdx.x == 0) {
    sPs.nreg = 0;
    sPs.zero = 0;
    sPs.wrong = 0;
    sPs.minAbs = INFINITY;
  }
  for (int64_t t = gt; t < rs; t += gs) M[t] = (T)0;
  bool ok = gridSync(g);
  for (int64_t i = nr + gt; i < (int64_t)Tn * kTile; i += gs) M[rootIdx(nr, (int)i, (int)i)] = (T)1;
  for (int64_t t = gt; t < nn; t += gs) {
    const int i = (int)(t % nr), j = (int)(t / nr);
    if (i >= j) M[rootIdx(nr, i, j)] = (T)K[t];
  }
  for (int64_t i = gt; i < (int64_t)Tn * kTile; i += gs) y[i] = (i < nr) ? (T)b[i] : (T)0;
  ok = ok && gridSync(g);
  const unsigned long long t0 = globalNs();
  ok = ok && gridLdlt<T>(g, nr, nx, st, M, &sPs, stage, slices);
  const unsigned long long t1 = globalNs();
  for (int64_t t = gt; t < nn; t += gs) {
    const int i = (int)(t % nr), j = (int)(t / nr);
    Lout[t] = (i > j) ? (double)M[rootIdx(nr, i, j)] : ((i == j) ? 1.0 : 0.0);
  }
  for (int64_t i = gt; i < nr; i += gs) Dout[i] = (double)M[rootIdx(nr, (int)i, (int)i)];
  const unsigned long long t2 = globalNs();
  ok = ok && gridSolve<T>(g, nr, M, y);
  const unsigned long long t3 = globalNs();
  for (int64_t i = gt; i < nr; i += gs) xout[i] = (double)y[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const bool regularized = st.linear_solver == 2;
    cyc[0] = (long long)(t1 - t0);
    cyc[1] = (long long)(t3 - t2);
    flags[0] = regularized ? (((double)sPs.nreg > 0.05 * (double)nr) ? 1 : 0) : sPs.zero;
    flags[1] = sPs.wrong;
    flags[2] = ok ? 0 : 1;
  }
}

template <typename T>
static cudaError_t probeGridLaunch(int nr, int nx, const double* K, const double* b, const DevSettings& st, double* L,
                                   double* D, double* x, long long* cyc, int* flags) {
  int dev = 0, numSM = 0, occ = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&numSM, cudaDevAttrMultiProcessorCount, dev);
  // FP32: the tensor-core trailing update stages TF32 hi/lo panels (kTcStageBytes)
  const size_t smem = (size_t)std::max<int64_t>(gridStageBytes((int)sizeof(T)), sizeof(T) == 4 ? kTcStageBytes : 0);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(denseProbeGridKernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, denseProbeGridKernel<T>, 256, smem);
  if (e != cudaSuccess) return e;
  if (occ * numSM < 2) return cudaErrorInvalidConfiguration;
  T *M = nullptr, *y = nullptr;
  GridCtl* g = nullptr;
  unsigned char* slices = nullptr;  // FP32 and double-float: the panels of the tensor-core trailing update
  e = cudaMalloc((void**)&M, (size_t)rootSize(nr) * sizeof(T));
  if (e == cudaSuccess && ArithOf<T>::v != 0) e = cudaMalloc((void**)&slices, (size_t)dfSliceBytes(nr));
  if (e == cudaSuccess) e = cudaMalloc((void**)&y, (size_t)rootTiles(nr) * kTile * sizeof(T));
  if (e == cudaSuccess) e = cudaMalloc((void**)&g, sizeof(GridCtl));
  if (e == cudaSuccess) e = cudaMemset(g, 0, sizeof(GridCtl));
  if (e == cudaSuccess) {
    int nrv = nr, nxv = nx;
    DevSettings stv = st;
    void* args[] = {&nrv, &nxv, (void*)&K, (void*)&b, &stv, (void*)&M, (void*)&y, (void*)&g,
                    (void*)&L, (void*)&D, (void*)&x, (void*)&cyc, (void*)&flags, (void*)&slices};
    e = cudaLaunchCooperativeKernel((const void*)denseProbeGridKernel<T>, dim3(occ * numSM), dim3(256), args, smem,
                                    nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  if (M) cudaFree(M);
  if (y) cudaFree(y);
  if (g) cudaFree(g);
  if (slices) cudaFree(slices);
  return e;
}

// Barrier time-out self-test: every CTA passes `rounds` grid barriers, except CTA `skip` (when
// >= 0), which returns at once. The others' first wait then runs out after ctl->waitNs, the error
// flag is set and every barrier fails, so the launch ends without that CTA. passed[b] = barriers
// CTA b got through (-1 for the skipping CTA).
__global__ void __launch_bounds__(256) gridBarrierTestKernel(GridCtl* g, int skip, int rounds, int* passed) {
  if ((int)blockIdx.x == skip) {
    if (threadIdx.x == 0) passed[blockIdx.x] = -1;
    return;
  }
  int n = 0;
  for (int r = 0; r < rounds; ++r) {
    if (!gridSync(g)) break;
    ++n;
  }
  if (threadIdx.x == 0) passed[blockIdx.x] = n;
}

cudaError_t launchGridBarrierTest(int skip, int rounds, double timeoutS, int* errorFlag, int* maxPassed,
                                  double* elapsedS) {
  int dev = 0, numSM = 0, occ = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&numSM, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gridBarrierTestKernel, 256, 0);
  if (e != cudaSuccess) return e;
  if (occ < 1 || numSM < 2) return cudaErrorInvalidConfiguration;
  const int grid = numSM;  // one CTA per SM, all resident
  GridCtl* g = nullptr;
  int* passed = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaMalloc((void**)&g, sizeof(GridCtl));
  if (e == cudaSuccess) e = cudaMalloc((void**)&passed, sizeof(int) * grid);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    GridCtl h;
    std::memset(&h, 0, sizeof(h));
    h.waitNs = (unsigned long long)(timeoutS * 1e9);
    e = cudaMemcpy(g, &h, sizeof(h), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) {
    int sk = skip, rd = rounds;
    void* args[] = {(void*)&g, &sk, &rd, (void*)&passed};
    e = cudaEventRecord(e0, nullptr);
    if (e == cudaSuccess)
      e = cudaLaunchCooperativeKernel((const void*)gridBarrierTestKernel, dim3(grid), dim3(256), args, 0, nullptr);
    if (e == cudaSuccess) e = cudaEventRecord(e1, nullptr);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  }
  if (e == cudaSuccess) {
    float ms = 0.0f;
    e = cudaEventElapsedTime(&ms, e0, e1);
    *elapsedS = 1e-3 * ms;
  }
  if (e == cudaSuccess) {
    GridCtl h;
    std::vector<int> p((size_t)grid);
    e = cudaMemcpy(&h, g, sizeof(h), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(p.data(), passed, sizeof(int) * grid, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) {
      *errorFlag = h.error;
      int mx = -1;
      for (int v : p) mx = std::max(mx, v);
      *maxPassed = mx;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (g) cudaFree(g);
  if (passed) cudaFree(passed);
  return e;
}

size_t denseProbeSmem(int arith, int nr) {
  const size_t elem = (arith == 1) ? 4 : 8;
  return (size_t)(rootSize(nr) + (int64_t)rootTiles(nr) * kTile) * elem;
}

cudaError_t launchDenseProbe(int arith, int nr, int nx, const double* K, const double* b, const DevSettings& st,
                             int threads, double* L, double* D, double* x, long long* cyc, int* flags) {
  if (threads < 0) {
    if (arith == 1) return probeGridLaunch<float>(nr, nx, K, b, st, L, D, x, cyc, flags);
    if (arith == 2) return probeGridLaunch<df64>(nr, nx, K, b, st, L, D, x, cyc, flags);
    return probeGridLaunch<double>(nr, nx, K, b, st, L, D, x, cyc, flags);
  }
  if (arith == 1) return probeLaunch<float>(nr, nx, K, b, st, threads, L, D, x, cyc, flags);
  if (arith == 2) return probeLaunch<df64>(nr, nx, K, b, st, threads, L, D, x, cyc, flags);
  return probeLaunch<double>(nr, nx, K, b, st, threads, L, D, x, cyc, flags);
}

}  // namespace cxg
