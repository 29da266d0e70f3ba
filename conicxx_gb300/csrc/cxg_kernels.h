// Launch interface of the device kernels (cxg_ipm.cuh and its instantiations cxg_ipm_*.cu) as seen by
// the host API.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cxg_layout.h"

namespace cxg {

struct GridCtl;

// Dynamic shared-memory layout of one launch (byte offsets), sized for the largest instance of
// the launch. Vectors go to shared memory when they fit, else to the CTA's scratch.
struct SmemLayout {
  int nMax, mMax, nrMax, nsocMax;
  int vecInSmem, rootInSmem, root64InSmem, pad;
  int64_t redOff, vecOff, rootOff, total;
};

// Shared memory of the whole-GPU FP32 trailing update on the tensor cores: four 16 KB TF32 operand
// panels (A hi/lo, B hi/lo) and two buffers of the 16 C tiles of a 128x128 super-block, plus
// 128 bytes of alignment slack.
constexpr int64_t kGridTcStageBytes = 4 * 16384 + 2 * 16 * (int64_t)kTileElems * 4 + 128;

// Doubles of FP64 vectors per CTA for given maxima (must match the carve-up in ipmKernel).
inline int64_t vecDoubles(int nMax, int mMax, int nrMax, int nsocMax) {
  auto r2 = [](int64_t v) { return (v + 1) & ~int64_t(1); };
  return 6 * r2(nMax) + 11 * r2(mMax) + 4 * r2((int64_t)nMax + mMax) + (int64_t)rootTiles(nrMax) * kTile +
         r2(8 * (int64_t)nsocMax);
}
// Vectors used once or twice per iteration (the cone identity e and the constant-solve z1), kept
// in the CTA's scratch so the shared-memory vector area stays small enough for the largest root.
inline int64_t vecGlobalDoubles(int mMax) { return 2 * ((int64_t)(mMax + 1) & ~int64_t(1)); }

// Columns of one iteration-trace row (the oracle's trace columns): mu, ||rx||/tau, ||rz||/tau,
// primal and dual objective, affine step, sigma, step, tau, kappa, the iteration's largest relative
// KKT residual, and the factorisation attempts of the iteration's refactorisation.
constexpr int kTraceCols = 12;

// Restarted GMRES refinement of the whole-GPU form: basis dimension per cycle and cycles.
constexpr int kGmresDim = 20;
constexpr int kGmresCycles = 3;
// Doubles of its Krylov area (CTA 0's scratch): V (kGmresDim + 1 vectors of n + m), Z (kGmresDim
// vectors), the Hessenberg matrix, the Givens rotations, the rotated right-hand side, y.
inline int64_t krylovDoubles(int nMax, int mMax) {
  const int64_t ld = ((int64_t)nMax + mMax + 1) & ~int64_t(1);
  return (2 * kGmresDim + 1) * ld + (kGmresDim + 1) * kGmresDim + 4 * kGmresDim + 2;
}

// Whole-GPU double-float factor: the BF16 slices of each pair of tile columns' panels (A = L_IJ
// and B = L_IJ D_J over 64 columns, six slices each, for every root row) and their row exponents,
// written once per column pair and copied into shared memory per super-block. Bytes for a root
// of nr rows (a multiple of 16).
inline int64_t dfSliceBytes(int nr) {
  const int64_t rows = (int64_t)((nr + 31) / 32) * 32;
  return rows * (2 * 6 * 8 * 16) + 2 * rows * 4;
}

struct LaunchArgs {
  const InstanceDesc* desc;
  const int* order;       // instances of this launch, heaviest first
  int count;
  int* counter;           // zeroed before the launch
  const int* ipool;
  const double* dpool;
  const double* Px;       // concatenated user values
  const double* q;
  const double* Ax;
  const double* b;
  double* x;              // concatenated outputs (user units)
  double* s;
  double* z;
  DevResult* results;
  double* warmX;          // device-resident warm start (equilibrated space), may be null
  double* warmS;
  double* warmZ;
  unsigned char* haveWarm;
  double* bwd;            // saved final states (differentiable), or null
  const double* gx;       // adjoint input dL/dx (concatenated, user units)
  double* gq;             // adjoint outputs: dL/dq, dL/db, dL/d(P values), dL/d(A values)
  double* gb;
  double* gP;
  double* gA;
  double* trace;          // record_timings: per-instance iteration trace (traceRows x kTraceCols), or null
  int traceRows;
  double* scratch;        // gridDim.x * scratchStride doubles
  int64_t scratchStride;
  DevSettings st;
  SmemLayout lay;
  struct GridCtl* grid;   // whole-GPU form of one instance (cooperative launch), else null
};

cudaError_t launchIpm(const LaunchArgs& a, int grid, int block, size_t smem, bool fp32, cudaStream_t stream);
// Whole-GPU form for a single instance (args.count == 1): a cooperative launch of `grid` CTAs of
// 256 threads; `ctl` is a zeroed device control block of gridCtlBytes().
size_t gridCtlBytes();
cudaError_t launchIpmGrid(const LaunchArgs& a, GridCtl* ctl, int grid, size_t smem, bool fp32, cudaStream_t stream);
cudaError_t ipmGridOccupancy(int* blocksPerSM, size_t smem, bool fp32);
// One adjoint solve per instance with the saved final factorisation (same launch shape as the
// forward groups).
cudaError_t launchAdjoint(const LaunchArgs& a, int grid, int block, size_t smem, cudaStream_t stream);
// Resident CTAs per SM of the IPM kernel for a block size and dynamic shared-memory size.
cudaError_t ipmOccupancy(int* blocksPerSM, int block, size_t smem, bool fp32);

// Diagnostic: factor the dense symmetric nr x nr matrix K (column-major, first nx pivots
// expected positive, the rest negative) with the IPM kernel's tiled root LDL' in the given
// arithmetic (0 FP64, 1 FP32, 2 double-float) on one CTA of `threads` threads, then solve K x = b.
// Outputs L (unit lower, column-major), D, x, cycles {ldlt, solve}, flags {fail, wrong sign}.
size_t denseProbeSmem(int arith, int nr);
// Diagnostic: the whole-GPU grid barrier with one CTA (skip >= 0) never arriving; the wait limit
// is timeoutS. Reports the error flag, the most barriers any CTA passed and the launch time.
cudaError_t launchGridBarrierTest(int skip, int rounds, double timeoutS, int* errorFlag, int* maxPassed,
                                  double* elapsedS);
cudaError_t launchDenseProbe(int arith, int nr, int nx, const double* K, const double* b, const DevSettings& st,
                             int threads, double* L, double* D, double* x, long long* cyc, int* flags);

}  // namespace cxg
