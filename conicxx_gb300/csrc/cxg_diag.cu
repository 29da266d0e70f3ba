// Diagnostic entry points used by the parity tests: the device cone algebra of the IPM kernel
// evaluated on one cone set, and the host equilibration of the set-up path.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "conicxx_gb300.h"
#include "cxg_cones.cuh"
#include "cxg_kernels.h"
#include "cxg_plan.h"

namespace cxg {

std::string& lastErrorRef();

// One CTA evaluates op over all units of the cone set K = Zero^zero x R^nn_+ x Q^d0 x ...
// (same per-unit device functions as ipmKernel; NN units inline as in the kernel).
__global__ void coneEvalKernel(int op, int zero, int nn, int nsoc, const int* off, const int* dim, const double* s,
                               const double* z, const double* u, const double* v, double amax, double* out,
                               double* scal, double* params) {
  extern __shared__ double sh[];
  const int m = zero + nn + (nsoc > 0 ? off[nsoc - 1] + dim[nsoc - 1] - zero - nn : 0);
  double* cw = sh;        // NN w by row
  double* cu = sh + m;    // SOC u by row
  SocScale* sp = reinterpret_cast<SocScale*>(sh + 2 * m);
  for (int t = threadIdx.x; t < nn + nsoc; t += blockDim.x) {
    if (t < nn) {
      const int r = zero + t;
      cw[r] = sqrt(s[r] / z[r]);
    } else {
      const int b = t - nn;
      socUpdateScaling(s + off[b], z + off[b], dim[b], sp[b], cu + off[b]);
    }
  }
  __syncthreads();
  if (op <= 2 || op == 7) {
    const int f = (op == 0) ? kW : (op == 1) ? kWinv : (op == 2) ? kHs : kGinv;
    for (int r = threadIdx.x; r < zero; r += blockDim.x) out[r] = 0.0;
    for (int t = threadIdx.x; t < nn + nsoc; t += blockDim.x) {
      if (t < nn) {
        const int r = zero + t;
        out[r] = wfun(f, cw[r], amax) * u[r];
      } else {
        const int b = t - nn;
        socApply(sp[b], cu + off[b], dim[b], f, amax, u + off[b], out + off[b]);
      }
    }
  } else if (op == 3 || op == 4) {
    for (int r = threadIdx.x; r < zero; r += blockDim.x) out[r] = 0.0;
    for (int t = threadIdx.x; t < nn + nsoc; t += blockDim.x) {
      if (t < nn) {
        const int r = zero + t;
        out[r] = (op == 4) ? v[r] / u[r] : u[r] * v[r];
      } else {
        const int b = t - nn;
        if (op == 4) socInverseProduct(u + off[b], v + off[b], dim[b], out + off[b]);
        else socProduct(u + off[b], v + off[b], dim[b], out + off[b]);
      }
    }
  } else if (op == 5 && threadIdx.x == 0) {
    // serial min over units (the reduction order does not matter for a min)
    double al = amax;
    for (int t = 0; t < nn; ++t) {
      const int r = zero + t;
      if (v[r] < 0) al = fmin(al, -u[r] / v[r]);
    }
    for (int b = 0; b < nsoc; ++b) al = fmin(al, socMaxStep(u + off[b], v + off[b], dim[b], amax));
    scal[0] = al;
  } else if (op == 6 && threadIdx.x == 0) {
    double mn = INFINITY, pos = 0.0;
    if (nn > 0) {
      double mg = u[zero];
      for (int t = 1; t < nn; ++t) mg = fmin(mg, u[zero + t]);
      mn = fmin(mn, mg);
      pos += fmax(mg, 0.0);
    }
    for (int b = 0; b < nsoc; ++b) {
      const double mg = socMargin(u + off[b], dim[b]);
      mn = fmin(mn, mg);
      pos += fmax(mg, 0.0);
    }
    scal[0] = isfinite(mn) ? mn : 0.0;
    scal[1] = pos;
  }
  if (params) {
    for (int b = threadIdx.x; b < nsoc; b += blockDim.x) {
      params[8 * b + 0] = sp[b].kind;
      params[8 * b + 1] = sp[b].beta;
      params[8 * b + 2] = sp[b].lam;
      params[8 * b + 3] = sp[b].qc;
      params[8 * b + 4] = sp[b].qs;
    }
  }
}

}  // namespace cxg

using namespace cxg;

#define DG_CUDA(call)                                                                     \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      for (void* p_ : bufs) cudaFree(p_);                                                 \
      lastErrorRef() = std::string(#call) + ": " + cudaGetErrorString(e_);                \
      return CXG_E_CUDA;                                                                  \
    }                                                                                     \
  } while (0)

extern "C" int cxg_cones_eval(int op, int zero_dim, int nonneg_dim, int n_soc, const int* soc_dims, const double* s,
                              const double* z, const double* u, const double* v, double alpha_or_eps, double* out,
                              double* scalars, double* soc_params) {
  if (op < 0 || op > 7 || zero_dim < 0 || nonneg_dim < 0 || n_soc < 0 || !s || !z || !u) {
    lastErrorRef() = "cxg_cones_eval: bad arguments";
    return CXG_E_INVALID;
  }
  std::vector<int> off((size_t)n_soc), dim((size_t)n_soc);
  int m = zero_dim + nonneg_dim;
  for (int b = 0; b < n_soc; ++b) {
    if (!soc_dims || soc_dims[b] < 1) {
      lastErrorRef() = "cxg_cones_eval: SOC dimension < 1";
      return CXG_E_INVALID;
    }
    off[(size_t)b] = m;
    dim[(size_t)b] = soc_dims[b];
    m += soc_dims[b];
  }
  if (m < 1) {
    lastErrorRef() = "cxg_cones_eval: empty cone";
    return CXG_E_INVALID;
  }
  std::vector<void*> bufs;
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 8) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    return p;
  };
  int* dOff = (int*)alloc(sizeof(int) * (size_t)std::max(n_soc, 1));
  int* dDim = (int*)alloc(sizeof(int) * (size_t)std::max(n_soc, 1));
  double* dS = (double*)alloc(sizeof(double) * (size_t)m);
  double* dZ = (double*)alloc(sizeof(double) * (size_t)m);
  double* dU = (double*)alloc(sizeof(double) * (size_t)m);
  double* dV = (double*)alloc(sizeof(double) * (size_t)m);
  double* dO = (double*)alloc(sizeof(double) * (size_t)m);
  double* dSc = (double*)alloc(sizeof(double) * 2);
  double* dP = (double*)alloc(sizeof(double) * 8 * (size_t)std::max(n_soc, 1));
  if (bufs.size() != 9) {
    for (void* p : bufs) cudaFree(p);
    lastErrorRef() = "cxg_cones_eval: device allocation failed";
    return CXG_E_NOMEM;
  }
  if (n_soc) {
    DG_CUDA(cudaMemcpy(dOff, off.data(), sizeof(int) * (size_t)n_soc, cudaMemcpyHostToDevice));
    DG_CUDA(cudaMemcpy(dDim, dim.data(), sizeof(int) * (size_t)n_soc, cudaMemcpyHostToDevice));
  }
  DG_CUDA(cudaMemcpy(dS, s, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(dZ, z, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(dU, u, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(dV, v ? v : u, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice));
  const size_t shBytes = sizeof(double) * (2 * (size_t)m + 8 * (size_t)n_soc);
  if (shBytes > 200 * 1024) {
    for (void* p : bufs) cudaFree(p);
    lastErrorRef() = "cxg_cones_eval: cone set too large";
    return CXG_E_UNSUPPORTED;
  }
  DG_CUDA(cudaFuncSetAttribute(coneEvalKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shBytes));
  coneEvalKernel<<<1, 128, shBytes>>>(op, zero_dim, nonneg_dim, n_soc, dOff, dDim, dS, dZ, dU, dV, alpha_or_eps, dO, dSc,
                                      soc_params ? dP : nullptr);
  DG_CUDA(cudaGetLastError());
  DG_CUDA(cudaDeviceSynchronize());
  if (out) DG_CUDA(cudaMemcpy(out, dO, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost));
  if (scalars) DG_CUDA(cudaMemcpy(scalars, dSc, sizeof(double) * 2, cudaMemcpyDeviceToHost));
  if (soc_params && n_soc) DG_CUDA(cudaMemcpy(soc_params, dP, sizeof(double) * 8 * (size_t)n_soc, cudaMemcpyDeviceToHost));
  for (void* p : bufs) cudaFree(p);
  return CXG_OK;
}

extern "C" int cxg_equilibration(const cxg_problem* pr, const cxg_settings* st, double* d, double* e, double* c) {
  if (!pr || !st) {
    lastErrorRef() = "cxg_equilibration: null argument";
    return CXG_E_INVALID;
  }
  const std::string err = validateProblem(*pr);
  if (!err.empty()) {
    lastErrorRef() = err;
    return CXG_E_INVALID;
  }
  std::vector<double> dv, ev;
  double cv = 1.0;
  computeEquilibration(*pr, *st, dv, ev, cv);
  if (d) std::memcpy(d, dv.data(), sizeof(double) * dv.size());
  if (e) std::memcpy(e, ev.data(), sizeof(double) * ev.size());
  if (c) *c = cv;
  return CXG_OK;
}

extern "C" int cxg_dense_ldlt(int nr, int nx, const double* K, const double* b, int arith, int threads,
                              int linear_solver, double* L, double* D, double* x, long long* cycles, int* flags) {
  using namespace cxg;
  const bool whole = threads == -1;
  if (nr < 1 || nx < 0 || nx > nr || !K || !b || arith < 0 || arith > 2 ||
      (!whole && (threads < 32 || threads > 256 || (threads % 32) != 0))) {
    lastErrorRef() = "cxg_dense_ldlt: bad arguments";
    return CXG_E_INVALID;
  }
  std::vector<void*> bufs;
  int dev = 0, optin = 0;
  DG_CUDA(cudaGetDevice(&dev));
  DG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (!whole && denseProbeSmem(arith, nr) + 2048 > (size_t)optin) {
    lastErrorRef() = "cxg_dense_ldlt: matrix too large for one CTA's shared memory";
    return CXG_E_UNSUPPORTED;
  }
  cxg_settings cs;
  cxg_default_settings(&cs);
  DevSettings st{};
  st.dynamic_reg_eps = cs.dynamic_reg_eps;
  st.dynamic_reg_delta = cs.dynamic_reg_delta;
  st.linear_solver = linear_solver;
  const size_t nn = (size_t)nr * (size_t)nr;
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 8) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    return p;
  };
  double* dK = (double*)alloc(nn * 8);
  double* dB = (double*)alloc((size_t)nr * 8);
  double* dL = (double*)alloc(nn * 8);
  double* dD = (double*)alloc((size_t)nr * 8);
  double* dX = (double*)alloc((size_t)nr * 8);
  long long* dC = (long long*)alloc(2 * sizeof(long long));
  int* dF = (int*)alloc(3 * sizeof(int));
  if (bufs.size() != 7) {
    for (void* p : bufs) cudaFree(p);
    lastErrorRef() = "cxg_dense_ldlt: device allocation failed";
    return CXG_E_NOMEM;
  }
  DG_CUDA(cudaMemcpy(dK, K, nn * 8, cudaMemcpyHostToDevice));
  DG_CUDA(cudaMemcpy(dB, b, (size_t)nr * 8, cudaMemcpyHostToDevice));
  DG_CUDA(launchDenseProbe(arith, nr, nx, dK, dB, st, threads, dL, dD, dX, dC, dF));
  DG_CUDA(cudaDeviceSynchronize());
  if (L) DG_CUDA(cudaMemcpy(L, dL, nn * 8, cudaMemcpyDeviceToHost));
  if (D) DG_CUDA(cudaMemcpy(D, dD, (size_t)nr * 8, cudaMemcpyDeviceToHost));
  if (x) DG_CUDA(cudaMemcpy(x, dX, (size_t)nr * 8, cudaMemcpyDeviceToHost));
  if (cycles) DG_CUDA(cudaMemcpy(cycles, dC, 2 * sizeof(long long), cudaMemcpyDeviceToHost));
  if (flags) DG_CUDA(cudaMemcpy(flags, dF, (whole ? 3 : 2) * sizeof(int), cudaMemcpyDeviceToHost));
  for (void* p : bufs) cudaFree(p);
  return CXG_OK;
}

extern "C" int cxg_grid_barrier_selftest(int skip_cta, int rounds, double timeout_s, int* error_flag,
                                         int* max_rounds_passed, double* elapsed_s) {
  using namespace cxg;
  if (rounds < 1 || rounds > 100000 || !(timeout_s >= 1e-3 && timeout_s <= 5.0) || !error_flag ||
      !max_rounds_passed || !elapsed_s) {
    lastErrorRef() = "cxg_grid_barrier_selftest: bad arguments";
    return CXG_E_INVALID;
  }
  cudaError_t e = launchGridBarrierTest(skip_cta, rounds, timeout_s, error_flag, max_rounds_passed, elapsed_s);
  if (e != cudaSuccess) {
    lastErrorRef() = std::string("cxg_grid_barrier_selftest: ") + cudaGetErrorString(e);
    return CXG_E_CUDA;
  }
  return CXG_OK;
}

extern "C" int cxg_plan_inspect(const cxg_problem* pr, const cxg_settings* st, long long* counts, long long* plow,
                                long long* az, long long* tgt, int cap) {
  if (!pr || !st || !counts) {
    lastErrorRef() = "cxg_plan_inspect: null argument";
    return CXG_E_INVALID;
  }
  std::string err = validateProblem(*pr);
  if (!err.empty()) {
    lastErrorRef() = err;
    return CXG_E_INVALID;
  }
  err = checkPlanCounts(*pr);
  if (!err.empty()) {
    lastErrorRef() = err;
    return CXG_E_UNSUPPORTED;
  }
  Pools pools;
  pools.ipool.push_back(0);  // an odd start: the plan must re-align its 64-bit maps
  try {
    planInstance(*pr, *st, pools);
  } catch (const LimitError& ex) {
    lastErrorRef() = ex.what();
    return CXG_E_UNSUPPORTED;
  } catch (const std::exception& ex) {
    lastErrorRef() = ex.what();
    return CXG_E_NOMEM;
  }
  const InstanceDesc& D = pools.desc[0];
  counts[0] = D.nr;
  counts[1] = rootSize(D.nr);
  counts[2] = D.nPlow;
  counts[3] = D.nAZ;
  counts[4] = D.nTgt;
  counts[5] = D.nnzPs;
  counts[6] = D.nAd;
  counts[7] = D.nContrib;
  counts[8] = ((D.iPlowIdx | D.iAZIdx | D.iTgtIdx) & 1) == 0 ? 1 : 0;
  auto copy = [&](long long* out, int64_t off, int len) {
    if (!out) return;
    const int k = len < cap ? len : cap;
    if (k > 0) std::memcpy(out, pools.ipool.data() + off, sizeof(long long) * (size_t)k);
  };
  copy(plow, D.iPlowIdx, D.nPlow);
  copy(az, D.iAZIdx, D.nAZ);
  copy(tgt, D.iTgtIdx, D.nTgt);
  return CXG_OK;
}
