// The interior-point hot path on the GPU (device code, instantiated by cxg_ipm_f32.cu,
// cxg_ipm_f32s.cu, cxg_ipm_f64.cu, cxg_ipm_gridf.cu, cxg_ipm_gridd.cu and cxg_ipm_probe.cu, which
// compile in parallel). One CTA runs the complete homogeneous self-dual embedding IPM of ConicXX
// (SolverImpl::solve and its helpers, src/conicxx/solver_impl.cpp:102-466) for one instance:
//  - batched form (ipmKernel): persistent CTAs take instances from an atomic queue per size
//    bucket; iterates in shared memory when they fit, the problem data in HBM/L2;
//  - whole-GPU form (ipmGridKernel): one large instance, CTA 0 running the iteration on vectors in
//    its scratch while every SM joins the root assembly, LDL' and triangular solves (gridSync).
//
// Precision: cone scaling, residuals, refinement residuals, step lengths and termination are
// FP64. The dense root LDL' (see cxg_layout.h) is FP32 (MIXED) or FP64. In MIXED mode a KKT
// solve whose FP64-refined relative residual stays above mixed_fallback_tol (or is not finite),
// or whose FP32 factor has a pivot of the wrong sign, switches that instance to the double-float
// factor (about 48 bits, on the FP32 pipe) for the rest of its solve ("sticky" fallback, counted
// in DevResult::fp64_fallbacks).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cxg_cones.cuh"
#include "cxg_df64.cuh"
#include "cxg_kernels.h"
#include "cxg_layout.h"
#include "cxg_tc.cuh"

namespace cxg {

#define FOR_T(i, n) for (int i = (int)threadIdx.x; i < (n); i += (int)blockDim.x)

// sum_{k=beg}^{end-1} val[k] * x[col[k]]: eight loads in flight per round (the values and
// column indices live in the CTA's scratch, in L2) and four independent accumulators (one would
// make every row a dependent FP64 chain, the cost on GB300's narrow FP64 pipe).
__device__ __forceinline__ double csrDot(const double* __restrict__ val, const int* __restrict__ col, int beg, int end,
                                         const double* x) {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  int k = beg;
  for (; k + 7 < end; k += 8) {
    double v[8];
    int ci[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      v[u] = val[k + u];
      ci[u] = col[k + u];
    }
    a0 = fma(v[0], x[ci[0]], a0);
    a1 = fma(v[1], x[ci[1]], a1);
    a2 = fma(v[2], x[ci[2]], a2);
    a3 = fma(v[3], x[ci[3]], a3);
    a0 = fma(v[4], x[ci[4]], a0);
    a1 = fma(v[5], x[ci[5]], a1);
    a2 = fma(v[6], x[ci[6]], a2);
    a3 = fma(v[7], x[ci[7]], a3);
  }
  for (; k < end; ++k) a0 = fma(val[k], x[col[k]], a0);
  return (a0 + a1) + (a2 + a3);
}

// Finiteness by the exponent bits (an integer test; FP64 compares run on the scarce FP64 pipe).
__device__ __forceinline__ bool finiteBits(double v) {
  return ((__double_as_longlong(v) >> 52) & 0x7ff) != 0x7ff;
}

// ------------------------------------------------------------------------------------------
// block reductions (deterministic: fixed summation order, identical result in every thread)
// ------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void blockSum(double (&v)[K], double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) red[k * 16 + w] = v[k];
  __syncthreads();
  // pairwise over the warps' partials (depth log2(nw), not nw: FP64 adds are long-latency here)
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double* r = red + k * 16;
    double t;
    if (nw == 1) t = r[0];
    else if (nw == 2) t = r[0] + r[1];
    else if (nw == 4) t = (r[0] + r[1]) + (r[2] + r[3]);
    else if (nw == 8) t = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    else {
      t = 0.0;
      for (int j = 0; j < nw; ++j) t += r[j];
    }
    v[k] = t;
  }
}

__device__ __forceinline__ double blockMin(double v, double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = red[0];
  for (int j = 1; j < nw; ++j) t = fmin(t, red[j]);
  return t;
}

__device__ __forceinline__ int blockOrInt(int v, int* redi) {
  __syncthreads();
  if (threadIdx.x == 0) redi[0] = 0;
  __syncthreads();
  if (v) atomicOr(redi, v);
  __syncthreads();
  return redi[0];
}

__device__ __forceinline__ int blockMaxInt(int v, int* redi) {
  __syncthreads();
  if (threadIdx.x == 0) redi[0] = 0;
  __syncthreads();
  if (v) atomicMax(redi, v);
  __syncthreads();
  return redi[0];
}

// ------------------------------------------------------------------------------------------
// per-instance context (pointers into shared memory, scratch and the pools)
// ------------------------------------------------------------------------------------------
struct GridCtl;

struct Ctx {
  int n, m, p, l, nsoc, nr, nUnits;
  const InstanceDesc* D;
  const int *psRow, *psCol, *pdiag, *plowSrc, *ap, *ai, *arRow, *arCol, *arSrc;
  const int *azSrc, *socOff, *socDim, *unitAd, *unitSup, *tgtBeg, *contrib;
  const long long *plowIdx, *azIdx, *tgtIdx;  // 64-bit root element offsets (8-byte aligned in the pool)
  // FP64 scratch (scaled data)
  double *Pu, *Pv, *Av, *Ad, *T, *qs, *bs, *root64;
  // shared-memory (or scratch) vectors
  double *x, *s, *z, *rx, *rz, *x1, *z1, *Px1, *dx, *dz, *ds, *dcon, *lam, *tn, *tm, *tm2;
  double *rhs, *sol, *res, *cor, *rr, *cw, *cu, *ev;
  SocScale* sp;
  void* root;      // FactT root (shared or scratch)
  double* red;
  int* redi;
  double* sc;      // scalar broadcast area
  double* kry;     // whole-GPU form: GMRES Krylov area (krylovDoubles) in scratch
  unsigned char* slices;  // whole-GPU mixed form: double-float panel slices (dfSliceBytes) in scratch
  GridCtl* grid;   // whole-GPU launch: the root jobs run on every CTA (null: this CTA alone)
};

// scalar slots in Ctx::sc
enum {
  SC_TAU = 0, SC_KAPPA, SC_EXTRA_P, SC_EXTRA_A, SC_USE64, SC_NFB, SC_RSTEPS, SC_MAXREL,
  SC_ATTEMPTS, SC_FACTOK, SC_GMRES, SC_ITREL, SC_FAULTF, SC_FAULTS, SC_ESC, SC_SOCLVL, SC_HSFLOOR, SC_COUNT
};



// Phase cycle counters (record_timings), kept by thread 0 in the scalar area after PivotStats.
enum { TM_FACTOR = 0, TM_SOLVE = 1, TM_ASSEMBLE = 2, TM_LDLT = 3, TM_DSOLVE = 4, TM_RESID = 5, TM_COUNT = 6 };
__device__ __forceinline__ long long* timers(Ctx& c) { return reinterpret_cast<long long*>(c.sc + SC_COUNT + 4); }

// ------------------------------------------------------------------------------------------
// instance prologue: scaled copies of the data (equilibration.cpp:102-127)
// ------------------------------------------------------------------------------------------
static __device__ __noinline__ void loadInstance(Ctx& c, const LaunchArgs& a) {
  const InstanceDesc& D = *c.D;
  const double* dvec = a.dpool + D.dD;
  const double* evec = a.dpool + D.dE;
  const double cs = D.cscale;
  const double* Px = a.Px + D.vPx;
  const double* Ax = a.Ax + D.vAx;
  const double* q = a.q + D.vQ;
  const double* b = a.b + D.vB;
  const int* Pp = a.ipool + D.iPp;
  const int* Pi = a.ipool + D.iPi;
  const int* psSrc = a.ipool + D.iPsSrc;
  // scaleP / scaleA / scaleQ / scaleB with the reference's operation order
  FOR_T(j, c.n) {
    for (int k = Pp[j]; k < Pp[j + 1]; ++k) c.Pu[k] = Px[k] * (cs * dvec[Pi[k]] * dvec[j]);
    for (int k = c.ap[j]; k < c.ap[j + 1]; ++k) c.Av[k] = Ax[k] * (evec[c.ai[k]] * dvec[j]);
    c.qs[j] = q[j] * (cs * dvec[j]);
  }
  FOR_T(r, c.m) {
    c.bs[r] = b[r] * evec[r];
    c.ev[r] = (r < c.p) ? 0.0 : ((r < c.p + c.l) ? 1.0 : 0.0);
  }
  __syncthreads();
  FOR_T(b2, c.nsoc) c.ev[c.socOff[b2]] = 1.0;
  FOR_T(k, D.nnzPs) c.Pv[k] = c.Pu[psSrc[k]];
  const int* adSrc = a.ipool + D.iAdSrc;
  FOR_T(k, D.nAd) {
    const int src = adSrc[k];
    c.Ad[k] = (src >= 0) ? c.Av[src] : 0.0;
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------------------
// cone-set operations over all units of the instance (cone_set.cpp)
// ------------------------------------------------------------------------------------------
// Also leaves in c.sc[SC_SOCLVL] the first attempt of the regularisation ladder at which every SOC
// block's dense pivots pass in the reference's arithmetic (socRefLadderLevel; 0 when the test is
// off): the earlier attempts of factorizeWithRetry fail as the reference's do. From the first
// iteration with such a failure on, the instance's blocks hold Hs at the dense form's resolution
// (kind 3, hsSmall; flag SC_HSFLOOR).
static __device__ __noinline__ void coneUpdateScaling(Ctx& c, const DevSettings& st, const double* s, const double* z) {
  int lvl = 0;
  FOR_T(t, c.l + c.nsoc) {
    if (t < c.l) {
      const int r = c.p + t;
      c.cw[r] = sqrt(s[r] / z[r]);  // nonnegative_cone.cpp:24
    } else {
      const int b = t - c.l;
      const int off = c.socOff[b], d = c.socDim[b];
      socUpdateScaling(s + off, z + off, d, c.sp[b], c.cu + off);
      if (st.soc_ref_dense && st.linear_solver != 2)
        lvl = max(lvl, socRefLadderLevel(s + off, z + off, d, st.static_reg_A, st.dynamic_reg_eps,
                                         st.dynamic_reg_delta, lvl));
    }
  }
  const int mx = blockMaxInt(lvl, c.redi);
  // once a block's dense form has lost its small eigenvalue (the reference's pivot test fails),
  // the instance's blocks take Hs at the dense form's resolution, from this iteration on (sticky)
  const bool floorHs = c.sc[SC_HSFLOOR] != 0.0 || mx > 0;
  if (floorHs) FOR_T(b, c.nsoc) if (c.sp[b].kind == 2.0) c.sp[b].kind = 3.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    c.sc[SC_SOCLVL] = (double)mx;
    if (floorHs) c.sc[SC_HSFLOOR] = 1.0;
  }
  __syncthreads();
}

// out = f(W) x on every cone row (Zero rows: 0, or eps * x for kHsEps).
static __device__ __noinline__ void coneApply(Ctx& c, int f, double eps, const double* x, double* out) {
  FOR_T(r, c.p) out[r] = (f == kHsEps) ? eps * x[r] : 0.0;
  FOR_T(t, c.l + c.nsoc) {
    if (t < c.l) {
      const int r = c.p + t;
      out[r] = wfun(f, c.cw[r], eps) * x[r];
    } else {
      const int b = t - c.l;
      const int off = c.socOff[b], d = c.socDim[b];
      socApply(c.sp[b], c.cu + off, d, f, eps, x + off, out + off);
    }
  }
  __syncthreads();
}

// out = G x on the cone rows with the G eigenvalues prepared at factorisation (Zero rows: 0).
static __device__ __noinline__ void coneApplyG(Ctx& c, const double* x, double* out) {
  FOR_T(r, c.p) out[r] = 0.0;
  FOR_T(t, c.l + c.nsoc) {
    if (t < c.l) {
      const int r = c.p + t;
      out[r] = c.cu[r] * x[r];
    } else {
      const int b = t - c.l;
      const int off = c.socOff[b], d = c.socDim[b];
      socApplyG(c.sp[b], c.cu + off, d, x + off, out + off);
    }
  }
  __syncthreads();
}

// Jordan product / inverse product (Zero rows -> 0).
static __device__ __noinline__ void coneProduct(Ctx& c, bool inverse, const double* u, const double* v, double* out) {
  FOR_T(r, c.p) out[r] = 0.0;
  FOR_T(t, c.l + c.nsoc) {
    if (t < c.l) {
      const int r = c.p + t;
      out[r] = inverse ? v[r] / u[r] : u[r] * v[r];
    } else {
      const int b = t - c.l;
      const int off = c.socOff[b], d = c.socDim[b];
      if (inverse) socInverseProduct(u + off, v + off, d, out + off);
      else socProduct(u + off, v + off, d, out + off);
    }
  }
  __syncthreads();
}

// ConeSet::maxStep (cone_set.cpp:108-115) as a block-wide min of per-unit limits.
static __device__ __noinline__ double coneMaxStep(Ctx& c, const double* x, const double* dx, double amax) {
  double al = amax;
  FOR_T(t, c.l + c.nsoc) {
    if (t < c.l) {
      const int r = c.p + t;
      if (dx[r] < 0) al = fmin(al, -x[r] / dx[r]);
    } else {
      const int b = t - c.l;
      const int off = c.socOff[b], d = c.socDim[b];
      al = fmin(al, socMaxStep(x + off, dx + off, d, amax));
    }
  }
  return blockMin(al, c.red);
}

// ConeSet::margins (cone_set.cpp:77-90): the NN block contributes ONE margin (its minimum).
static __device__ __noinline__ void coneMargins(Ctx& c, const double* x, double& mn, double& pos) {
  double nnmin = INFINITY;
  FOR_T(t, c.l) nnmin = fmin(nnmin, x[c.p + t]);
  double smin = INFINITY, spos = 0.0;
  FOR_T(b, c.nsoc) {
    const double mg = socMargin(x + c.socOff[b], c.socDim[b]);
    smin = fmin(smin, mg);
    spos += fmax(mg, 0.0);
  }
  nnmin = blockMin(nnmin, c.red);
  smin = blockMin(smin, c.red);
  double v[1] = {spos};
  blockSum<1>(v, c.red);
  mn = fmin(nnmin, smin);
  pos = v[0] + ((c.l > 0) ? fmax(nnmin, 0.0) : 0.0);
  if (!isfinite(mn)) mn = 0.0;
}

static __device__ void coneShift(Ctx& c, double* x, double alpha) {
  FOR_T(t, c.l) x[c.p + t] += alpha;
  FOR_T(b, c.nsoc) x[c.socOff[b]] += alpha;
  __syncthreads();
}

// shiftToInteriorCold (solver_impl.cpp:104-116 in the reference numbering of SolverImpl)
static __device__ void shiftToInteriorCold(Ctx& c, double* v, int degree) {
  double mn, pos;
  coneMargins(c, v, mn, pos);
  const double deg = (double)max(degree, 1);
  const double target = fmax(1.0, 0.1 * pos / deg);
  if (mn <= 0.0) {
    coneShift(c, v, -mn);
    coneShift(c, v, target);
  } else if (mn < target) {
    coneShift(c, v, target - mn);
  }
}

static __device__ void ensureStrictlyInteriorWarm(Ctx& c, double* v) {
  double mn, pos;
  coneMargins(c, v, mn, pos);
  if (mn <= 1e-8) coneShift(c, v, -mn + 1e-6);
}

// ------------------------------------------------------------------------------------------
// SpMVs with the scaled data (FP64)
// ------------------------------------------------------------------------------------------
// y = P_sym x (full symmetric CSR, one thread per row)
static __device__ __noinline__ void pmul(Ctx& c, const double* x, double* y) {
  FOR_T(i, c.n) y[i] = csrDot(c.Pv, c.psCol, c.psRow[i], c.psRow[i + 1], x);
  __syncthreads();
}

// res = rhs - K sol for the statically-regularised K (the matrix refinement targets,
// kkt_system.cpp:296-311): top = (P + epsP I) x + A'z, bottom = A x - (Hs + epsA I) z.
static __device__ __noinline__ double kktResidualImpl(Ctx& c, const DevSettings& st, const double* rhs, const double* sol,
                                  double* res, double& rhsNorm) {
  const int n = c.n, m = c.m;
  const double* xs = sol;
  const double* zs = sol + n;
  double acc2[2] = {0.0, 0.0};
  FOR_T(t, n + m) {
    if (t < n) {
      double acc = st.static_reg_P * xs[t] + csrDot(c.Pv, c.psCol, c.psRow[t], c.psRow[t + 1], xs);
      acc += csrDot(c.Av, c.ai, c.ap[t], c.ap[t + 1], zs);
      res[t] = rhs[t] - acc;
    } else {
      const int r = t - n;
      double acc = 0.0;
      for (int k = c.arRow[r]; k < c.arRow[r + 1]; ++k) acc += c.Av[c.arSrc[k]] * xs[c.arCol[k]];
      res[t] = rhs[t] - acc;
    }
  }
  __syncthreads();
  // + (Hs + epsA I) z on the cone rows
  coneApply(c, kHsEps, st.static_reg_A, zs, c.tm2);
  FOR_T(r, m) res[n + r] += c.tm2[r];
  __syncthreads();
  FOR_T(t, n + m) {
    acc2[0] += res[t] * res[t];
    acc2[1] += rhs[t] * rhs[t];
  }
  blockSum<2>(acc2, c.red);
  rhsNorm = fmax(sqrt(acc2[1]), 1e-30);
  return sqrt(acc2[0]) / rhsNorm;
}

// y = K sol for the same statically regularised K (the operator of the GMRES refinement).
static __device__ __noinline__ void kktApply(Ctx& c, const DevSettings& st, const double* sol, double* y) {
  const int n = c.n, m = c.m;
  const double* xs = sol;
  const double* zs = sol + n;
  FOR_T(t, n + m) {
    if (t < n) {
      double acc = st.static_reg_P * xs[t] + csrDot(c.Pv, c.psCol, c.psRow[t], c.psRow[t + 1], xs);
      acc += csrDot(c.Av, c.ai, c.ap[t], c.ap[t + 1], zs);
      y[t] = acc;
    } else {
      const int r = t - n;
      double acc = 0.0;
      for (int k = c.arRow[r]; k < c.arRow[r + 1]; ++k) acc += c.Av[c.arSrc[k]] * xs[c.arCol[k]];
      y[t] = acc;
    }
  }
  __syncthreads();
  coneApply(c, kHsEps, st.static_reg_A, zs, c.tm2);
  FOR_T(r, m) y[n + r] -= c.tm2[r];
  __syncthreads();
}

static __device__ double kktResidual(Ctx& c, const DevSettings& st, const double* rhs, const double* sol, double* res,
                              double& rhsNorm) {
  const long long t0 = (st.record_timings && threadIdx.x == 0) ? clock64() : 0;
  const double r = kktResidualImpl(c, st, rhs, sol, res, rhsNorm);
  if (st.record_timings && threadIdx.x == 0) timers(c)[TM_RESID] += clock64() - t0;
  return r;
}

// ------------------------------------------------------------------------------------------
// dense LDL' of the tiled root (no pivoting) and its solve
// ------------------------------------------------------------------------------------------
// Right-looking over 32-wide tile columns J:
//   (1) one warp factors the diagonal tile (rows in registers, shuffles), stores L (lower),
//       D (diagonal) and Linv^T (upper half) of the tile;
//   (2) warps compute the off-diagonal tiles L_IJ = A_IJ Linv_JJ^T D_J^-1;
//   (3) warps apply the trailing updates A_IK -= L_IJ D_J L_KJ^T, one tile pair per warp.
// Three barriers per tile column. Pivot rules: QDLDL (qdldl_ldlt.cpp:64-68) fails on an exact
// zero pivot; REGULARIZED (regularized_ldlt.cpp:132-139, 251-253) corrects a pivot below eps with
// the expected sign (+ on x rows, - on Zero-cone rows) and fails if > 5% were corrected.

// Pivot statistics written by the factoring warp (shared memory, read after a barrier).
struct PivotStats {
  int nreg, zero, wrong, pad;
  double minAbs;
};

template <typename T>
__device__ __forceinline__ T shflT(T v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ df64 shflT(df64 v, int src) {
  return df64(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
// c + a b and c - a b in the tile arithmetic (one FMA for float/double, the fused double-float form)
template <typename T>
__device__ __forceinline__ T madT(T c, T a, T b) { return c + a * b; }
__device__ __forceinline__ df64 madT(df64 c, df64 a, df64 b) { return dfMad(c, a, b); }
template <typename T>
__device__ __forceinline__ T msubT(T c, T a, T b) { return c - a * b; }
__device__ __forceinline__ df64 msubT(df64 c, df64 a, df64 b) { return dfMad(c, -a, b); }
// Accumulation inside tile products: accT (no renormalisation for double-float), then accEnd.
template <typename T>
__device__ __forceinline__ T accT(T c, T a, T b) { return c + a * b; }
__device__ __forceinline__ df64 accT(df64 c, df64 a, df64 b) { return dfMadLoose(c, a, b); }
template <typename T>
__device__ __forceinline__ T accEnd(T c) { return c; }
__device__ __forceinline__ df64 accEnd(df64 c) { return dfNorm(c); }

// A row of 32 values held in registers (indices are compile-time after unrolling). The
// double-float row is kept as two float arrays so that it stays in registers.
template <typename T>
struct Row32 {
  T v[32];
  __device__ __forceinline__ T get(int k) const { return v[k]; }
  __device__ __forceinline__ void set(int k, T x) { v[k] = x; }
};
template <>
struct Row32<df64> {
  float h[32], l[32];
  __device__ __forceinline__ df64 get(int k) const { return df64(h[k], l[k]); }
  __device__ __forceinline__ void set(int k, df64 x) {
    h[k] = x.hi;
    l[k] = x.lo;
  }
};

// 1/d for a pivot. FP32: the IEEE reciprocal intrinsic. FP64 and double-float: Newton-Raphson
// iteration r <- r + r (1 - d r) from the FP32 reciprocal of the leading part (each step doubles
// the correct bits: 23 -> 46 -> full; two steps for FP64, one for double-float), falling back to
// a division when d is outside the float range or not finite.
__device__ __forceinline__ float recipT(float d) { return __frcp_rn(d); }
__device__ __forceinline__ double recipT(double d) {
  const float f = __double2float_rn(d);
  const float af = fabsf(f);
  if (!(af >= 1e-37f && af <= 1e37f)) return 1.0 / d;
  double r = (double)__frcp_rn(f);
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}
__device__ __forceinline__ df64 recipT(df64 d) {
  const float af = fabsf(d.hi);
  if (!(af >= 1e-37f && af <= 1e37f)) return df64(1.0f, 0.0f) / d;
  // one step from the 23-bit seed gives ~46 bits, the double-float rounding level
  const df64 r(__frcp_rn(d.hi), 0.0f);
  const df64 one(1.0f, 0.0f);
  return r + r * (one - d * r);
}

// Factors diagonal tile J in place (one warp), FP32 form. Global row of tile row r is J*32 + r.
// Lane r keeps row r of the tile in registers (entries right of the diagonal mirrored from the
// lower triangle) and the 32 elimination steps broadcast pivot column j by shuffles. The same
// steps applied to the identity (Gauss-Jordan) give row r of the inverse of the unit-lower
// factor, which is stored transposed in the upper half: Linv(r, c) at r*ld + c. Only the
// per-pivot regularisation test runs inside the loop, in the tile's own arithmetic; the pivot
// statistics (exact zero, wrong sign, smallest |D|) are taken once from the final D.
template <typename T>
__device__ void tileFactorDiagRegs(T* A, int J, int nr, int nx, const DevSettings& st, PivotStats* ps) {
  const int r = threadIdx.x & 31;
  const bool regularized = st.linear_solver == 2;
  const T epsT = (T)st.dynamic_reg_eps, deltaT = (T)st.dynamic_reg_delta;
  Row32<T> a, e;
#pragma unroll
  for (int col = 0; col < 32; ++col) {
    a.set(col, (col <= r) ? A[col * kTileLd + r] : A[r * kTileLd + col]);
    e.set(col, (col == r) ? (T)1 : (T)0);
  }
  int nreg = 0;
  T dr = (T)0;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    T dj = shflT(a.get(j), j);
    if (regularized) {
      const int g = J * 32 + j;
      if (g < nr) {
        const T sg = (g < nx) ? (T)1 : (T)-1;
        if (dj * sg < epsT) {
          dj = dj + sg * deltaT;
          if (dj * sg < epsT) dj = sg * deltaT;
          ++nreg;
        }
      }
    }
    const T inv = recipT(dj);
    const T lj = a.get(j) * inv;
#pragma unroll
    for (int k = j + 1; k < 32; ++k) {
      const T akj = shflT(a.get(j), k);
      a.set(k, msubT(a.get(k), lj, akj));
    }
    // Gauss-Jordan on the identity: row j of the inverse is final at step j
#pragma unroll
    for (int c = 0; c <= j; ++c) {
      const T ejc = shflT(e.get(c), j);
      if (r > j) e.set(c, msubT(e.get(c), lj, ejc));
    }
    if (r > j) a.set(j, lj);
    if (r == j) {
      a.set(j, dj);
      dr = dj;
    }
  }
  // pivot statistics of the real rows of this tile
  {
    const int g = J * 32 + r;
    const bool real = g < nr;
    const double d = (double)dr;
    const double sgn = (g < nx) ? 1.0 : -1.0;
    const unsigned zeroMask = __ballot_sync(0xffffffffu, real && d == 0.0);
    const unsigned wrongMask = __ballot_sync(0xffffffffu, real && !(d * sgn > 0.0));
    double ad = real ? fabs(d) : INFINITY;
    if (real && !isfinite(ad)) ad = NAN;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o = __shfl_xor_sync(0xffffffffu, ad, off);
      ad = (isnan(ad) || isnan(o)) ? NAN : fmin(ad, o);
    }
    if (r == 0) {
      ps->nreg += nreg;
      if (!regularized && zeroMask) ps->zero = 1;
      if (wrongMask) ps->wrong = 1;
      ps->minAbs = (isnan(ad) || isnan(ps->minAbs)) ? NAN : fmin(ps->minAbs, ad);
    }
  }
  __syncwarp();
#pragma unroll
  for (int col = 0; col < 32; ++col) {
    if (col <= r) A[col * kTileLd + r] = a.get(col);
    if (col < r) A[r * kTileLd + col] = e.get(col);
  }
  __syncwarp();
}

// Factors diagonal tile J in place (one warp), form for 8-byte arithmetic (FP64, double-float),
// whose fully unrolled register version would be too large. Global row of tile row r is J*32 + r.
// Blocked right-looking LDL' in 8-column blocks, in shared memory (entry (i, k) at k*ld + i):
//  (1) leaf: the 8x8 diagonal block, rows in registers of its 8 lanes, pivots by shuffle;
//  (2) panel: every row below finishes its 8 entries of the block by substitution with the leaf
//      (unscaled values kept in registers for (3)) and scales them by the pivot reciprocals;
//  (3) trailing: rows below subtract the block's rank-8 product from their remaining entries.
// Only the per-pivot regularisation test runs inside the pivot loop, in the tile's own
// arithmetic; the pivot statistics (exact zero, wrong sign, smallest |D|) are taken once from D.
// Then the inverse of the unit-lower factor, blocked the same way (four 8x8 leaf inverses, then
// the blocks below the diagonal by distance), is stored transposed in the upper half:
// Linv(R, C) at R*ld + C for C < R.
template <typename T>
__device__ void tileFactorDiagBlocked(T* A, int J, int nr, int nx, const DevSettings& st, PivotStats* ps) {
  const int r = threadIdx.x & 31;
  const bool regularized = st.linear_solver == 2;
  const T epsT = (T)st.dynamic_reg_eps, deltaT = (T)st.dynamic_reg_delta;
  int nreg = 0;
  T invMine = (T)0;  // 1 / D(r), kept by lane r
  for (int b = 0; b < 4; ++b) {
    const int c0 = 8 * b;
    const int li = r - c0;
    const bool leaf = li >= 0 && li < 8;
    // (1) leaf
    T a[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int ct = c0 + t;
      a[t] = leaf ? ((t <= li) ? A[ct * kTileLd + r] : A[r * kTileLd + ct]) : (T)0;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      T dj = shflT(a[j], c0 + j);
      if (regularized) {
        const int g = J * 32 + c0 + j;
        if (g < nr) {
          const T sg = (g < nx) ? (T)1 : (T)-1;
          if (dj * sg < epsT) {
            dj = dj + sg * deltaT;
            if (dj * sg < epsT) dj = sg * deltaT;
            ++nreg;
          }
        }
      }
      const T inv = recipT(dj);
      if (li == j) invMine = inv;
      const T lj = a[j] * inv;
#pragma unroll
      for (int k = j + 1; k < 8; ++k) {
        const T akj = shflT(a[j], c0 + k);
        a[k] = msubT(a[k], lj, akj);
      }
      if (li > j) a[j] = lj;
      if (li == j) a[j] = dj;
    }
    if (leaf) {
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (t <= li) A[(c0 + t) * kTileLd + r] = a[t];
    }
    __syncwarp();
    if (c0 + 8 >= 32) break;
    // (2) panel
    const bool below = r >= c0 + 8;
    T u[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) u[t] = below ? A[(c0 + t) * kTileLd + r] : (T)0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
#pragma unroll
      for (int s2 = t + 1; s2 < 8; ++s2) u[s2] = msubT(u[s2], u[t], A[(c0 + t) * kTileLd + c0 + s2]);
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const T idt = shflT(invMine, c0 + t);
      if (below) A[(c0 + t) * kTileLd + r] = u[t] * idt;
    }
    __syncwarp();
    // (3) trailing
    if (below) {
      int k = c0 + 8;
      for (; k + 3 <= r; k += 4) {
        T acc0 = A[k * kTileLd + r], acc1 = A[(k + 1) * kTileLd + r];
        T acc2 = A[(k + 2) * kTileLd + r], acc3 = A[(k + 3) * kTileLd + r];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const T* Lc = A + (c0 + t) * kTileLd;
          const T nu = -u[t];
          acc0 = accT(acc0, nu, Lc[k]);
          acc1 = accT(acc1, nu, Lc[k + 1]);
          acc2 = accT(acc2, nu, Lc[k + 2]);
          acc3 = accT(acc3, nu, Lc[k + 3]);
        }
        A[k * kTileLd + r] = accEnd(acc0);
        A[(k + 1) * kTileLd + r] = accEnd(acc1);
        A[(k + 2) * kTileLd + r] = accEnd(acc2);
        A[(k + 3) * kTileLd + r] = accEnd(acc3);
      }
      for (; k <= r; ++k) {
        T acc = A[k * kTileLd + r];
#pragma unroll
        for (int t = 0; t < 8; ++t) acc = accT(acc, -u[t], A[(c0 + t) * kTileLd + k]);
        A[k * kTileLd + r] = accEnd(acc);
      }
    }
    __syncwarp();
  }
  // pivot statistics of the real rows of this tile
  {
    const int g = J * 32 + r;
    const bool real = g < nr;
    const double d = (double)A[r * kTileLd + r];
    const double sgn = (g < nx) ? 1.0 : -1.0;
    const unsigned zeroMask = __ballot_sync(0xffffffffu, real && d == 0.0);
    const unsigned wrongMask = __ballot_sync(0xffffffffu, real && !(d * sgn > 0.0));
    double ad = real ? fabs(d) : INFINITY;
    if (real && !isfinite(ad)) ad = NAN;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o = __shfl_xor_sync(0xffffffffu, ad, off);
      ad = (isnan(ad) || isnan(o)) ? NAN : fmin(ad, o);
    }
    if (r == 0) {
      ps->nreg += nreg;
      if (!regularized && zeroMask) ps->zero = 1;
      if (wrongMask) ps->wrong = 1;
      ps->minAbs = (isnan(ad) || isnan(ps->minAbs)) ? NAN : fmin(ps->minAbs, ad);
    }
  }
  // (a) inverses of the four 8x8 unit-lower leaf blocks, lane r -> block r/8, column r%8
  {
    const int o = r & ~7, c = r & 7;
    T y[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      T acc = (T)0;
#pragma unroll
      for (int k = 0; k < i; ++k) acc = accT(acc, A[(o + k) * kTileLd + o + i], y[k]);
      y[i] = (i < c) ? (T)0 : ((i == c) ? (T)1 : -accEnd(acc));
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (i > c) A[(o + i) * kTileLd + o + c] = y[i];
  }
  __syncwarp();
  // (b) blocks (I, J) = (Jb + d, Jb): Linv(I,J) = -Linv(I,I) sum_{K=J}^{I-1} L(I,K) Linv(K,J)
  for (int d = 1; d < 4; ++d) {
    const int nb = 4 - d;
    for (int e = r; e < nb * 64; e += 32) {
      const int Jb = e >> 6, i = (e >> 3) & 7, j = e & 7;
      const int R = 8 * (Jb + d) + i, C = 8 * Jb + j;
      T acc0 = (T)0, acc1 = (T)0;
      for (int kk = 8 * Jb; kk < 8 * (Jb + d); kk += 2) {
        const T lv0 = (kk > C) ? A[kk * kTileLd + C] : ((kk == C) ? (T)1 : (T)0);
        const T lv1 = (kk + 1 > C) ? A[(kk + 1) * kTileLd + C] : ((kk + 1 == C) ? (T)1 : (T)0);
        acc0 = accT(acc0, A[kk * kTileLd + R], lv0);
        acc1 = accT(acc1, A[(kk + 1) * kTileLd + R], lv1);
      }
      A[R * kTileLd + C] = accEnd(acc0) + accEnd(acc1);
    }
    __syncwarp();
    if (r < nb * 8) {
      const int Jb = r >> 3, j = r & 7;
      const int o = 8 * (Jb + d), C = 8 * Jb + j;
      for (int i = 7; i >= 0; --i) {
        T acc = A[(o + i) * kTileLd + C];
        for (int i2 = 0; i2 < i; ++i2) acc = accT(acc, A[(o + i) * kTileLd + o + i2], A[(o + i2) * kTileLd + C]);
        A[(o + i) * kTileLd + C] = -accEnd(acc);
      }
    }
    __syncwarp();
  }
}

// Diagonal tile factorisation: the register form for FP32, the blocked form for 8-byte types.
template <typename T>
__device__ __forceinline__ void tileFactorDiag(T* A, int J, int nr, int nx, const DevSettings& st, PivotStats* ps) {
  if constexpr (sizeof(T) == 4)
    tileFactorDiagRegs<T>(A, J, nr, nx, st, ps);
  else
    tileFactorDiagBlocked<T>(A, J, nr, nx, st, ps);
}

// L_IJ = A_IJ Linv_JJ^T D_J^-1 for one off-diagonal tile (one warp), in place. Column c of the
// result needs columns k <= c of A only, so the right half (c >= 16) is produced first.
template <typename T>
__device__ void tileOffDiag(T* Aij, const T* Ajj) {
  const int lane = threadIdx.x & 31, lr = lane & 7, lc = lane >> 3;
#pragma unroll
  for (int pass = 1; pass >= 0; --pass) {
    const int c0 = pass * 16 + lc * 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = (T)0;
#pragma unroll 2
    for (int k = 0; k < 32; ++k) {
      T av[4], cv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = Aij[k * kTileLd + lr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int col = c0 + j;
        cv[j] = (k < col) ? Ajj[col * kTileLd + k] : ((k == col) ? (T)1 : (T)0);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = accT(acc[i][j], av[i], cv[j]);
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = c0 + j;
      const T dinv = recipT(Ajj[col * kTileLd + col]);
#pragma unroll
      for (int i = 0; i < 4; ++i) Aij[col * kTileLd + lr * 4 + i] = accEnd(acc[i][j]) * dinv;
    }
    __syncwarp();
  }
}

// C -= A diag(d) B^T for 32x32 tiles (one warp); d = diagonal of the factored tile Ajj.
template <typename T>
__device__ void tileSyrk(T* C, const T* A, const T* B, const T* Ajj) {
  const int lane = threadIdx.x & 31, lr = lane & 7, lc = lane >> 3;
#pragma unroll
  for (int pass = 0; pass < 2; ++pass) {
    const int c0 = pass * 16 + lc * 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = (T)0;
#pragma unroll 2
    for (int k = 0; k < 32; ++k) {
      const T dk = Ajj[k * kTileLd + k];
      T av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = A[k * kTileLd + lr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = B[k * kTileLd + c0 + j] * dk;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = accT(acc[i][j], av[i], bv[j]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int i = 0; i < 4; ++i) C[(c0 + j) * kTileLd + lr * 4 + i] -= accEnd(acc[i][j]);
  }
}

// One 16x16 quadrant (qr, qc) of tileSyrk's C -= A diag(d) B^T, one warp: lane (r4, c2) takes
// rows qr*16 + 4 r4 + {0..3} and columns qc*16 + 2 c2 + {0, 1}. Every entry gets tileSyrk's
// operations in its order, so the result is the same.
template <typename T>
__device__ void tileSyrkQuad(T* C, const T* A, const T* B, const T* Ajj, int qr, int qc) {
  const int lane = threadIdx.x & 31, r0 = qr * 16 + (lane & 3) * 4, c0 = qc * 16 + (lane >> 2) * 2;
  T acc[4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i) acc[i][0] = acc[i][1] = (T)0;
#pragma unroll 4
  for (int k = 0; k < 32; ++k) {
    const T dk = Ajj[k * kTileLd + k];
    T av[4], bv[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) av[i] = A[k * kTileLd + r0 + i];
#pragma unroll
    for (int j = 0; j < 2; ++j) bv[j] = B[k * kTileLd + c0 + j] * dk;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) acc[i][j] = accT(acc[i][j], av[i], bv[j]);
  }
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) C[(c0 + j) * kTileLd + r0 + i] -= accEnd(acc[i][j]);
}

template <typename T>
__device__ __noinline__ void denseLdlt(Ctx& c, T* M, const DevSettings& st, int& fail, int& wrongSign, double& minAbsD) {
  const int nr = c.nr, nx = c.n, Tn = rootTiles(nr);
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  PivotStats* ps = reinterpret_cast<PivotStats*>(c.sc + SC_COUNT);
  if (threadIdx.x == 0) {
    ps->nreg = 0;
    ps->zero = 0;
    ps->wrong = 0;
    ps->minAbs = INFINITY;
  }
  __syncthreads();
  // Right-looking by tile column with a one-column lookahead: warp 0 applies column J's update
  // to the next diagonal tile and factors it while the other warps apply the rest of column J.
  if (warp == 0) tileFactorDiag<T>(M, 0, nr, nx, st, ps);
  __syncthreads();
  for (int J = 0; J + 1 < Tn; ++J) {
    T* Ajj = M + tileBase(Tn, J, J);
    for (int I = J + 1 + warp; I < Tn; I += nw) tileOffDiag<T>(M + tileBase(Tn, I, J), Ajj);
    __syncthreads();
    const int rem = Tn - J - 1;
    const int npairs = rem * (rem + 1) / 2;
    if (nw >= 4 && warp < 3) {
      // the next diagonal tile's update, the head of the critical path, on three warps: the
      // quadrants the factorisation reads (the upper-right one is overwritten by Linv anyway)
      T* Anext = M + tileBase(Tn, J + 1, J + 1);
      const T* Lnext = M + tileBase(Tn, J + 1, J);
      tileSyrkQuad<T>(Anext, Lnext, Lnext, Ajj, warp == 0 ? 0 : 1, warp == 2 ? 1 : 0);
      asm volatile("bar.sync 1, 96;" ::: "memory");
    }
    if (warp == 0 || nw == 1) {
      T* Anext = M + tileBase(Tn, J + 1, J + 1);
      const T* Lnext = M + tileBase(Tn, J + 1, J);
      if (nw < 4) tileSyrk<T>(Anext, Lnext, Lnext, Ajj);
      if (nw == 1) {
        for (int t = 1; t < npairs; ++t) {
          int K = J + 1, tt = t, len = rem;
          while (tt >= len) { tt -= len; --len; ++K; }
          const int I = K + tt;
          tileSyrk<T>(M + tileBase(Tn, I, K), M + tileBase(Tn, I, J), M + tileBase(Tn, K, J), Ajj);
        }
      }
      tileFactorDiag<T>(Anext, J + 1, nr, nx, st, ps);
    } else {
      // pairs t >= 1: (I, K) with J < K <= I < Tn, enumerated column by column (t = 0 is the
      // next diagonal tile)
      for (int t = warp; t < npairs; t += nw - 1) {
        int K = J + 1, tt = t, len = rem;
        while (tt >= len) { tt -= len; --len; ++K; }
        const int I = K + tt;
        tileSyrk<T>(M + tileBase(Tn, I, K), M + tileBase(Tn, I, J), M + tileBase(Tn, K, J), Ajj);
      }
    }
    __syncthreads();
  }
  const bool regularized = st.linear_solver == 2;
  fail = regularized ? (((double)ps->nreg > 0.05 * (double)nr) ? 1 : 0) : ps->zero;
  wrongSign = ps->wrong;
  minAbsD = ps->minAbs;
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ T shflXorT(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ df64 shflXorT(df64 v, int m) {
  return df64(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
}

// Largest split s in {1, 2, 4, 8} of a 32-term dot product such that rows * s threads fit in
// one pass of the block (rows is a multiple of 32, so each warp holds whole groups of s lanes).
__device__ __forceinline__ int dotSplit(int rows) {
  int s = 1;
  while (s < 8 && rows * s * 2 <= (int)blockDim.x) s *= 2;
  return s;
}

// Sum of a dot-product partial over the s consecutive lanes of a group (s a power of two <= 8).
template <typename T>
__device__ __forceinline__ T groupSum(T v, int s) {
  for (int m = 1; m < s; m <<= 1) v = v + shflXorT(v, m);
  return v;
}

// y <- M^-1 y for the factored tiled root; y has Tn*32 entries (padding entries are zero).
// Every block product (the diagonal tile's Linv and each off-diagonal tile) is a set of 32-term
// dot products, split over s lanes per row (dotSplit) and reduced by shuffles, so that the few
// rows of the late steps still occupy the whole block.
template <typename T>
__device__ void denseSolve(Ctx& c, const T* M, T* y) {
  const int Tn = rootTiles(c.nr);
  const int nth = blockDim.x;
  // forward: y_J = Linv_JJ y_J, then y_I -= L_IJ y_J for I > J
  for (int J = 0; J < Tn; ++J) {
    const T* Ajj = M + tileBase(Tn, J, J);
    T* yJ = y + J * 32;
    {
      const int sd = dotSplit(32), w = 32 / sd;
      T tot = (T)0;
      int i = 0, p = 0;
      if ((int)threadIdx.x < 32 * sd) {
        i = threadIdx.x / sd;
        p = threadIdx.x % sd;
        T acc = (T)0;
        for (int col = p * w; col < (p + 1) * w && col < i; ++col) acc = accT(acc, Ajj[i * kTileLd + col], yJ[col]);
        tot = groupSum(accEnd(acc), sd);
      }
      __syncthreads();
      if ((int)threadIdx.x < 32 * sd && p == 0) yJ[i] = yJ[i] + tot;
      __syncthreads();
    }
    const int rows = (Tn - J - 1) * 32;
    if (rows > 0) {
      const int s = dotSplit(rows), w = 32 / s;
      for (int t = threadIdx.x; t < rows * s; t += nth) {
        const int row = t / s, p = t % s;
        const int I = J + 1 + row / 32, rr = row % 32;
        const T* Lij = M + tileBase(Tn, I, J);
        T acc = (T)0;
#pragma unroll 4
        for (int col = p * w; col < (p + 1) * w; ++col) acc = accT(acc, Lij[col * kTileLd + rr], yJ[col]);
        acc = groupSum(accEnd(acc), s);
        if (p == 0) y[I * 32 + rr] -= acc;
      }
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < Tn * 32; t += nth) {
    const int J = t / 32, rr = t % 32;
    y[t] /= M[tileBase(Tn, J, J) + rr * kTileLd + rr];
  }
  __syncthreads();
  // backward: x_J = Linv_JJ^T y_J, then y_K -= L_JK^T x_J for K < J
  for (int J = Tn - 1; J >= 0; --J) {
    const T* Ajj = M + tileBase(Tn, J, J);
    T* yJ = y + J * 32;
    {
      const int sd = dotSplit(32), w = 32 / sd;
      T tot = (T)0;
      int i = 0, p = 0;
      if ((int)threadIdx.x < 32 * sd) {
        i = threadIdx.x / sd;
        p = threadIdx.x % sd;
        T acc = (T)0;
        for (int row = p * w; row < (p + 1) * w; ++row)
          if (row > i) acc = accT(acc, Ajj[row * kTileLd + i], yJ[row]);
        tot = groupSum(accEnd(acc), sd);
      }
      __syncthreads();
      if ((int)threadIdx.x < 32 * sd && p == 0) yJ[i] = yJ[i] + tot;
      __syncthreads();
    }
    if (J == 0) break;
    const int rows = J * 32;
    const int s = dotSplit(rows), w = 32 / s;
    for (int t = threadIdx.x; t < rows * s; t += nth) {
      const int row = t / s, p = t % s;
      const int K = row / 32, cc = row % 32;
      const T* Ljk = M + tileBase(Tn, J, K);
      T acc = (T)0;
#pragma unroll 4
      for (int r2 = p * w; r2 < (p + 1) * w; ++r2) acc = accT(acc, Ljk[cc * kTileLd + r2], yJ[r2]);
      acc = groupSum(accEnd(acc), s);
      if (p == 0) y[K * 32 + cc] -= acc;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------
// whole-GPU root (single large instance)
// ------------------------------------------------------------------------------------------
// One instance whose root is too large for one SM runs as a cooperative launch with one CTA
// per SM: CTA 0 runs the interior-point iteration exactly as the batched kernel does, and at the
// two root-sized steps, assembly + LDL' and the triangular solves, it posts a job that every
// CTA runs with it. Jobs are the same tile operations in the same order per tile as the
// single-CTA root, spread over the warps of the grid, with a grid barrier between dependent
// steps (two per tile column of the factor, one per tile of each triangular pass).
enum { kGridOpFactor = 1, kGridOpSolve = 2, kGridOpExit = 3 };

struct GridCtl {
  unsigned arrive;   // barrier: arrivals in the current round
  unsigned gen;      // barrier: completed rounds
  int error;         // a barrier wait ran out; every later barrier fails at once
  int op;            // job posted by CTA 0
  int arith;         // root arithmetic of the job: 0 FP64, 1 FP32, 2 double-float
  int pad;
  void* M;           // root of the job
  void* y;           // solve vector (root arithmetic), rootTiles(nr) * 32 entries
  double ep, ea;     // regularisation bumps of the assembly
  int64_t stageOff;  // byte offset of the tile staging area in dynamic shared memory
  unsigned long long waitNs;  // longest barrier wait; 0 = kGridWaitNs
  Ctx ctx;           // CTA 0's instance context (pointers into global memory only)
};

// Shared memory of the whole-GPU trailing update for one 128x128 super-block (4x4 tiles): the
// panel rows A[32][128] and the D-scaled panel columns B[32][128] (k-major), and the 16 result
// tiles in tile layout.
constexpr int kSbDim = 128;
constexpr int kStageElems = 2 * kTile * kSbDim + 16 * kTileElems;
constexpr int64_t gridStageBytes(int elemBytes) { return (int64_t)kStageElems * elemBytes; }

template <typename T> struct ArithOf;
template <> struct ArithOf<double> { static constexpr int v = 0; };
template <> struct ArithOf<float> { static constexpr int v = 1; };
template <> struct ArithOf<df64> { static constexpr int v = 2; };

__device__ __forceinline__ unsigned long long globalNs() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Longest wait at one grid barrier. CTA 0's own work between two root jobs (cone scaling,
// residuals, KKT residual products) takes milliseconds; a wait this long means a CTA is gone.
constexpr unsigned long long kGridWaitNs = 30ull * 1000ull * 1000ull * 1000ull;

// Grid-wide barrier of a cooperative launch (every CTA resident). Thread 0 of each CTA arrives
// after a fence (release); the last arrival resets the count and opens the next round; the
// others poll the round number and fence after it changes (acquire). Each wait is bounded by
// kGridWaitNs: a wait that runs out records an error, and from then on every barrier of every
// CTA returns false at once, so the launch always ends.
static __device__ __noinline__ bool gridSync(GridCtl* g) {
  __shared__ int sOk;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile GridCtl* vg = g;
    int ok = vg->error == 0;
    if (ok) {
      unsigned long long limit = vg->waitNs;
      if (limit == 0) limit = kGridWaitNs;
      const unsigned gen = vg->gen;
      __threadfence();
      const unsigned prev = atomicAdd(&g->arrive, 1u);
      if (prev == gridDim.x - 1) {
        atomicExch(&g->arrive, 0u);
        __threadfence();
        atomicAdd(&g->gen, 1u);
      } else {
        const unsigned long long t0 = globalNs();
        unsigned backoff = 32;  // ns, doubled up to 512 while the wait lasts
        while (vg->gen == gen) {
          if (vg->error) { ok = 0; break; }
          if (globalNs() - t0 > limit) {
            atomicExch(&g->error, 1);
            ok = 0;
            break;
          }
          __nanosleep(backoff);
          if (backoff < 512) backoff <<= 1;
        }
      }
      __threadfence();
    }
    sOk = ok;
  }
  __syncthreads();
  return sOk != 0;
}

// Root assembly spread over the grid, the same writes as the single-CTA assembly in
// assembleFactor: zero, then the distinct entries (padding identity, P diagonal + bump,
// strictly-upper P, Zero-row A, Zero-row diagonal), then the cone-unit contributions (one target
// root entry per thread, so no two threads add into the same entry).
template <typename T>
__device__ __noinline__ bool gridAssemble(GridCtl* g, const Ctx& c, const DevSettings& st, T* M, double ep, double ea) {
  const InstanceDesc& D = *c.D;
  const int n = c.n, nr = c.nr;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
  const int64_t rs = rootSize(nr);
  for (int64_t t = gt; t < rs; t += gs) M[t] = (T)0;
  if (!gridSync(g)) return false;
  for (int64_t i = nr + gt; i < (int64_t)rootTiles(nr) * kTile; i += gs) M[rootIdx(nr, (int)i, (int)i)] = (T)1;
  for (int64_t i = gt; i < n; i += gs) {
    const int src = c.pdiag[i];
    M[rootIdx(nr, (int)i, (int)i)] = (T)(((src >= 0) ? c.Pu[src] : 0.0) + st.static_reg_P + ep);
  }
  for (int64_t k = gt; k < D.nPlow; k += gs) M[c.plowIdx[k]] = (T)c.Pu[c.plowSrc[k]];
  for (int64_t k = gt; k < D.nAZ; k += gs) M[c.azIdx[k]] = (T)c.Av[c.azSrc[k]];
  for (int64_t r = gt; r < c.p; r += gs) M[rootIdx(nr, n + (int)r, n + (int)r)] = (T)(-(st.static_reg_A + ea));
  if (!gridSync(g)) return false;
  for (int64_t t = gt; t < D.nTgt; t += gs) {
    double acc = 0.0;
    for (int q = c.tgtBeg[t]; q < c.tgtBeg[t + 1]; ++q) {
      const int oi = c.contrib[3 * q], oj = c.contrib[3 * q + 1], d = c.contrib[3 * q + 2];
      for (int r = 0; r < d; ++r) acc += c.Ad[oi + r] * c.T[oj + r];
    }
    M[c.tgtIdx[t]] += (T)acc;
  }
  return gridSync(g);
}

// Four consecutive entries of a shared-memory row (16-byte aligned for 4-byte T, two 16-byte
// halves for 8-byte T).
template <typename T>
__device__ __forceinline__ void lds4(const T* p, T (&v)[4]) {
  if constexpr (sizeof(T) == 4) {
    const float4 f = *reinterpret_cast<const float4*>(p);
    v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = p[i];
  }
}

// C -= A D B^T for one super-block of up to 4x4 tiles, by one CTA of 256 threads:
// rows I0 .. I0+ni-1 and columns K0 .. K0+nk-1 (tile indices); only tiles with column <= row when
// the super-block is on the diagonal, and not its first tile when skip00 (updated elsewhere).
// A = the panel tiles L_IJ, B = L_KJ, D = diag of tile (J, J).
// The C tiles are copied into shared memory asynchronously (cp.async) while the panel is staged
// k-major (B pre-scaled by D exactly as tileSyrk scales it) and each thread accumulates an 8x8
// block of the 128x128 product over k = 0..31 in the order tileSyrk uses; then C -= product in
// shared memory (so every entry gets the same bits as tileSyrk) and the tiles are stored back
// with 16-byte vectors.
template <typename T>
__device__ __noinline__ void superSyrk(T* M, int Tn, int J, int I0, int K0, int ni, int nk, bool diagSb, bool skip00,
                                      T* sm) {
  T* As = sm;
  T* Bs = sm + kTile * kSbDim;
  T* Cs = sm + 2 * kTile * kSbDim;
  const T* Ajj = M + tileBase(Tn, J, J);
  const int tid = threadIdx.x;
  constexpr int per16 = 16 / (int)sizeof(T);
  constexpr int vpt = kTileElems / per16;  // 16-byte vectors per tile
  // (1) the C tiles of this super-block, global -> Cs, as asynchronous 16-byte copies that
  //     proceed while the panel is staged and the product computed
  for (int v = tid; v < 16 * vpt; v += blockDim.x) {
    const int t = v / vpt, a = t >> 2, b = t & 3;
    if (a < ni && b < nk && !(diagSb && b > a) && !(skip00 && t == 0)) {
      const T* src = M + tileBase(Tn, I0 + a, K0 + b) + (v - t * vpt) * per16;
      const unsigned dst = (unsigned)__cvta_generic_to_shared(Cs + v * per16);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  {
    // (2) the panel: thread tid stages column i = tid & 127 for k = tid >> 7, +2, ... (all loads
    //     of a half issued before any store, so their latencies overlap)
    const int i = tid & (kSbDim - 1), a = i >> 5, rr = i & 31, k0 = tid >> 7;
    const T* pa = (a < ni) ? M + tileBase(Tn, I0 + a, J) + rr : nullptr;
    const T* pb = (a < nk) ? M + tileBase(Tn, K0 + a, J) + rr : nullptr;
    constexpr int kPer = 8;  // 256 threads: two k rows per step, 8 steps per half
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      T va[kPer], vb[kPer], dk[kPer];
#pragma unroll
      for (int t = 0; t < kPer; ++t) {
        const int k = k0 + 2 * (h * kPer + t);
        va[t] = pa ? pa[k * kTileLd] : (T)0;
        vb[t] = pb ? pb[k * kTileLd] : (T)0;
        dk[t] = Ajj[k * kTileLd + k];
      }
#pragma unroll
      for (int t = 0; t < kPer; ++t) {
        const int k = k0 + 2 * (h * kPer + t);
        As[k * kSbDim + i] = va[t];
        Bs[k * kSbDim + i] = pb ? vb[t] * dk[t] : (T)0;
      }
    }
  }
  __syncthreads();
  // (3) the product, 8x8 per thread, k = 0..31 in the tile routine's order
  const int tx = tid & 15, ty = tid >> 4;  // rows tx*4 + {0..3, 64..67}, columns ty*4 + {0..3, 64..67}
  T acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = (T)0;
#pragma unroll 2
  for (int k = 0; k < kTile; ++k) {
    T a0[4], a1[4], b0[4], b1[4];
    lds4(As + k * kSbDim + tx * 4, a0);
    lds4(As + k * kSbDim + 64 + tx * 4, a1);
    lds4(Bs + k * kSbDim + ty * 4, b0);
    lds4(Bs + k * kSbDim + 64 + ty * 4, b1);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc[i][j] = accT(acc[i][j], a0[i], b0[j]);
        acc[i][4 + j] = accT(acc[i][4 + j], a0[i], b1[j]);
        acc[4 + i][j] = accT(acc[4 + i][j], a1[i], b0[j]);
        acc[4 + i][4 + j] = accT(acc[4 + i][4 + j], a1[i], b1[j]);
      }
  }
  // (4) C -= product in shared memory (each thread its own 64 entries of the copied C tiles;
  //     entries of tiles that are not updated are never stored back)
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int R = (i < 4) ? tx * 4 + i : 64 + tx * 4 + (i - 4);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int Cc = (j < 4) ? ty * 4 + j : 64 + ty * 4 + (j - 4);
      T& cref = Cs[((R >> 5) * 4 + (Cc >> 5)) * kTileElems + (Cc & 31) * kTileLd + (R & 31)];
      cref = cref - accEnd(acc[i][j]);
    }
  }
  __syncthreads();
  // (5) back to global memory, 16-byte vectors
  for (int v = tid; v < 16 * vpt; v += blockDim.x) {
    const int t = v / vpt, a = t >> 2, b = t & 3;
    if (a < ni && b < nk && !(diagSb && b > a) && !(skip00 && t == 0))
      *reinterpret_cast<uint4*>(M + tileBase(Tn, I0 + a, K0 + b) + (v - t * vpt) * per16) =
          *reinterpret_cast<const uint4*>(Cs + v * per16);
  }
}

// FP32 trailing update of tile column J on the tensor cores (tcgen05, kind::tf32): the same
// C_IK -= L_IJ D_J L_KJ^T as superSyrk, over every super-block this CTA owns in the step
// (sb = blockIdx.x - 1, + gridDim.x - 1, ...). Each FP32 operand is split as hi + lo (hi = its
// TF32 rounding, lo = the TF32 rounding of the remainder) and the product taken as
// A_lo B_hi + A_hi B_lo + A_hi B_hi (3xTF32; the A_lo B_lo term is below FP32 rounding): twelve
// 128x128x8 MMAs accumulating in FP32 in TMEM, issued by one thread. Software pipeline: the C tiles
// of the next super-block arrive by bulk copies (TMA) into the other of two shared-memory buffers
// while the current super-block's panels are staged (generic loads, TF32 split), multiplied and
// its tiles updated from TMEM and written back by bulk copies. All bulk stores of the step are
// complete (and ordered before later generic accesses) when it returns.
// Shared memory `sm` (128-byte aligned, kGridTcStageBytes): the operand panels A_hi, A_lo, B_hi,
// B_lo (16 KB each, layout of cxg_tc.cuh), then two buffers of 16 C tiles. `tmem`: this CTA's 128
// accumulator columns; mbarriers: MMA completion and one per C buffer, with their phase parities.
// Returns false when a wait ran out (after waiting once more for the copies in flight).
constexpr int64_t kTcStageBytes = kGridTcStageBytes;
constexpr unsigned long long kTcWaitNs = 2ull * 1000ull * 1000ull * 1000ull;
constexpr uint32_t kTileBytes = (uint32_t)kTileElems * 4u;

struct SbGeo {
  int I0, K0, ni, nk;
  bool diag, skip00;
};

// the super-block sb of step J (row order: sb = r (r + 1) / 2 + k, tile rows J+1+4r.., tile
// columns J+1+4k..; super-block 0 without the tile (J+1, J+1), which CTA 0 updates)
__device__ __forceinline__ SbGeo sbGeo(long long sb, int J, int Tn) {
  int r = (int)((sqrtf(8.0f * (float)sb + 1.0f) - 1.0f) * 0.5f);
  while ((long long)r * (r + 1) / 2 > sb) --r;
  while ((long long)(r + 1) * (r + 2) / 2 <= sb) ++r;
  const int k = (int)(sb - (long long)r * (r + 1) / 2);
  SbGeo g;
  g.I0 = J + 1 + 4 * r;
  g.K0 = J + 1 + 4 * k;
  g.ni = min(4, Tn - g.I0);
  g.nk = min(4, Tn - g.K0);
  g.diag = r == k;
  g.skip00 = sb == 0;
  return g;
}

// tile t = 4a + b of the super-block is updated (and so loaded and stored) by it
__device__ __forceinline__ bool sbTile(const SbGeo& g, int t) {
  const int a = t >> 2, b = t & 3;
  return a < g.ni && b < g.nk && !(g.diag && b > a) && !(g.skip00 && t == 0);
}

static __device__ __noinline__ bool tcTrailingStep(float* M, int Tn, int J, long long nsb, unsigned char* sm,
                                                   uint32_t tmem, uint32_t mbarMma, uint32_t mbarLd0,
                                                   uint32_t mbarLd1, uint32_t& phMma, uint32_t& phLd0,
                                                   uint32_t& phLd1) {
  const int tid = threadIdx.x;
  const long long first = (long long)blockIdx.x - 1, stride = (long long)gridDim.x - 1;
  if (first >= nsb) return true;
  const float* Ajj = M + tileBase(Tn, J, J);
  const uint32_t opBase = tc::smemAddr(sm);
  const uint32_t cAddr[2] = {opBase + 4u * tc::kPanelBytes, opBase + 4u * tc::kPanelBytes + 16u * kTileBytes};
  float* cPtr[2] = {reinterpret_cast<float*>(sm + 4 * tc::kPanelBytes),
                    reinterpret_cast<float*>(sm + 4 * tc::kPanelBytes + 16 * kTileBytes)};
  const uint32_t mbarLd[2] = {mbarLd0, mbarLd1};
  // thread 0: the C tiles of super-block g into buffer buf, completing on that buffer's mbarrier
  auto issueLoads = [&](const SbGeo& g, int buf) {
    uint32_t bytes = 0;
    for (int t = 0; t < 16; ++t)
      if (sbTile(g, t)) bytes += kTileBytes;
    tc::mbarArriveExpectTx(mbarLd[buf], bytes);
    for (int t = 0; t < 16; ++t)
      if (sbTile(g, t))
        tc::bulkLoad(cAddr[buf] + (uint32_t)t * kTileBytes, M + tileBase(Tn, g.I0 + (t >> 2), g.K0 + (t & 3)),
                     kTileBytes, mbarLd[buf]);
  };
  if (tid == 0) {
    tc::fenceProxyAsyncGlobal();  // the previous step's generic writes before these async reads
    issueLoads(sbGeo(first, J, Tn), 0);
  }
  int buf = 0;
  for (long long sb = first; sb < nsb; sb += stride, buf ^= 1) {
    const SbGeo g = sbGeo(sb, J, Tn);
    if (tid == 0 && sb + stride < nsb) {
      tc::bulkWaitRead0();  // the previous super-block's stores have read the other buffer
      issueLoads(sbGeo(sb + stride, J, Tn), buf ^ 1);
    }
    // panels: thread tid stages row i = tid & 127 of A (L_IJ, tid < 128) or of B (D-scaled L_KJ),
    // four k at a time, as TF32 hi and lo parts; row m sits at byte (k / 4) * 2048 + m * 16 + (k % 4) * 4
    if (tid < 2 * tc::kRows) {
      const int i = tid & (tc::kRows - 1), isB = tid >> 7, a = i >> 5, rr = i & 31;
      const int nt = isB ? g.nk : g.ni;
      const float* src = (a < nt) ? M + tileBase(Tn, (isB ? g.K0 : g.I0) + a, J) + rr : nullptr;
      unsigned char* hiBase = sm + (isB ? 2 : 0) * tc::kPanelBytes;
      unsigned char* loBase = hiBase + tc::kPanelBytes;
#pragma unroll 2
      for (int kq = 0; kq < kTile / 4; ++kq) {
        float hi[4], lo[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int k = 4 * kq + t;
          float x = src ? src[k * kTileLd] : 0.0f;
          if (isB) x = x * Ajj[k * kTileLd + k];
          hi[t] = tc::toTf32(x);
          lo[t] = tc::toTf32(x - hi[t]);
        }
        *reinterpret_cast<float4*>(hiBase + kq * 2048 + i * 16) = make_float4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<float4*>(loBase + kq * 2048 + i * 16) = make_float4(lo[0], lo[1], lo[2], lo[3]);
      }
    }
    tc::fenceProxyAsyncShared();
    __syncthreads();
    if (tid == 0) {
      tc::fenceAfterSync();
      const uint32_t aHi = opBase, aLo = opBase + tc::kPanelBytes, bHi = opBase + 2 * tc::kPanelBytes,
                     bLo = opBase + 3 * tc::kPanelBytes;
      constexpr uint32_t idesc = tc::idescTf32(tc::kRows, tc::kRows);
      for (int sK = 0; sK < kTile / 8; ++sK) {
        const uint32_t o = (uint32_t)sK * 4096u;
        tc::mmaTf32(tmem, tc::smemDesc(aLo + o), tc::smemDesc(bHi + o), idesc, sK > 0);
        tc::mmaTf32(tmem, tc::smemDesc(aHi + o), tc::smemDesc(bLo + o), idesc, true);
      }
      for (int sK = 0; sK < kTile / 8; ++sK) {
        const uint32_t o = (uint32_t)sK * 4096u;
        tc::mmaTf32(tmem, tc::smemDesc(aHi + o), tc::smemDesc(bHi + o), idesc, true);
      }
      tc::commitTo(mbarMma);
    }
    // the product and this buffer's C tiles (bounded waits; one vote for the whole CTA)
    uint32_t& phLd = buf ? phLd1 : phLd0;
    bool ok = tc::mbarWait(mbarMma, phMma, kTcWaitNs);
    ok = tc::mbarWait(mbarLd[buf], phLd, kTcWaitNs) && ok;
    phMma ^= 1u;
    phLd ^= 1u;
    tc::fenceAfterSync();
    if (!__syncthreads_and(ok)) {
      // a wait ran out: give the copies and MMAs in flight one more period, then give up
      tc::mbarWait(mbarMma, phMma ^ 1u, kTcWaitNs);
      tc::mbarWait(mbarLd[buf ^ 1], buf ? phLd0 : phLd1, kTcWaitNs);
      if (tid == 0) tc::bulkWait0();
      __syncthreads();
      return false;
    }
    // C -= product: warp w reads TMEM lanes 32 (w % 4) .. +31 (its rows), columns 64 (w / 4) ..
    // +63, sixteen at a time
    {
      float* Cs = cPtr[buf];
      const int warp = tid >> 5, lane = tid & 31;
      if (warp < 8) {
        const int q = warp & 3, h = warp >> 2;
        const int R = 32 * q + lane;
        for (int cb = 0; cb < 4; ++cb) {
          float d[16];
          const int c0 = 64 * h + 16 * cb;
          tc::tmemLoad16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, d);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int Cc = c0 + j;
            float& cref = Cs[((R >> 5) * 4 + (Cc >> 5)) * kTileElems + (Cc & 31) * kTileLd + (R & 31)];
            cref = cref - d[j];
          }
        }
      }
    }
    tc::fenceProxyAsyncShared();  // the updated tiles visible to the bulk stores
    tc::fenceBeforeSync();
    __syncthreads();
    if (tid == 0) {
      for (int t = 0; t < 16; ++t)
        if (sbTile(g, t))
          tc::bulkStore(M + tileBase(Tn, g.I0 + (t >> 2), g.K0 + (t & 3)), cAddr[buf] + (uint32_t)t * kTileBytes,
                        kTileBytes);
      tc::bulkCommit();
    }
  }
  if (tid == 0) {
    tc::bulkWait0();
    tc::fenceProxyAsyncGlobal();  // the stores before the grid barrier's generic release
  }
  __syncthreads();
  return true;
}

// tensor-core state of a CTA for the length of one factorisation job
struct TcState {
  unsigned char* stage;  // kGridTcStageBytes, 128-byte aligned
  uint32_t tmem, mbar;   // TMEM base; three mbarriers at mbar, mbar + 8, mbar + 16
  uint32_t phMma, phLd0, phLd1;
};

// Double-float trailing update on the tensor cores (tcgen05, kind::f16 with BF16 operands), over a
// pair of tile columns (J0, J0 + 1) at once: C_IK -= L_I,pair D_pair L_K,pair^T, K = 64, by an
// error-free split of the double-float operands into BF16 slices (the splitting scheme of Ozaki,
// Ogita, Oishi and Rump, Numer. Algorithms 59, 2012, on BF16 tensor products with FP32
// accumulation):
//  - each 64-wide row of the panels A = [L_I,J0 L_I,J0+1] and B = A D (the double-float products
//    of the tile routine) is scaled by a power of two 2^-e (e = 1 + the exponent of its largest
//    entry), so that every entry r lies in [-1, 1], and split as r = a_0 + a_1 + ... + a_5 + rest
//    with a_s = round(r_s 2^(8 s + 8)) 2^(-8 s - 8), r_0 = r, r_(s+1) = r_s - a_s: each a_s has at
//    most eight significant bits (a BF16 value), every subtraction is exact (Sterbenz), and the
//    rest is below 2^-48, the resolution of the double-float value (sliceRowPair, once per tile
//    row, by the warp that computed the row's second tile);
//  - a slice product a_i b_j is an integer multiple of 2^(-8(i + j) - 16) of at most 2^16, so a
//    sum of 64 of them over one, two or three pairs of one order i + j stays below 2^24, exact in
//    an FP32 accumulator: orders 0, 1, 2 accumulate exactly in three 128 x 128 TMEM accumulators,
//    orders 3 to 5 (whose rounding lies below 2^-48 of the product) in a fourth; the pairs of
//    order 6 and above are below 2^-48 and left out. 84 MMAs of 128 x 128 x 16 per super-block,
//    issued by one thread;
//  - the four accumulators are summed in double-float (error-free sums), scaled back by
//    2^(e_A + e_B) and subtracted from the C tiles in place in global memory.
// Against the double-float product on the CUDA cores the error bound changes from 2^-48 times the
// sum of |a_k b_k| to about 2^-45 times (max_k |a_k|)(max_k |b_k|); on quasi-definite roots with
// pivots spread over 1e20 the factor's componentwise backward error stays near 3e-14 (FP64:
// 8e-16).
//
// Slice area (global, `slices`, dfSliceBytes): for operand o (0 = A, 1 = B), slice s and k-group
// kg (8 of the 64 columns), the 16 bytes of root row m at ((o * 6 + s) * 8 + kg) * rows * 16 +
// m * 16, i.e. each (o, s, kg) plane holds the canonical shared-memory layout of cxg_tc.cuh for
// every row, so the 128 rows of a super-block are one contiguous copy per plane; then the row
// exponents, int32, at 1536 * rows + (o * rows + m) * 4.
constexpr int kDfSlices = 6;
constexpr int kDfK = 2 * kTile;                                          // columns per C visit
constexpr uint32_t kDfPanelBytes = (uint32_t)tc::kRows * kDfK * 2;       // 16 KB: 128 x 64 BF16
constexpr uint32_t kDfTmemCols = 512;                                    // four FP32 accumulators
constexpr uint32_t kDfOpBytes = 2 * kDfSlices * kDfPanelBytes;           // 192 KB of operands
constexpr uint32_t kDfExpBytes = 2 * tc::kRows * 4;                      // row exponents, A and B
constexpr int64_t kDfStageBytes = (int64_t)kDfOpBytes + 2 * kDfExpBytes; // one operand + two exponent buffers
static_assert(kDfStageBytes + 128 <= kGridTcStageBytes, "double-float staging exceeds the stage area");

// x 2^ex, by one exact multiplication where 2^ex is a normal float (scalbnf otherwise)
__device__ __forceinline__ float pow2Scale(float x, int ex) {
  if (ex >= -126 && ex <= 127) return __fmul_rn(x, __int_as_float((ex + 127) << 23));
  return scalbnf(x, ex);
}

// Writes the slices (A and B) of the 32 rows of tile row I over the tile columns J0, J0 + 1 and
// their exponents; one warp, lane rr takes row 32 I + rr. L_I,J0 and L_I,J0+1 must be complete
// in M (the second written by this warp, the first before the last grid barrier).
static __device__ __noinline__ void sliceRowPair(const df64* M, int Tn, int I, int J0, unsigned char* slices) {
  __syncwarp();
  const int rr = threadIdx.x & 31;
  const int64_t rows = (int64_t)Tn * kTile, m = (int64_t)I * kTile + rr;
  const df64* src[2] = {M + tileBase(Tn, I, J0) + rr, M + tileBase(Tn, I, J0 + 1) + rr};
  const df64* dg[2] = {M + tileBase(Tn, J0, J0), M + tileBase(Tn, J0 + 1, J0 + 1)};
  for (int o = 0; o < 2; ++o) {
    auto value = [&](int k) -> df64 {
      const int t = k >> 5, kk = k & 31;
      df64 x = src[t][kk * kTileLd];
      if (o) x = x * dg[t][kk * kTileLd + kk];
      return x;
    };
    float mx = 0.0f;
#pragma unroll 8
    for (int k = 0; k < kDfK; ++k) mx = fmaxf(mx, fabsf(value(k).hi));
    const int e = (mx > 0.0f && mx <= 3.0e38f) ? ilogbf(mx) + 1 : 0;
    reinterpret_cast<int*>(slices + 1536 * rows)[o * rows + m] = e;
#pragma unroll 1
    for (int kg = 0; kg < kDfK / 8; ++kg) {
      uint32_t w[kDfSlices][4];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const df64 v = value(8 * kg + t);
        float rh = pow2Scale(v.hi, -e), rl = pow2Scale(v.lo, -e);
        float p = 256.0f, pinv = 1.0f / 256.0f;
#pragma unroll
        for (int sl = 0; sl < kDfSlices; ++sl) {
          const float as = __fmul_rn(rintf(__fmul_rn(rh, p)), pinv);  // exact: <= 8 significant bits
          const uint32_t bits = __float_as_uint(as) >> 16;               // its BF16 pattern
          if (t & 1) w[sl][t >> 1] |= bits << 16;
          else w[sl][t >> 1] = bits;
          dfTwoSum(__fsub_rn(rh, as), rl, rh, rl);
          p = __fmul_rn(p, 256.0f);
          pinv = __fmul_rn(pinv, 1.0f / 256.0f);
        }
      }
#pragma unroll
      for (int sl = 0; sl < kDfSlices; ++sl)
        *reinterpret_cast<uint4*>(slices + ((int64_t)(o * kDfSlices + sl) * (kDfK / 8) + kg) * rows * 16 + m * 16) =
            make_uint4(w[sl][0], w[sl][1], w[sl][2], w[sl][3]);
    }
  }
}

// The trailing update of column pair (J - 1, J) over the super-blocks this CTA owns (sb =
// blockIdx.x - 1, + gridDim.x - 1, ...; tile rows and columns from J + 1). Per super-block: its
// slices and exponents arrive by bulk copies (TMA); one thread issues its 84 MMAs; once they are
// complete the operand buffer holds the super-block's C tiles instead (bulk copies from HBM),
// which are updated there from the accumulators and written back by bulk copies; once those have
// read the buffer, the next super-block's slices are issued into it (the exponents alternate
// between two buffers). Shared memory `sm` (128-byte aligned): kDfStageBytes. `tmem`: this CTA's
// 512 accumulator columns; mbarriers: MMA completion, slice copies and C copies, with their phase
// parities. Returns false when a wait ran out (after waiting once more for what is in flight).
static __device__ __noinline__ bool tcDfTrailingStep(df64* M, int Tn, int J, long long nsb, const unsigned char* slices,
                                                     unsigned char* sm, uint32_t tmem, uint32_t mbarMma,
                                                     uint32_t mbarLd, uint32_t mbarC, uint32_t& phMma, uint32_t& phLd,
                                                     uint32_t& phC) {
  const int tid = threadIdx.x;
  const long long first = (long long)blockIdx.x - 1, stride = (long long)gridDim.x - 1;
  if (first >= nsb) return true;
  const int64_t rows = (int64_t)Tn * kTile;
  const uint32_t opAddr = tc::smemAddr(sm);
  const uint32_t expAddr[2] = {opAddr + kDfOpBytes, opAddr + kDfOpBytes + kDfExpBytes};
  constexpr int kPlanes = kDfSlices * (kDfK / 8);  // per operand
  constexpr uint32_t kTileBytesDf = (uint32_t)kTileElems * 8u;
  df64* Cs = reinterpret_cast<df64*>(sm);  // the C tiles, where the operands were
  // thread 0: the slices of super-block g's A rows (tiles I0 ..) and B rows (K0 ..), exponents
  // into exponent buffer eb
  auto issueOps = [&](const SbGeo& g, int eb) {
    const int nt[2] = {g.ni, g.nk};
    const int64_t row0[2] = {(int64_t)g.I0 * kTile, (int64_t)g.K0 * kTile};
    uint32_t bytes = 0;
    for (int o = 0; o < 2; ++o) bytes += (uint32_t)nt[o] * (kPlanes * 512 + 128);
    tc::mbarArriveExpectTx(mbarLd, bytes);
    for (int o = 0; o < 2; ++o) {
      for (int sl = 0; sl < kDfSlices; ++sl)
        for (int kg = 0; kg < kDfK / 8; ++kg)
          tc::bulkLoad(opAddr + (uint32_t)(o * kDfSlices + sl) * kDfPanelBytes + (uint32_t)kg * 2048u,
                       slices + ((int64_t)(o * kDfSlices + sl) * (kDfK / 8) + kg) * rows * 16 + row0[o] * 16,
                       (uint32_t)nt[o] * 512u, mbarLd);
      tc::bulkLoad(expAddr[eb] + (uint32_t)o * tc::kRows * 4, slices + 1536 * rows + (o * rows + row0[o]) * 4,
                   (uint32_t)nt[o] * 128u, mbarLd);
    }
  };
  // thread 0: super-block g's C tiles (tile t = 4 a + b at t x 8448 bytes) into the operand buffer
  auto issueC = [&](const SbGeo& g) {
    uint32_t bytes = 0;
    for (int t = 0; t < 16; ++t)
      if (sbTile(g, t)) bytes += kTileBytesDf;
    tc::mbarArriveExpectTx(mbarC, bytes);
    for (int t = 0; t < 16; ++t)
      if (sbTile(g, t))
        tc::bulkLoad(opAddr + (uint32_t)t * kTileBytesDf, M + tileBase(Tn, g.I0 + (t >> 2), g.K0 + (t & 3)),
                     kTileBytesDf, mbarC);
  };
  if (tid == 0) {
    tc::fenceProxyAsyncGlobal();  // the slices and C written this step (generic stores) before the copies
    issueOps(sbGeo(first, J, Tn), 0);
  }
  int eb = 0;
  for (long long sb = first; sb < nsb; sb += stride, eb ^= 1) {
    const SbGeo g = sbGeo(sb, J, Tn);
    const bool okLd = tc::mbarWait(mbarLd, phLd, kTcWaitNs);
    phLd ^= 1u;
    if (!__syncthreads_and(okLd)) {
      tc::mbarWait(mbarLd, phLd ^ 1u, kTcWaitNs);  // the copies in flight, once more
      __syncthreads();
      return false;
    }
    // the slice products into four accumulators, by one thread
    if (tid == 0) {
      tc::fenceAfterSync();
      constexpr uint32_t idesc = tc::idescBf16(tc::kRows, tc::kRows);
      bool used[4] = {false, false, false, false};
      for (int si = 0; si < kDfSlices; ++si)
        for (int sj = 0; si + sj < kDfSlices; ++sj) {
          const int o = min(si + sj, 3);
          const uint32_t d = tmem + (uint32_t)(o * tc::kRows);
          const uint32_t aAddr = opAddr + (uint32_t)si * kDfPanelBytes;
          const uint32_t bAddr = opAddr + (uint32_t)(kDfSlices + sj) * kDfPanelBytes;
          for (int sK = 0; sK < kDfK / 16; ++sK) {
            const uint32_t off = (uint32_t)sK * 4096u;
            tc::mmaBf16(d, tc::smemDesc(aAddr + off), tc::smemDesc(bAddr + off), idesc, used[o] || sK > 0);
          }
          used[o] = true;
        }
      tc::commitTo(mbarMma);
      // the C tiles into the operand buffer once the MMAs have read it
      const bool okM = tc::mbarWait(mbarMma, phMma, kTcWaitNs);
      if (okM) issueC(g);
    }
    const bool ok = tc::mbarWait(mbarMma, phMma, kTcWaitNs);
    phMma ^= 1u;
    const bool okC = ok && tc::mbarWait(mbarC, phC, kTcWaitNs);
    if (ok) phC ^= 1u;
    tc::fenceAfterSync();
    if (!__syncthreads_and(ok && okC)) {
      tc::mbarWait(mbarMma, phMma ^ 1u, kTcWaitNs);  // the MMAs and copies in flight, once more
      if (ok) tc::mbarWait(mbarC, phC ^ 1u, kTcWaitNs);
      __syncthreads();
      return false;
    }
    // C -= scaled sum of the accumulators, in shared memory: warp w owns TMEM lanes 32 (w % 4) ..
    // +31 (its rows) and columns 64 (w / 4) .. +63, eight at a time
    {
      const int warp = tid >> 5, lane = tid & 31;
      const int q = warp & 3, hh = (warp >> 2) & 1;
      const int R = 32 * q + lane;
      const int* expA = reinterpret_cast<const int*>(sm + kDfOpBytes + (uint32_t)eb * kDfExpBytes);
      const int* expB = expA + tc::kRows;
      const int eR = expA[R];
      const uint32_t lanes = (uint32_t)(32 * q) << 16;
#pragma unroll 2
      for (int cb = 0; cb < 8; ++cb) {
        const int c0 = 64 * hh + 8 * cb;
        float d[4][8];
        tc::tmemLoad8x4(tmem + lanes + (uint32_t)c0, (uint32_t)tc::kRows, d);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int Cc = c0 + j;
          float h, e1, h2, e2;
          dfTwoSum(d[0][j], d[1][j], h, e1);
          dfTwoSum(h, d[2][j], h2, e2);
          e1 = __fadd_rn(e1, e2);
          dfTwoSum(h2, d[3][j], h, e2);
          e1 = __fadd_rn(e1, e2);
          float sh, sl;
          dfFastTwoSum(h, e1, sh, sl);
          // x 2^(eR + eB) as two exact power-of-two factors, each within the normal range
          const int ex = eR + expB[Cc];
          const int ex1 = min(max(ex >> 1, -126), 127), ex2 = min(max(ex - (ex >> 1), -126), 127);
          const float f1 = __int_as_float((ex1 + 127) << 23), f2 = __int_as_float((ex2 + 127) << 23);
          const int t = 4 * (R >> 5) + (Cc >> 5);
          if (sbTile(g, t)) {
            df64& cref = Cs[t * kTileElems + (Cc & 31) * kTileLd + (R & 31)];
            cref = cref - df64(__fmul_rn(__fmul_rn(sh, f1), f2), __fmul_rn(__fmul_rn(sl, f1), f2));
          }
        }
      }
    }
    tc::fenceProxyAsyncShared();  // the updated tiles visible to the bulk stores
    tc::fenceBeforeSync();
    __syncthreads();  // TMEM read, the C tiles updated, this exponent buffer consumed
    if (tid == 0) {
      for (int t = 0; t < 16; ++t)
        if (sbTile(g, t))
          tc::bulkStore(M + tileBase(Tn, g.I0 + (t >> 2), g.K0 + (t & 3)), opAddr + (uint32_t)t * kTileBytesDf,
                        kTileBytesDf);
      tc::bulkCommit();
      tc::bulkWaitRead0();  // the stores have read the buffer: the next slices may land in it
      if (sb + stride < nsb) issueOps(sbGeo(sb + stride, J, Tn), eb ^ 1);
    }
  }
  if (tid == 0) {
    tc::bulkWait0();
    tc::fenceProxyAsyncGlobal();  // the stores before the grid barrier's generic release
  }
  __syncthreads();
  return true;
}

// FP32 trailing update on the tensor cores over a pair of tile columns (J0, J0 + 1): C_IK -=
// L_I,pair D_pair L_K,pair^T with K = 64, as three TF32 products A_hi B_lo + A_lo B_hi + A_hi B_hi
// (each FP32 operand x split as hi = tf32(x), lo = tf32(x - hi)) into one FP32 TMEM accumulator:
// 24 MMAs of 128 x 128 x 8 per super-block, issued by one thread.
//
// Panel area (global, `slices`, within dfSliceBytes): for operand o (0 = A = L, 1 = B = L D), part
// p (0 = hi, 1 = lo) and k-group kg (4 of the 64 columns), the 16 bytes of root row m at
// ((o * 2 + p) * 16 + kg) * rows * 16 + m * 16: each (o, p, kg) plane is the canonical
// shared-memory layout of cxg_tc.cuh for every row, so the 128 rows of a super-block are one
// contiguous copy per plane.
constexpr int kF32Parts = 2;
constexpr int kF32Groups = kDfK / 4;                                     // 16-byte k-groups per row
constexpr uint32_t kF32PanelBytes = (uint32_t)tc::kRows * kDfK * 4;      // 32 KB: 128 x 64 TF32
constexpr uint32_t kF32OpBytes = 2 * kF32Parts * kF32PanelBytes;         // 128 KB of operands
constexpr int64_t kF32StageBytes = (int64_t)kF32OpBytes + 16 * (int64_t)kTileBytes;  // operands + C tiles
static_assert(kF32StageBytes + 128 <= kGridTcStageBytes, "FP32 pair staging exceeds the stage area");
static_assert(2 * kF32Parts * kF32Groups * 16 <= 2 * kDfSlices * (kDfK / 8) * 16, "FP32 panels exceed the slice area");

// Writes the TF32 parts (A and B) of the 32 rows of tile row I over the tile columns J0, J0 + 1;
// one warp, lane rr takes row 32 I + rr. L_I,J0 and L_I,J0+1 must be complete in M.
static __device__ __noinline__ void sliceRowPair(const float* M, int Tn, int I, int J0, unsigned char* slices) {
  __syncwarp();
  const int rr = threadIdx.x & 31;
  const int64_t rows = (int64_t)Tn * kTile, m = (int64_t)I * kTile + rr;
  const float* src[2] = {M + tileBase(Tn, I, J0) + rr, M + tileBase(Tn, I, J0 + 1) + rr};
  const float* dg[2] = {M + tileBase(Tn, J0, J0), M + tileBase(Tn, J0 + 1, J0 + 1)};
  for (int o = 0; o < 2; ++o) {
#pragma unroll 2
    for (int kg = 0; kg < kF32Groups; ++kg) {
      float hi[4], lo[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int k = 4 * kg + t, tt = k >> 5, kk = k & 31;
        float x = src[tt][kk * kTileLd];
        if (o) x = x * dg[tt][kk * kTileLd + kk];
        hi[t] = tc::toTf32(x);
        lo[t] = tc::toTf32(x - hi[t]);
      }
      *reinterpret_cast<float4*>(slices + ((int64_t)(o * kF32Parts) * kF32Groups + kg) * rows * 16 + m * 16) =
          make_float4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<float4*>(slices + ((int64_t)(o * kF32Parts + 1) * kF32Groups + kg) * rows * 16 + m * 16) =
          make_float4(lo[0], lo[1], lo[2], lo[3]);
    }
  }
}

// The FP32 trailing update of column pair (J - 1, J) over the super-blocks this CTA owns (sb =
// blockIdx.x - 1, + gridDim.x - 1, ...). Shared memory `sm` (128-byte aligned, kF32StageBytes)
// holds an operand buffer (the TF32 parts, by bulk copies from the panel area) and a C buffer (the
// super-block's C tiles, by bulk copies from the root). Per super-block: one thread issues the 24
// MMAs; once they have read the operands, the next super-block's operands are issued into that
// buffer; the C tiles are updated from the accumulator and written back by bulk stores; once
// those have read the C buffer, the next super-block's C tiles are issued into it. So the operand
// copies overlap the epilogue and the C copies the next MMAs. `tmem`: this CTA's 128 accumulator
// columns. Returns false when a wait ran out (after waiting once more for what is in flight).
static __device__ __noinline__ bool tcF32PairTrailingStep(float* M, int Tn, int J, long long nsb,
                                                          const unsigned char* slices, unsigned char* sm, uint32_t tmem,
                                                          uint32_t mbarMma, uint32_t mbarLd, uint32_t mbarC,
                                                          uint32_t& phMma, uint32_t& phLd, uint32_t& phC) {
  const int tid = threadIdx.x;
  const long long first = (long long)blockIdx.x - 1, stride = (long long)gridDim.x - 1;
  if (first >= nsb) return true;
  const int64_t rows = (int64_t)Tn * kTile;
  const uint32_t opAddr = tc::smemAddr(sm), cAddr = opAddr + kF32OpBytes;
  float* Cs = reinterpret_cast<float*>(sm + kF32OpBytes);
  // thread 0: the TF32 parts of super-block g's A rows (tiles I0 ..) and B rows (K0 ..)
  auto issueOps = [&](const SbGeo& g) {
    const int nt[2] = {g.ni, g.nk};
    const int64_t row0[2] = {(int64_t)g.I0 * kTile, (int64_t)g.K0 * kTile};
    uint32_t bytes = 0;
    for (int o = 0; o < 2; ++o) bytes += (uint32_t)nt[o] * (uint32_t)(kF32Parts * kF32Groups * 512);
    tc::mbarArriveExpectTx(mbarLd, bytes);
    for (int o = 0; o < 2; ++o)
      for (int p = 0; p < kF32Parts; ++p)
        for (int kg = 0; kg < kF32Groups; ++kg)
          tc::bulkLoad(opAddr + (uint32_t)(o * kF32Parts + p) * kF32PanelBytes + (uint32_t)kg * 2048u,
                       slices + ((int64_t)(o * kF32Parts + p) * kF32Groups + kg) * rows * 16 + row0[o] * 16,
                       (uint32_t)nt[o] * 512u, mbarLd);
  };
  // thread 0: super-block g's C tiles (tile t = 4 a + b at t x kTileBytes) into the C buffer
  auto issueC = [&](const SbGeo& g) {
    uint32_t bytes = 0;
    for (int t = 0; t < 16; ++t)
      if (sbTile(g, t)) bytes += kTileBytes;
    tc::mbarArriveExpectTx(mbarC, bytes);
    for (int t = 0; t < 16; ++t)
      if (sbTile(g, t))
        tc::bulkLoad(cAddr + (uint32_t)t * kTileBytes, M + tileBase(Tn, g.I0 + (t >> 2), g.K0 + (t & 3)), kTileBytes,
                     mbarC);
  };
  if (tid == 0) {
    tc::fenceProxyAsyncGlobal();  // the panels and C written this step (generic stores) before the copies
    const SbGeo g0 = sbGeo(first, J, Tn);
    issueOps(g0);
    issueC(g0);
  }
  for (long long sb = first; sb < nsb; sb += stride) {
    const SbGeo g = sbGeo(sb, J, Tn);
    const bool more = sb + stride < nsb;
    const bool okLd = tc::mbarWait(mbarLd, phLd, kTcWaitNs);
    phLd ^= 1u;
    if (!__syncthreads_and(okLd)) {
      tc::mbarWait(mbarLd, phLd ^ 1u, kTcWaitNs);  // the copies in flight, once more
      tc::mbarWait(mbarC, phC, kTcWaitNs);
      __syncthreads();
      return false;
    }
    if (tid == 0) {
      tc::fenceAfterSync();
      constexpr uint32_t idesc = tc::idescTf32(tc::kRows, tc::kRows);
      const uint32_t aHi = opAddr, aLo = opAddr + kF32PanelBytes, bHi = opAddr + 2 * kF32PanelBytes,
                     bLo = opAddr + 3 * kF32PanelBytes;
      for (int sK = 0; sK < kDfK / 8; ++sK) {
        const uint32_t o = (uint32_t)sK * 4096u;
        tc::mmaTf32(tmem, tc::smemDesc(aLo + o), tc::smemDesc(bHi + o), idesc, sK > 0);
        tc::mmaTf32(tmem, tc::smemDesc(aHi + o), tc::smemDesc(bLo + o), idesc, true);
      }
      for (int sK = 0; sK < kDfK / 8; ++sK) {
        const uint32_t o = (uint32_t)sK * 4096u;
        tc::mmaTf32(tmem, tc::smemDesc(aHi + o), tc::smemDesc(bHi + o), idesc, true);
      }
      tc::commitTo(mbarMma);
      // the next super-block's operands once the MMAs have read this one's
      const bool okM = tc::mbarWait(mbarMma, phMma, kTcWaitNs);
      if (okM && more) issueOps(sbGeo(sb + stride, J, Tn));
    }
    const bool ok = tc::mbarWait(mbarMma, phMma, kTcWaitNs);
    phMma ^= 1u;
    const bool okC = ok && tc::mbarWait(mbarC, phC, kTcWaitNs);
    if (ok) phC ^= 1u;
    tc::fenceAfterSync();
    if (!__syncthreads_and(ok && okC)) {
      tc::mbarWait(mbarMma, phMma ^ 1u, kTcWaitNs);  // the MMAs and copies in flight, once more
      if (ok) tc::mbarWait(mbarC, phC ^ 1u, kTcWaitNs);
      if (ok && more) tc::mbarWait(mbarLd, phLd, kTcWaitNs);
      __syncthreads();
      return false;
    }
    // C -= product, in shared memory: warp w reads TMEM lanes 32 (w % 4) .. +31 (its rows),
    // columns 64 (w / 4) .. +63, sixteen at a time
    {
      const int warp = tid >> 5, lane = tid & 31;
      if (warp < 8) {
        const int q = warp & 3, h = warp >> 2;
        const int R = 32 * q + lane;
        for (int cb = 0; cb < 4; ++cb) {
          float d[16];
          const int c0 = 64 * h + 16 * cb;
          tc::tmemLoad16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, d);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int Cc = c0 + j;
            float& cref = Cs[((R >> 5) * 4 + (Cc >> 5)) * kTileElems + (Cc & 31) * kTileLd + (R & 31)];
            cref = cref - d[j];
          }
        }
      }
    }
    tc::fenceProxyAsyncShared();  // the updated tiles visible to the bulk stores
    tc::fenceBeforeSync();
    __syncthreads();  // TMEM read, the C tiles updated
    if (tid == 0) {
      for (int t = 0; t < 16; ++t)
        if (sbTile(g, t))
          tc::bulkStore(M + tileBase(Tn, g.I0 + (t >> 2), g.K0 + (t & 3)), cAddr + (uint32_t)t * kTileBytes,
                        kTileBytes);
      tc::bulkCommit();
      tc::bulkWaitRead0();  // the stores have read the C buffer: the next C tiles may land in it
      if (more) issueC(sbGeo(sb + stride, J, Tn));
    }
  }
  if (tid == 0) {
    tc::bulkWait0();
    tc::fenceProxyAsyncGlobal();  // the stores before the grid barrier's generic release
  }
  __syncthreads();
  return true;
}

// Whole-GPU FP32 and double-float LDL' over pairs of tile columns (J0, J1 = J0 + 1), three grid
// barriers per pair:
//  (A0) the off-diagonal tiles of column J0, one warp each; CTA 0's warp 0 takes L_J1,J0, then
//       updates the diagonal tile (J1, J1) with it and factors it;
//  (A1) column J1's tiles I > J1, one warp each: the update by column J0 (tile routine),
//       L_I,J1, and the tensor-core operands of the row pair (sliceRowPair: TF32 parts for FP32,
//       BF16 slices for double-float);
//  (B)  the trailing update of both columns at once (tcF32PairTrailingStep / tcDfTrailingStep,
//       CTAs 1..), while CTA 0's warp 0 updates the diagonal tile (J1 + 1, J1 + 1) with both
//       columns and factors it.
// Only CTA 0's warp 0 factors diagonal tiles, so the pivot statistics stay in its shared memory.
template <typename T>
__device__ __noinline__ bool gridLdltPairs(GridCtl* g, int nr, int nx, const DevSettings& st, T* M, PivotStats* ps,
                                           unsigned char* slices, int Tn, int warp, int gw, int GW, bool cta0,
                                           TcState& tcs) {
  if (cta0 && warp == 0) tileFactorDiag<T>(M, 0, nr, nx, st, ps);
  if (!gridSync(g)) return false;
  for (int J0 = 0; J0 + 1 < Tn; J0 += 2) {
    const int J1 = J0 + 1;
    const T* A0 = M + tileBase(Tn, J0, J0);
    T* A1 = M + tileBase(Tn, J1, J1);
    // (A0)
    if (cta0 && warp == 0) {
      T* L10 = M + tileBase(Tn, J1, J0);
      tileOffDiag<T>(L10, A0);
      __syncwarp();
      tileSyrk<T>(A1, L10, L10, A0);
      __syncwarp();
      tileFactorDiag<T>(A1, J1, nr, nx, st, ps);
    } else {
      for (int I = J1 + 1 + (gw - 1); I < Tn; I += GW - 1) tileOffDiag<T>(M + tileBase(Tn, I, J0), A0);
    }
    if (!gridSync(g)) return false;
    // (A1)
    for (int I = J1 + 1 + gw; I < Tn; I += GW) {
      T* C = M + tileBase(Tn, I, J1);
      tileSyrk<T>(C, M + tileBase(Tn, I, J0), M + tileBase(Tn, J1, J0), A0);
      __syncwarp();
      tileOffDiag<T>(C, A1);
      sliceRowPair(M, Tn, I, J0, slices);
    }
    if (!gridSync(g)) return false;
    if (J1 + 1 >= Tn) break;
    // (B)
    const int rem = Tn - J1 - 1;
    const int nb = (rem + 3) >> 2;
    const long long nsb = (long long)nb * (nb + 1) / 2;
    if (cta0) {
      if (warp == 0) {
        T* An = M + tileBase(Tn, J1 + 1, J1 + 1);
        tileSyrk<T>(An, M + tileBase(Tn, J1 + 1, J0), M + tileBase(Tn, J1 + 1, J0), A0);
        __syncwarp();
        tileSyrk<T>(An, M + tileBase(Tn, J1 + 1, J1), M + tileBase(Tn, J1 + 1, J1), A1);
        __syncwarp();
        tileFactorDiag<T>(An, J1 + 1, nr, nx, st, ps);
      }
    } else {
      bool okT;
      if constexpr (sizeof(T) == 4)
        okT = tcF32PairTrailingStep(M, Tn, J1, nsb, slices, tcs.stage, tcs.tmem, tcs.mbar, tcs.mbar + 8u,
                                    tcs.mbar + 16u, tcs.phMma, tcs.phLd0, tcs.phLd1);
      else
        okT = tcDfTrailingStep(M, Tn, J1, nsb, slices, tcs.stage, tcs.tmem, tcs.mbar, tcs.mbar + 8u, tcs.mbar + 16u,
                               tcs.phMma, tcs.phLd0, tcs.phLd1);
      if (!okT) {
        if (threadIdx.x == 0) atomicExch(&g->error, 1);
        return false;
      }
    }
    if (!gridSync(g)) return false;
  }
  return true;
}

// Tiled right-looking LDL' of the root over the whole grid. Per tile column J:
//  (A) the off-diagonal tiles of column J, one warp each; barrier;
//  (B) the trailing update C_IK -= L_IJ D_J L_KJ^T, J < K <= I, in super-blocks of 4x4 tiles, one
//      CTA each (CTAs 1..: FP32 on the tensor cores, tcTrailingStep; FP64 and double-float on the
//      CUDA cores, superSyrk), while warp 0 of CTA 0 updates the tile (J+1, J+1) with the tile
//      routine and factors it (one-column lookahead); barrier.
// In FP64 every root entry receives its updates in increasing J with the same operations and
// rounding as the single-CTA factor, so both give the same bits. Only warp 0 of CTA 0 factors
// diagonal tiles, so the pivot statistics stay in CTA 0's shared memory (ps). `stage` holds
// gridStageBytes. Large FP32 and double-float roots run over column pairs instead (gridLdltPairs).
template <typename T>
__device__ __noinline__ bool gridLdltSteps(GridCtl* g, int nr, int nx, const DevSettings& st, T* M, PivotStats* ps,
                                           T* stage, unsigned char* slices, int Tn, int warp, int gw, int GW, bool cta0,
                                           TcState& tcs);

// Roots of at least this many tile columns factor over column pairs (gridLdltPairs): half the C
// traffic of the trailing update, but a longer serial chain per pair. Below it, one column at a
// time (gridLdltSteps: FP32 on the tensor cores, double-float on the CUDA cores). The thresholds
// are the measured crossovers of the two forms on GB300.
constexpr int kPairMinTilesF32 = 352;  // 11264 rows
constexpr int kPairMinTilesDf = 160;   // 5120 rows
template <typename T>
__device__ __forceinline__ constexpr int pairMinTiles() {
  return (ArithOf<T>::v == 1) ? kPairMinTilesF32 : kPairMinTilesDf;
}

// `slices`: the tensor-core panel area of the FP32 and double-float pair forms (dfSliceBytes(nr),
// 16-byte aligned); unused by FP64.
template <typename T>
__device__ __noinline__ bool gridLdlt(GridCtl* g, int nr, int nx, const DevSettings& st, T* M, PivotStats* ps, T* stage,
                                      unsigned char* slices) {
  const int Tn = rootTiles(nr);
  const int warp = threadIdx.x >> 5, W = blockDim.x >> 5;
  const int gw = (int)blockIdx.x * W + warp, GW = (int)gridDim.x * W;
  const bool cta0 = blockIdx.x == 0;
  // FP32 and double-float: the super-blocks go to the tensor cores; every CTA but 0 holds TMEM
  // (128 columns for FP32, 512 for double-float) and the mbarriers for the length of the job
  constexpr bool kTc = ArithOf<T>::v != 0;
  constexpr uint32_t kCols = (ArithOf<T>::v == 2) ? kDfTmemCols : tc::kTmemCols;
  __shared__ __align__(8) unsigned long long sMbar[3];  // MMA completion, C buffer 0, C buffer 1
  __shared__ uint32_t sTmem;
  TcState tcs{};
  tcs.mbar = tc::smemAddr(&sMbar[0]);
  tcs.stage = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(stage) + 127) & ~static_cast<uintptr_t>(127));
  if (kTc && !cta0) {
    if (warp == 0) tc::tmemAlloc(tc::smemAddr(&sTmem), kCols);
    if (threadIdx.x == 32)
      for (int i = 0; i < 3; ++i) tc::mbarInit(tcs.mbar + 8u * i, 1);
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    tcs.tmem = sTmem;
  }
  bool ok = false;
  if constexpr (kTc) {
    if (Tn >= pairMinTiles<T>()) ok = gridLdltPairs<T>(g, nr, nx, st, M, ps, slices, Tn, warp, gw, GW, cta0, tcs);
  }
  if (!kTc || Tn < pairMinTiles<T>())
    ok = gridLdltSteps<T>(g, nr, nx, st, M, ps, stage, slices, Tn, warp, gw, GW, cta0, tcs);
  if (kTc && !cta0) {
    tc::fenceBeforeSync();
    __syncthreads();
    if (warp == 0) tc::tmemDealloc(tcs.tmem, kCols);
    if (threadIdx.x == 32)
      for (int i = 0; i < 3; ++i) tc::mbarInval(tcs.mbar + 8u * i);
  }
  return ok;
}

template <typename T>
__device__ __noinline__ bool gridLdltSteps(GridCtl* g, int nr, int nx, const DevSettings& st, T* M, PivotStats* ps,
                                           T* stage, unsigned char* slices, int Tn, int warp, int gw, int GW, bool cta0,
                                           TcState& tcs) {
  if (cta0 && warp == 0) tileFactorDiag<T>(M, 0, nr, nx, st, ps);
  if (!gridSync(g)) return false;
  for (int J = 0; J + 1 < Tn; ++J) {
    T* Ajj = M + tileBase(Tn, J, J);
    for (int I = J + 1 + gw; I < Tn; I += GW) tileOffDiag<T>(M + tileBase(Tn, I, J), Ajj);
    if (!gridSync(g)) return false;
    const int rem = Tn - J - 1;
    const int nb = (rem + 3) >> 2;
    const long long nsb = (long long)nb * (nb + 1) / 2;
    // CTA 0's warp 0 updates and factors the next diagonal tile (J+1, J+1), the critical path of
    // the next column; the super-blocks (row order: sb = r (r + 1) / 2 + k, tile rows J+1+4r..,
    // tile columns J+1+4k..) go to CTAs 1.. cyclically, super-block 0 without that tile
    if (cta0) {
      if (warp == 0) {
        T* An = M + tileBase(Tn, J + 1, J + 1);
        const T* Ln = M + tileBase(Tn, J + 1, J);
        tileSyrk<T>(An, Ln, Ln, Ajj);
        tileFactorDiag<T>(An, J + 1, nr, nx, st, ps);
      }
      if (!gridSync(g)) return false;
      continue;
    }
    if constexpr (sizeof(T) == 4) {
      if (!tcTrailingStep(M, Tn, J, nsb, tcs.stage, tcs.tmem, tcs.mbar, tcs.mbar + 8u, tcs.mbar + 16u, tcs.phMma,
                          tcs.phLd0, tcs.phLd1)) {
        if (threadIdx.x == 0) atomicExch(&g->error, 1);
        return false;
      }
    } else {
      for (long long sb = (long long)blockIdx.x - 1; sb < nsb; sb += (long long)gridDim.x - 1) {
        const SbGeo gg = sbGeo(sb, J, Tn);
        __syncthreads();  // the previous super-block is done with the staging area
        superSyrk<T>(M, Tn, J, gg.I0, gg.K0, gg.ni, gg.nk, gg.diag, gg.skip00, stage);
      }
    }
    if (!gridSync(g)) return false;
  }
  return true;
}

// y_J <- Linv_JJ y_J (unit-lower inverse kept transposed in the diagonal tile), by one CTA:
// 32 rows, each a dot product split over 4 lanes.
template <typename T>
__device__ void ctaDiagForward(const T* Ajj, T* yJ) {
  constexpr int sd = 4, w = 32 / sd;
  T tot = (T)0;
  int i = 0, p = 0;
  if ((int)threadIdx.x < 32 * sd) {
    i = threadIdx.x / sd;
    p = threadIdx.x % sd;
    T acc = (T)0;
    for (int col = p * w; col < (p + 1) * w && col < i; ++col) acc = accT(acc, Ajj[i * kTileLd + col], yJ[col]);
    tot = groupSum(accEnd(acc), sd);
  }
  __syncthreads();
  if ((int)threadIdx.x < 32 * sd && p == 0) yJ[i] = yJ[i] + tot;
  __syncthreads();
}

// x_J <- Linv_JJ^T y_J, by one CTA.
template <typename T>
__device__ void ctaDiagBackward(const T* Ajj, T* yJ) {
  constexpr int sd = 4, w = 32 / sd;
  T tot = (T)0;
  int i = 0, p = 0;
  if ((int)threadIdx.x < 32 * sd) {
    i = threadIdx.x / sd;
    p = threadIdx.x % sd;
    T acc = (T)0;
    for (int row = p * w; row < (p + 1) * w; ++row)
      if (row > i) acc = accT(acc, Ajj[row * kTileLd + i], yJ[row]);
    tot = groupSum(accEnd(acc), sd);
  }
  __syncthreads();
  if ((int)threadIdx.x < 32 * sd && p == 0) yJ[i] = yJ[i] + tot;
  __syncthreads();
}

// y_I -= L_IJ y_J for one off-diagonal tile, one warp (lane = row of the tile).
template <typename T>
__device__ __forceinline__ void warpRowsForward(const T* Lij, const T* yJ, T* yI) {
  const int lane = threadIdx.x & 31;
  const T yv = yJ[lane];
  T acc = (T)0;
#pragma unroll 8
  for (int col = 0; col < 32; ++col) acc = accT(acc, Lij[col * kTileLd + lane], shflT(yv, col));
  yI[lane] = yI[lane] - accEnd(acc);
}

// y_K -= L_JK^T x_J for one off-diagonal tile, one warp (lane = column of the tile).
template <typename T>
__device__ __forceinline__ void warpRowsBackward(const T* Ljk, const T* xJ, T* yK) {
  const int lane = threadIdx.x & 31;
  const T xv = xJ[lane];
  T acc = (T)0;
#pragma unroll 8
  for (int r2 = 0; r2 < 32; ++r2) acc = accT(acc, Ljk[lane * kTileLd + r2], shflT(xv, r2));
  yK[lane] = yK[lane] - accEnd(acc);
}

// y <- M^-1 y over the grid, in blocks of kSolveBlk tiles (one barrier per block step).
// Forward step B: warps 0..3 of CTA 0 update the tiles of block B+1 from block B, warp 4 scales
// block B-1 (finished) by D, then CTA 0 solves block B+1 within itself (ctaBlockForward, CTA
// barriers only); meanwhile the warps of the other CTAs update
// every tile of blocks B+2.. from block B, one tile each. The backward pass mirrors it. Each
// y tile receives its updates one source tile at a time, in increasing (forward) / decreasing
// (backward) source order. Needs at least two CTAs.
constexpr int kSolveBlk = 4;

// Solve of one block of tiles b0 .. b1-1 within itself by the calling CTA: per tile j, the
// diagonal block (ctaDiag*) then the updates of the block's other tiles from tile j, one warp
// each, with CTA barriers only.
template <typename T>
__device__ void ctaBlockForward(const T* M, int Tn, int b0, int b1, T* y) {
  const int warp = threadIdx.x >> 5;
  for (int j = b0; j < b1; ++j) {
    ctaDiagForward<T>(M + tileBase(Tn, j, j), y + j * 32);
    const int i = j + 1 + warp;
    if (i < b1) warpRowsForward<T>(M + tileBase(Tn, i, j), y + j * 32, y + i * 32);
    __syncthreads();
  }
}

template <typename T>
__device__ void ctaBlockBackward(const T* M, int Tn, int b0, int b1, T* y) {
  const int warp = threadIdx.x >> 5;
  for (int j = b1 - 1; j >= b0; --j) {
    ctaDiagBackward<T>(M + tileBase(Tn, j, j), y + j * 32);
    const int k = j - 1 - warp;
    if (k >= b0) warpRowsBackward<T>(M + tileBase(Tn, j, k), y + j * 32, y + k * 32);
    __syncthreads();
  }
}

// L2 prefetch of tile rows [I0, I1) of tile column j (contiguous in the packed layout), spread
// over nt threads: one prefetch per 128-byte line.
template <typename T>
__device__ __forceinline__ void prefetchTileRun(const T* M, int Tn, int I0, int I1, int j, int t, int nt) {
  if (I0 >= I1) return;
  const char* p = reinterpret_cast<const char*>(M + tileBase(Tn, I0, j));
  const int64_t bytes = (int64_t)(I1 - I0) * kTileElems * (int64_t)sizeof(T);
  for (int64_t o = (int64_t)t * 128; o < bytes; o += (int64_t)nt * 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + o));
}

template <typename T>
__device__ __noinline__ bool gridSolve(GridCtl* g, int nr, const T* M, T* y) {
  const int Tn = rootTiles(nr);
  const int NB = (Tn + kSolveBlk - 1) / kSolveBlk;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, W = blockDim.x >> 5;
  const bool drv = blockIdx.x == 0;
  const int ww = ((int)blockIdx.x - 1) * W + warp, WW = ((int)gridDim.x - 1) * W;
  auto blo = [&](int B) { return B * kSolveBlk; };
  auto bhi = [&](int B) { return min(Tn, (B + 1) * kSolveBlk); };
  auto scaleBlock = [&](int B) {  // one warp
    for (int j = blo(B); j < bhi(B); ++j) y[j * 32 + lane] /= M[tileBase(Tn, j, j) + lane * kTileLd + lane];
  };
  // CTA 0's step reads its tiles one dependent round after another; the last CTA, whose warps
  // have no far tiles to update at this size, prefetches them into L2 one step ahead.
  const bool pf = (int)blockIdx.x == (int)gridDim.x - 1 && !drv;
  auto prefetchFwd = [&](int B) {  // the tiles of forward step B: block B+1 from block B, block B+1 itself
    if (B + 1 >= NB) return;
    for (int j = blo(B); j < bhi(B); ++j) prefetchTileRun<T>(M, Tn, blo(B + 1), bhi(B + 1), j, threadIdx.x, blockDim.x);
    for (int j = blo(B + 1); j < bhi(B + 1); ++j) prefetchTileRun<T>(M, Tn, j, bhi(B + 1), j, threadIdx.x, blockDim.x);
  };
  auto prefetchBwd = [&](int B) {  // the tiles of backward step B: block B-1 from block B, block B-1 itself
    if (B < 1) return;
    for (int k = blo(B - 1); k < bhi(B - 1); ++k) {
      prefetchTileRun<T>(M, Tn, blo(B), bhi(B), k, threadIdx.x, blockDim.x);
      prefetchTileRun<T>(M, Tn, k, bhi(B - 1), k, threadIdx.x, blockDim.x);
    }
  };
  // forward
  if (drv) ctaBlockForward<T>(M, Tn, blo(0), bhi(0), y);
  if (pf) prefetchFwd(0);
  if (!gridSync(g)) return false;
  for (int B = 0; B + 1 < NB; ++B) {
    if (drv) {
      const int I = blo(B + 1) + warp;
      if (warp < kSolveBlk && I < bhi(B + 1)) {
        for (int j = blo(B); j < bhi(B); ++j) {
          warpRowsForward<T>(M + tileBase(Tn, I, j), y + j * 32, y + I * 32);
          __syncwarp();
        }
      } else if (warp == kSolveBlk && B >= 1) {
        scaleBlock(B - 1);
      }
      __syncthreads();
      ctaBlockForward<T>(M, Tn, blo(B + 1), bhi(B + 1), y);
    } else {
      if (pf) prefetchFwd(B + 1);
      for (int I = blo(B + 2) + ww; I < Tn; I += WW) {
        for (int j = blo(B); j < bhi(B); ++j) {
          warpRowsForward<T>(M + tileBase(Tn, I, j), y + j * 32, y + I * 32);
          __syncwarp();
        }
      }
    }
    if (!gridSync(g)) return false;
  }
  // backward
  if (drv) {
    // blocks NB-2 and NB-1 are not scaled yet (the forward steps scale blocks up to NB-3)
    if (warp < 2 && NB - 1 - warp >= 0) scaleBlock(NB - 1 - warp);
    __syncthreads();
    ctaBlockBackward<T>(M, Tn, blo(NB - 1), bhi(NB - 1), y);
  }
  if (pf) prefetchBwd(NB - 1);
  if (!gridSync(g)) return false;
  for (int B = NB - 1; B >= 1; --B) {
    if (drv) {
      const int K = blo(B - 1) + warp;
      if (warp < kSolveBlk && K < bhi(B - 1)) {
        for (int j = bhi(B) - 1; j >= blo(B); --j) {
          warpRowsBackward<T>(M + tileBase(Tn, j, K), y + j * 32, y + K * 32);
          __syncwarp();
        }
      }
      __syncthreads();
      ctaBlockBackward<T>(M, Tn, blo(B - 1), bhi(B - 1), y);
    } else {
      if (pf) prefetchBwd(B - 1);
      for (int K = blo(B - 1) - 1 - ww; K >= 0; K -= WW) {
        for (int j = bhi(B) - 1; j >= blo(B); --j) {
          warpRowsBackward<T>(M + tileBase(Tn, j, K), y + j * 32, y + K * 32);
          __syncwarp();
        }
      }
    }
    if (!gridSync(g)) return false;
  }
  return true;
}

// One posted job, run by every CTA (CTA 0 passes its pivot statistics).
template <typename T>
__device__ bool gridJobT(GridCtl* g, const DevSettings& st, int op, PivotStats* ps) {
  volatile GridCtl* vg = g;
  T* M = reinterpret_cast<T*>(vg->M);
  const Ctx& c = g->ctx;
  extern __shared__ __align__(16) unsigned char dynSmem[];
  T* stage = reinterpret_cast<T*>(dynSmem + vg->stageOff);
  if (op == kGridOpFactor)
    return gridAssemble<T>(g, c, st, M, vg->ep, vg->ea) && gridLdlt<T>(g, c.nr, c.n, st, M, ps, stage, c.slices);
  if (op == kGridOpSolve) return gridSolve<T>(g, c.nr, M, reinterpret_cast<T*>(vg->y));
  return false;
}

// CTAs 1 .. of a whole-GPU launch: wait for a job, run it, until CTA 0 posts the exit.
template <typename FT>
__device__ __noinline__ void gridWorker(GridCtl* g, const DevSettings& st) {
  for (;;) {
    if (!gridSync(g)) return;
    volatile GridCtl* vg = g;
    const int op = vg->op, arith = vg->arith;
    if (op == kGridOpExit) return;
    bool ok;
    if constexpr (sizeof(FT) == 4)
      ok = (arith == 1) ? gridJobT<float>(g, st, op, nullptr) : gridJobT<df64>(g, st, op, nullptr);
    else
      ok = gridJobT<double>(g, st, op, nullptr);
    if (!ok) return;
  }
}

// CTA 0: post a job (the barrier publishes it) and run it with the other CTAs.
template <typename T>
__device__ bool gridPost(Ctx& c, const DevSettings& st, int op, T* M, T* y, double ep, double ea, PivotStats* ps) {
  GridCtl* g = c.grid;
  if (threadIdx.x == 0) {
    g->op = op;
    g->arith = ArithOf<T>::v;
    g->M = M;
    g->y = y;
    g->ep = ep;
    g->ea = ea;
  }
  if (!gridSync(g)) return false;
  return gridJobT<T>(g, st, op, ps);
}

// ------------------------------------------------------------------------------------------
// reduced KKT: assembly + factorisation, and one solve through it
// ------------------------------------------------------------------------------------------
// Builds the root for the current cone scaling with extra diagonal bumps (ep on x rows, -ea on
// all cone rows, the regularisation ladder of kkt_system.cpp:152-168) and factors it in T.
template <typename T, bool G = false>
__device__ __noinline__ void assembleFactor(Ctx& c, const DevSettings& st, T* M, double ep, double ea,
                               int& fail, int& wrongSign, double& minAbsD) {
  const InstanceDesc& D = *c.D;
  const int n = c.n, nr = c.nr;
  const double epsA = st.static_reg_A + ea;
  const long long t0 = (st.record_timings && threadIdx.x == 0) ? clock64() : 0;
  // G_u = (Hs_u + epsA I)^-1 as eigenvalues (NN: cu[row]; SOC: sp.r0..r2), then
  // T_u = G_u Ad_u column by column
  FOR_T(u, c.nUnits) {
    const int a0 = c.unitAd[u], a1 = c.unitAd[u + 1];
    if (u < c.l) {
      const double w = c.cw[c.p + u];
      const double g = 1.0 / (w * w + epsA);
      c.cu[c.p + u] = g;
      for (int k = a0; k < a1; ++k) c.T[k] = g * c.Ad[k];
    } else {
      const int b = u - c.l;
      const int off = c.socOff[b], d = c.socDim[b];
      socPrepareG(c.sp[b], epsA);
      for (int k = a0; k < a1; k += d) socApplyG(c.sp[b], c.cu + off, d, c.Ad + k, c.T + k);
    }
  }
  if constexpr (G) {
    // whole-GPU launch: the assembly and the LDL' run on every CTA
    PivotStats* ps = reinterpret_cast<PivotStats*>(c.sc + SC_COUNT);
    if (threadIdx.x == 0) {
      ps->nreg = 0;
      ps->zero = 0;
      ps->wrong = 0;
      ps->minAbs = INFINITY;
    }
    __syncthreads();
    const long long t1 = (st.record_timings && threadIdx.x == 0) ? clock64() : 0;
    // post the job, then run its two parts here (timed separately: assembly, LDL')
    GridCtl* g = c.grid;
    if (threadIdx.x == 0) {
      g->op = kGridOpFactor;
      g->arith = ArithOf<T>::v;
      g->M = M;
      g->y = nullptr;
      g->ep = ep;
      g->ea = ea;
    }
    extern __shared__ __align__(16) unsigned char dynSmem[];
    bool ok = gridSync(g) && gridAssemble<T>(g, g->ctx, st, M, ep, ea);
    const long long t2 = (st.record_timings && threadIdx.x == 0) ? clock64() : 0;
    ok = ok && gridLdlt<T>(g, nr, n, st, M, ps, reinterpret_cast<T*>(dynSmem + g->stageOff), c.slices);
    __syncthreads();
    const bool regularized = st.linear_solver == 2;
    fail = !ok ? 1 : (regularized ? (((double)ps->nreg > 0.05 * (double)nr) ? 1 : 0) : ps->zero);
    wrongSign = ps->wrong;
    minAbsD = ok ? ps->minAbs : NAN;
    __syncthreads();
    if (st.record_timings && threadIdx.x == 0) {
      timers(c)[TM_ASSEMBLE] += (t1 - t0) + (t2 - t1);
      timers(c)[TM_LDLT] += clock64() - t2;
    }
    return;
  }
  const int64_t rs = rootSize(nr);
  for (int64_t t = threadIdx.x; t < rs; t += blockDim.x) M[t] = (T)0;
  __syncthreads();
  for (int i = nr + (int)threadIdx.x; i < rootTiles(nr) * kTile; i += blockDim.x) M[rootIdx(nr, i, i)] = (T)1;
  FOR_T(i, n) {
    const int src = c.pdiag[i];
    M[rootIdx(nr, i, i)] = (T)(((src >= 0) ? c.Pu[src] : 0.0) + st.static_reg_P + ep);
  }
  FOR_T(k, D.nPlow) M[c.plowIdx[k]] = (T)c.Pu[c.plowSrc[k]];
  FOR_T(k, D.nAZ) M[c.azIdx[k]] = (T)c.Av[c.azSrc[k]];
  FOR_T(r, c.p) M[rootIdx(nr, n + r, n + r)] = (T)(-(st.static_reg_A + ea));
  __syncthreads();
  FOR_T(t, D.nTgt) {
    double acc = 0.0;
    for (int q = c.tgtBeg[t]; q < c.tgtBeg[t + 1]; ++q) {
      const int oi = c.contrib[3 * q], oj = c.contrib[3 * q + 1], d = c.contrib[3 * q + 2];
      for (int r = 0; r < d; ++r) acc += c.Ad[oi + r] * c.T[oj + r];
    }
    M[c.tgtIdx[t]] += (T)acc;
  }
  __syncthreads();
  const long long t1 = (st.record_timings && threadIdx.x == 0) ? clock64() : 0;
  denseLdlt<T>(c, M, st, fail, wrongSign, minAbsD);
  if (st.record_timings && threadIdx.x == 0) {
    timers(c)[TM_ASSEMBLE] += t1 - t0;
    timers(c)[TM_LDLT] += clock64() - t1;
  }
}

// sol = Kreg^-1 rhs through the factored root (T) with the bump ea used at factorisation.
template <typename T, bool G = false>
__device__ __noinline__ void reducedSolve(Ctx& c, const DevSettings& st, const T* M, double ea,
                             const double* rhs, double* sol) {
  const int n = c.n, m = c.m, p = c.p, nr = c.nr;
  const double epsA = st.static_reg_A + ea;
  const double* r1 = rhs;
  const double* r2 = rhs + n;
  // u = G_C r2_C (eigenvalues of G prepared at factorisation time)
  coneApplyG(c, r2, c.tm);
  // t = [r1 + A_C' u ; r2_Z] in T precision
  T* y = reinterpret_cast<T*>(c.rr);
  FOR_T(j, n) {
    double acc = r1[j];
    for (int k = c.ap[j]; k < c.ap[j + 1]; ++k) {
      const int r = c.ai[k];
      if (r >= p) acc += c.Av[k] * c.tm[r];
    }
    y[j] = (T)acc;
  }
  FOR_T(r, p) y[n + r] = (T)r2[r];
  for (int i = nr + (int)threadIdx.x; i < rootTiles(nr) * kTile; i += blockDim.x) y[i] = (T)0;
  __syncthreads();
  const long long t0 = (st.record_timings && threadIdx.x == 0) ? clock64() : 0;
  if constexpr (G) {
    // whole-GPU launch; a failed barrier leaves a non-finite solution, which the caller's
    // finiteness test turns into NumericalError
    if (!gridPost<T>(c, st, kGridOpSolve, const_cast<T*>(M), y, 0.0, 0.0, nullptr) && threadIdx.x == 0)
      y[0] = (T)NAN;
    __syncthreads();
  } else {
    denseSolve<T>(c, M, y);
  }
  if (st.record_timings && threadIdx.x == 0) timers(c)[TM_DSOLVE] += clock64() - t0;
  FOR_T(j, n) sol[j] = (double)y[j];
  FOR_T(r, p) sol[n + r] = (double)y[n + r];
  __syncthreads();
  // z_C = G_C (A_C x - r2_C)
  FOR_T(r, m) {
    if (r >= p) {
      double acc = -r2[r];
      for (int k = c.arRow[r]; k < c.arRow[r + 1]; ++k) acc += c.Av[c.arSrc[k]] * sol[c.arCol[k]];
      c.tm[r] = acc;
    }
  }
  __syncthreads();
  FOR_T(t, c.l + c.nsoc) {
    if (t < c.l) {
      const int r = p + t;
      sol[n + r] = c.tm[r] * c.cu[r];
    } else {
      const int b = t - c.l;
      const int off = c.socOff[b], d = c.socDim[b];
      socApplyG(c.sp[b], c.cu + off, d, c.tm + off, sol + n + off);
    }
  }
  __syncthreads();
  (void)nr;
  (void)epsA;
}

// Factorisation state of the current iteration.
struct FactState {
  int use64;      // the high-precision factor (in root64) is the one held
  double ep, ea;  // bumps of the held factor
};

template <typename FT>
__device__ __forceinline__ FT* rootT(Ctx& c) { return reinterpret_cast<FT*>(c.root); }

// Arithmetic of the high-precision factor held in root64: FP64 for the FP64 kernel, double-float
// (FP32 pipe, ~48 bits) as the fallback of the mixed-precision kernel.
template <typename FT> struct HighT { using type = double; };
template <> struct HighT<float> { using type = df64; };
template <typename FT>
__device__ __forceinline__ typename HighT<FT>::type* rootHigh(Ctx& c) {
  return reinterpret_cast<typename HighT<FT>::type*>(c.root64);
}

// factorizeWithRetry (kkt_system.cpp:242-264) on the reduced system. In MIXED precision an FP32
// factor with a wrong-signed pivot is replaced by the double-float factor (sticky).
template <typename FT, bool G = false>
__device__ __noinline__ bool factorizeWithRetryImpl(Ctx& c, const DevSettings& st, FactState& fs) {
  double ep = 0.0, ea = 0.0;
  // attempts below this level fail in the reference's dense SOC blocks (coneUpdateScaling)
  const int socLvl = (int)c.sc[SC_SOCLVL];
  for (int attempt = 0; attempt < 18; ++attempt) {
    int fail = 0, wrong = 0;
    double mind = 0.0;
    // fault injection (tests): this attempt reports failure before any work, as does an attempt
    // the reference's SOC-block pivots fail
    const bool injected = c.sc[SC_FAULTF] < (double)st.fault_factor_failures;
    __syncthreads();
    if (injected || attempt < socLvl) {
      if (threadIdx.x == 0) {
        c.sc[SC_ATTEMPTS] += 1.0;
        if (injected) c.sc[SC_FAULTF] += 1.0;
      }
      __syncthreads();
      ep = fmax(ep * 10.0, st.dynamic_reg_delta);
      ea = fmax(ea * 10.0, st.dynamic_reg_delta);
      continue;
    }
    if (!fs.use64) {
      assembleFactor<FT, G>(c, st, rootT<FT>(c), ep, ea, fail, wrong, mind);
      if (sizeof(FT) == 4 && (wrong || !isfinite(mind))) {
        fs.use64 = 1;
        if (threadIdx.x == 0) c.sc[SC_NFB] += 1.0;
        attempt -= 1;  // retry this attempt in FP64
        continue;
      }
    } else {
      assembleFactor<typename HighT<FT>::type, G>(c, st, rootHigh<FT>(c), ep, ea, fail, wrong, mind);
    }
    if (threadIdx.x == 0) c.sc[SC_ATTEMPTS] += 1.0;
    __syncthreads();
    if (!fail && isfinite(mind) && mind > st.dynamic_reg_eps) {
      fs.ep = ep;
      fs.ea = ea;
      return true;
    }
    ep = fmax(ep * 10.0, st.dynamic_reg_delta);
    ea = fmax(ea * 10.0, st.dynamic_reg_delta);
  }
  return false;
}

template <typename FT, bool G>
__device__ void solveOnce(Ctx& c, const DevSettings& st, const FactState& fs, const double* rhs, double* sol) {
  if (fs.use64)
    reducedSolve<typename HighT<FT>::type, G>(c, st, rootHigh<FT>(c), fs.ea, rhs, sol);
  else
    reducedSolve<FT, G>(c, st, rootT<FT>(c), fs.ea, rhs, sol);
  // fault injection (tests): this solve returns a non-finite vector
  if (st.fault_nonfinite_solves > 0) {
    const bool injected = c.sc[SC_FAULTS] < (double)st.fault_nonfinite_solves;
    __syncthreads();
    if (injected && threadIdx.x == 0) {
      c.sc[SC_FAULTS] += 1.0;
      sol[0] = NAN;
    }
    __syncthreads();
  }
}

static __device__ __noinline__ bool vecFinite(Ctx& c, const double* v, int len) {
  int bad = 0;
  FOR_T(i, len) bad |= !finiteBits(v[i]);
  return blockOrInt(bad, c.redi) == 0;
}

// Refinement of the whole-GPU form: restarted GMRES in FP64 on the statically regularised K
// (the matrix the reference refines against, kkt_system.cpp:296-311), right-preconditioned by
// the held factor (FP32, double-float or FP64 LDL' of the bumped reduced system). Where a
// large root is ill-conditioned enough that plain refinement x += K^-1 (rhs - K x) with that
// factor stalls or diverges (the factor's relative error times cond(K) near or above 1), GMRES
// still converges, in a few iterations per cluster of poorly resolved eigenvalues (the mixed
// precision GMRES-IR of Carson and Higham, SIAM J. Sci. Comput. 40(2), 2018). Each iteration is one
// solve with the factor (every SM), one K product and modified Gram-Schmidt (CTA 0). On entry
// sol is the first solve and c.res = rhs - K sol with relative norm rel; a cycle's correction is
// kept only if the true residual drops. Returns the final relative residual; counts iterations
// in SC_RSTEPS.
template <typename FT, bool G>
__device__ void solveOnce(Ctx& c, const DevSettings& st, const FactState& fs, const double* rhs, double* sol);

template <typename FT, bool G>
__device__ __noinline__ double gmresRefine(Ctx& c, const DevSettings& st, const FactState& fs, const double* rhs,
                                           double* sol, double rel, double rhsNorm) {
  const int N = c.n + c.m;
  const int64_t ld = ((int64_t)N + 1) & ~int64_t(1);
  constexpr int hl = kGmresDim + 1;  // leading dimension of H (column-major)
  double* V = c.kry;
  double* Z = V + (int64_t)(kGmresDim + 1) * ld;
  double* H = Z + (int64_t)kGmresDim * ld;
  double* cs = H + hl * kGmresDim;
  double* sn = cs + kGmresDim;
  double* g = sn + kGmresDim;
  double* y = g + kGmresDim + 1;
  int total = 0;
  for (int cyc = 0; cyc < kGmresCycles && rel > st.refine_tol; ++cyc) {
    const double beta = rel * rhsNorm;
    FOR_T(i, N) V[i] = c.res[i] / beta;
    if (threadIdx.x == 0) g[0] = beta;
    __syncthreads();
    int k = 0;
    for (int j = 0; j < kGmresDim; ++j) {
      double* vj = V + (int64_t)j * ld;
      double* zj = Z + (int64_t)j * ld;
      solveOnce<FT, G>(c, st, fs, vj, zj);
      double* w = V + (int64_t)(j + 1) * ld;
      kktApply(c, st, zj, w);
      for (int i = 0; i <= j; ++i) {
        const double* vi = V + (int64_t)i * ld;
        double d[1] = {0.0};
        FOR_T(t, N) d[0] += w[t] * vi[t];
        blockSum<1>(d, c.red);
        FOR_T(t, N) w[t] -= d[0] * vi[t];
        if (threadIdx.x == 0) H[j * hl + i] = d[0];
        __syncthreads();
      }
      double nn[1] = {0.0};
      FOR_T(t, N) nn[0] += w[t] * w[t];
      blockSum<1>(nn, c.red);
      const double hn = sqrt(nn[0]);
      if (threadIdx.x == 0) {
        double* h = H + j * hl;
        h[j + 1] = hn;
        for (int i = 0; i < j; ++i) {
          const double t = cs[i] * h[i] + sn[i] * h[i + 1];
          h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
          h[i] = t;
        }
        const double den = hypot(h[j], h[j + 1]);
        const double cj = den > 0.0 ? h[j] / den : 1.0, sj = den > 0.0 ? h[j + 1] / den : 0.0;
        cs[j] = cj;
        sn[j] = sj;
        h[j] = den;
        h[j + 1] = 0.0;
        g[j + 1] = -sj * g[j];
        g[j] = cj * g[j];
        c.sc[SC_GMRES] = fabs(g[j + 1]) / rhsNorm;
      }
      __syncthreads();
      k = j + 1;
      // stop at a residual estimate well below the target (the true residual is checked below),
      // or at breakdown (the Krylov space holds the solution)
      if (!(hn > 0.0) || !(c.sc[SC_GMRES] > 0.25 * st.refine_tol)) break;
      const double inv = 1.0 / hn;
      FOR_T(t, N) w[t] *= inv;
      __syncthreads();
    }
    total += k;
    if (threadIdx.x == 0) {
      for (int i = k - 1; i >= 0; --i) {
        double acc = g[i];
        for (int l = i + 1; l < k; ++l) acc -= H[l * hl + i] * y[l];
        y[i] = acc / H[i * hl + i];
      }
    }
    __syncthreads();
    FOR_T(t, N) {
      double acc = sol[t];
      for (int l = 0; l < k; ++l) acc += y[l] * Z[(int64_t)l * ld + t];
      c.cor[t] = acc;
    }
    __syncthreads();
    double rn = 1.0;
    const double relNew = kktResidual(c, st, rhs, c.cor, c.res, rn);
    if (!(relNew < rel)) break;  // no progress (or a non-finite candidate): keep sol
    FOR_T(t, N) sol[t] = c.cor[t];
    __syncthreads();
    rel = relNew;
  }
  if (threadIdx.x == 0) c.sc[SC_RSTEPS] += total;
  __syncthreads();
  return rel;
}

// KktSystem::solve (kkt_system.cpp:296-311) incl. escalateAndResolve (:266-294), plus the
// MIXED-precision fallback to the double-float factor. Returns the final relative residual.
template <typename FT, bool G = false>
__device__ bool factorizeWithRetry(Ctx& c, const DevSettings& st, FactState& fs);

template <typename FT, bool G = false>
__device__ __noinline__ double kktSolveImpl(Ctx& c, const DevSettings& st, FactState& fs, const double* rhs, double* sol) {
  const int N = c.n + c.m;
  for (int pass = 0; pass < 2; ++pass) {
    solveOnce<FT, G>(c, st, fs, rhs, sol);
    if (!vecFinite(c, sol, N)) {
      // escalate: x1000 bumps from the held factor's, up to 10 times
      double ep = fs.ep, ea = fs.ea;
      bool ok = false;
      const double socEa = ladderBump((int)c.sc[SC_SOCLVL], st.dynamic_reg_delta);
      for (int att = 0; att < 10 && !ok; ++att) {
        ep = fmax(ep * 1000.0, st.dynamic_reg_delta);
        ea = fmax(ea * 1000.0, st.dynamic_reg_delta);
        int fail = 0, wrong = 0;
        double mind = 0.0;
        if (threadIdx.x == 0) c.sc[SC_ESC] += 1.0;
        if (ea < socEa) continue;  // the reference's SOC-block pivots still fail at this bump
        if (fs.use64)
          assembleFactor<typename HighT<FT>::type, G>(c, st, rootHigh<FT>(c), ep, ea, fail, wrong, mind);
        else
          assembleFactor<FT, G>(c, st, rootT<FT>(c), ep, ea, fail, wrong, mind);
        if (fail || !isfinite(mind) || !(mind > st.dynamic_reg_eps)) continue;
        fs.ep = ep;
        fs.ea = ea;
        solveOnce<FT, G>(c, st, fs, rhs, sol);
        ok = vecFinite(c, sol, N);
      }
    }
    double rhsNorm = 1.0;
    double rel = kktResidual(c, st, rhs, sol, c.res, rhsNorm);
    const bool fp32Factor = (sizeof(FT) == 4) && !fs.use64;
    const int maxRef = G ? 0 : (fp32Factor ? st.mixed_refine_max_iter : st.refine_max_iter);
    if constexpr (G) {
      if (rel > st.refine_tol) rel = gmresRefine<FT, G>(c, st, fs, rhs, sol, rel, rhsNorm);
    }
    int steps = 0;
    for (int it = 0; it < maxRef && rel > st.refine_tol; ++it) {
      solveOnce<FT, G>(c, st, fs, c.res, c.cor);
      FOR_T(i, N) sol[i] += c.cor[i];
      __syncthreads();
      const double prev = rel;
      rel = kktResidual(c, st, rhs, sol, c.res, rhsNorm);
      ++steps;
      // an FP32 factor whose refinement contracts by less than 4x per step will not reach the
      // tolerance in the remaining steps: go to the high-precision factor now
      if (fp32Factor && !(rel <= st.mixed_fallback_tol) && !(rel <= 0.25 * prev)) break;
      // a step of the high-precision refinement that does not lower the residual: keep the
      // better solution and stop (further steps with the same factor do not converge either)
      if (!fp32Factor && !(rel < prev)) {
        FOR_T(i, N) sol[i] -= c.cor[i];
        __syncthreads();
        rel = prev;
        break;
      }
    }
    if (threadIdx.x == 0) c.sc[SC_RSTEPS] += steps;
    const bool mixedFp32 = (sizeof(FT) == 4) && !fs.use64;
    if (mixedFp32 && !(rel <= st.mixed_fallback_tol)) {
      // sticky fallback: refactor in double-float (with the retry ladder) and redo this solve
      fs.use64 = 1;
      if (threadIdx.x == 0) c.sc[SC_NFB] += 1.0;
      if (!factorizeWithRetry<FT, G>(c, st, fs)) return INFINITY;
      continue;
    }
    if (threadIdx.x == 0) {
      if (!(rel <= c.sc[SC_MAXREL])) c.sc[SC_MAXREL] = rel;
      if (!(rel <= c.sc[SC_ITREL])) c.sc[SC_ITREL] = rel;
    }
    __syncthreads();
    return rel;
  }
  return INFINITY;
}

template <typename FT, bool G>
__device__ bool factorizeWithRetry(Ctx& c, const DevSettings& st, FactState& fs) {
  const long long t0 = st.record_timings ? clock64() : 0;
  const bool ok = factorizeWithRetryImpl<FT, G>(c, st, fs);
  if (st.record_timings && threadIdx.x == 0) timers(c)[TM_FACTOR] += clock64() - t0;
  return ok;
}

template <typename FT, bool G = false>
__device__ double kktSolve(Ctx& c, const DevSettings& st, FactState& fs, const double* rhs, double* sol) {
  const long long t0 = st.record_timings ? clock64() : 0;
  const long long f0 = st.record_timings ? timers(c)[TM_FACTOR] : 0;
  __syncthreads();
  // a fallback refactorisation inside counts as factorisation time only
  const double r = kktSolveImpl<FT, G>(c, st, fs, rhs, sol);
  if (st.record_timings && threadIdx.x == 0) timers(c)[TM_SOLVE] += (clock64() - t0) - (timers(c)[TM_FACTOR] - f0);
  return r;
}

// ------------------------------------------------------------------------------------------
// the IPM driver for one instance (solver_impl.cpp SolverImpl::solve and helpers)
// ------------------------------------------------------------------------------------------
template <typename FT, bool G = false>
__device__ __noinline__ void solveInstance(Ctx& c, const LaunchArgs& a, int inst) {
  const DevSettings& st = a.st;
  const InstanceDesc& D = *c.D;
  const int n = c.n, m = c.m, N = n + m;
  const int degree = c.l + c.nsoc;
  FactState fs{0, 0.0, 0.0};
  double tau = 1.0, kappa = 1.0;
  int status = 4;  // MaxIterations
  int iterations = 0;
  double dqx = 0, dbz = 0, dsz = 0, dxPx = 0, rtau = 0;
  if (threadIdx.x < SC_COUNT) c.sc[threadIdx.x] = 0.0;
  if (threadIdx.x < TM_COUNT) timers(c)[threadIdx.x] = 0;
  const long long tStart = clock64();
  unsigned long long wallStart = 0;
  if (st.record_timings && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(wallStart));
  __syncthreads();

  const bool useWarm = st.warm_start && a.haveWarm && a.haveWarm[inst];
  bool initOk = true;
  if (useWarm) {
    FOR_T(j, n) c.x[j] = a.warmX[D.vQ + j];
    FOR_T(r, m) {
      c.s[r] = (r < c.p) ? 0.0 : a.warmS[D.vB + r];
      c.z[r] = a.warmZ[D.vB + r];
    }
    __syncthreads();
    ensureStrictlyInteriorWarm(c, c.s);
    ensureStrictlyInteriorWarm(c, c.z);
  } else {
    // computeInitialPoint: Hs = I scaling of the identity element, 1 or 2 KKT solves
    coneUpdateScaling(c, st, c.ev, c.ev);
    if (!factorizeWithRetry<FT, G>(c, st, fs)) {
      initOk = false;
    } else {
      if (D.pStoredNnz == 0) {
        FOR_T(j, n) c.rhs[j] = 0.0;
        FOR_T(r, m) c.rhs[n + r] = c.bs[r];
        __syncthreads();
        kktSolve<FT, G>(c, st, fs, c.rhs, c.sol);
        FOR_T(j, n) c.x[j] = c.sol[j];
        FOR_T(r, m) c.s[r] = -c.sol[n + r];
        FOR_T(j, n) c.rhs[j] = -c.qs[j];
        FOR_T(r, m) c.rhs[n + r] = 0.0;
        __syncthreads();
        kktSolve<FT, G>(c, st, fs, c.rhs, c.sol);
        FOR_T(r, m) c.z[r] = c.sol[n + r];
      } else {
        FOR_T(j, n) c.rhs[j] = -c.qs[j];
        FOR_T(r, m) c.rhs[n + r] = c.bs[r];
        __syncthreads();
        kktSolve<FT, G>(c, st, fs, c.rhs, c.sol);
        FOR_T(j, n) c.x[j] = c.sol[j];
        FOR_T(r, m) {
          c.z[r] = c.sol[n + r];
          c.s[r] = -c.sol[n + r];
        }
      }
      __syncthreads();
      FOR_T(r, c.p) c.s[r] = 0.0;
      __syncthreads();
      shiftToInteriorCold(c, c.s, degree);
      shiftToInteriorCold(c, c.z, degree);
      int bad = 0;
      FOR_T(j, n) bad |= !finiteBits(c.x[j]);
      FOR_T(r, m) bad |= !finiteBits(c.s[r]) | !finiteBits(c.z[r]);
      initOk = blockOrInt(bad, c.redi) == 0;
    }
  }
  if (!initOk) status = 5;

  // record_timings: one trace row per iteration (columns as kTraceCols), written by thread 0
  double* trow = nullptr;
  for (int iter = 0; initOk && iter < st.max_iter; ++iter) {
    iterations = iter + 1;
    trow = (a.trace && iter < a.traceRows) ? a.trace + ((int64_t)inst * a.traceRows + iter) * kTraceCols : nullptr;
    if (threadIdx.x == 0) {
      c.sc[SC_ITREL] = 0.0;
      if (trow)
        for (int k = 0; k < kTraceCols; ++k) trow[k] = 0.0;
    }
    const double att0 = c.sc[SC_ATTEMPTS];
    __syncthreads();
    // 1. refactorise for the current scaling
    coneUpdateScaling(c, st, c.s, c.z);
    if (!factorizeWithRetry<FT, G>(c, st, fs)) { status = 5; break; }
    if (trow && threadIdx.x == 0) trow[11] = c.sc[SC_ATTEMPTS] - att0;
    // 2. constant solve (-q, b) -> x1, z1; Px1
    FOR_T(j, n) c.rhs[j] = -c.qs[j];
    FOR_T(r, m) c.rhs[n + r] = c.bs[r];
    __syncthreads();
    kktSolve<FT, G>(c, st, fs, c.rhs, c.sol);
    FOR_T(j, n) c.x1[j] = c.sol[j];
    FOR_T(r, m) c.z1[r] = c.sol[n + r];
    __syncthreads();
    if (!vecFinite(c, c.sol, N)) { status = 5; break; }
    pmul(c, c.x1, c.Px1);
    // 3. residuals
    pmul(c, c.x, c.tn);  // Px
    {
      double v[6] = {0, 0, 0, 0, 0, 0};
      FOR_T(t, n + m) {
        if (t < n) {
          double atz = 0.0;
          for (int k = c.ap[t]; k < c.ap[t + 1]; ++k) atz += c.Av[k] * c.z[c.ai[k]];
          const double r = -atz - c.tn[t] - tau * c.qs[t];
          c.rx[t] = r;
          v[0] += r * r;
          v[2] += c.qs[t] * c.x[t];
          v[5] += c.x[t] * c.tn[t];
        } else {
          const int r = t - n;
          double ax = 0.0;
          for (int k = c.arRow[r]; k < c.arRow[r + 1]; ++k) ax += c.Av[c.arSrc[k]] * c.x[c.arCol[k]];
          const double rr = ax + c.s[r] - tau * c.bs[r];
          c.rz[r] = rr;
          v[1] += rr * rr;
          v[3] += c.bs[r] * c.z[r];
          v[4] += c.s[r] * c.z[r];
        }
      }
      blockSum<6>(v, c.red);
      dqx = v[2];
      dbz = v[3];
      dsz = v[4];
      dxPx = v[5];
      rtau = dqx + dbz + kappa + dxPx / tau;
      const double mu = (dsz + tau * kappa) / (double)(degree + 1);
      const double nrx = sqrt(v[0]) / tau, nrz = sqrt(v[1]) / tau;
      const double pobj = (0.5 * dxPx / tau + dqx) / tau;
      const double dobj = (-0.5 * dxPx / tau - dbz) / tau;
      // 4. convergence / infeasibility (solver_impl.cpp checkConvergence / checkInfeasibility)
      if (trow && threadIdx.x == 0) {
        trow[0] = mu; trow[1] = nrx; trow[2] = nrz; trow[3] = pobj; trow[4] = dobj; trow[8] = tau; trow[9] = kappa;
      }
      const double gapAbs = fabs(pobj - dobj);
      const double gapTol = st.tol_gap_abs + st.tol_gap_rel * fmax(fabs(pobj), fabs(dobj));
      if (nrx < st.tol_feas && nrz < st.tol_feas && gapAbs < gapTol && tau > 1e-6) { status = 1; break; }
      const double ratio = tau / fmax(kappa, 1e-30);
      if (ratio <= st.tol_infeas) {
        double w[2] = {0.0, 0.0};
        FOR_T(r, m) w[0] += c.z[r] * c.z[r];
        FOR_T(j, n) w[1] += c.x[j] * c.x[j];
        blockSum<2>(w, c.red);
        if (dbz < -st.tol_infeas * fmax(1.0, sqrt(w[0]))) { status = 2; break; }
        if (dqx < -st.tol_infeas * fmax(1.0, sqrt(w[1]))) { status = 3; break; }
      }
      // tau_den is the same for the affine and the combined step (solver_impl.cpp:309-310,
      // 364-365): kappa/tau - q'x1 - b'z1 + (xi-x1)'P(xi-x1) - x1'Px1, xi = x/tau
      FOR_T(j, n) c.tn[j] = c.x[j] / tau - c.x1[j];
      __syncthreads();
      pmul(c, c.tn, c.dx);
      double td[4] = {0, 0, 0, 0};
      FOR_T(j, n) {
        td[0] += c.qs[j] * c.x1[j];
        td[2] += c.tn[j] * c.dx[j];
        td[3] += c.x1[j] * c.Px1[j];
      }
      FOR_T(r, m) td[1] += c.bs[r] * c.z1[r];
      blockSum<4>(td, c.red);
      const double tauDen = kappa / tau - td[0] - td[1] + td[2] - td[3];

      // 5. affine step: rhs (rx, s - rz)
      FOR_T(j, n) c.rhs[j] = c.rx[j];
      FOR_T(r, m) c.rhs[n + r] = c.s[r] - c.rz[r];
      __syncthreads();
      kktSolve<FT, G>(c, st, fs, c.rhs, c.sol);
      if (!vecFinite(c, c.sol, N)) { status = 5; break; }
      pmul(c, c.sol, c.tn);  // P xv
      double tn3[3] = {0, 0, 0};
      FOR_T(j, n) {
        tn3[0] += c.qs[j] * c.sol[j];
        tn3[2] += (c.x[j] / tau) * c.tn[j];
      }
      FOR_T(r, m) tn3[1] += c.bs[r] * c.sol[n + r];
      blockSum<3>(tn3, c.red);
      const double dkrA = tau * kappa;
      const double tauNumA = rtau - dkrA / tau + tn3[0] + tn3[1] + 2.0 * tn3[2];
      if (tauDen == 0.0 || !isfinite(tauNumA) || !isfinite(tauDen)) { status = 5; break; }
      const double dtauA = tauNumA / tauDen;
      FOR_T(j, n) c.dx[j] = c.sol[j] + dtauA * c.x1[j];
      FOR_T(r, m) c.dz[r] = c.sol[n + r] + dtauA * c.z1[r];
      __syncthreads();
      coneApply(c, kHs, 0.0, c.dz, c.tm);
      FOR_T(r, m) c.ds[r] = -(c.tm[r] + c.s[r]);
      __syncthreads();
      const double dkappaA = -(dkrA + kappa * dtauA) / tau;
      {
        int bad = !finiteBits(dtauA) || !finiteBits(dkappaA);
        FOR_T(j, n) bad |= !finiteBits(c.dx[j]);
        FOR_T(r, m) bad |= !finiteBits(c.dz[r]) | !finiteBits(c.ds[r]);
        if (blockOrInt(bad, c.redi)) { status = 5; break; }
      }
      // 6. affine step length (no fraction), mu_aff, sigma
      double aaff = 1.0;
      if (dtauA < 0) aaff = fmin(aaff, -tau / dtauA);
      if (dkappaA < 0) aaff = fmin(aaff, -kappa / dkappaA);
      aaff = coneMaxStep(c, c.z, c.dz, aaff);
      aaff = coneMaxStep(c, c.s, c.ds, aaff);
      double sa[1] = {0.0};
      FOR_T(r, m) sa[0] += (c.s[r] + aaff * c.ds[r]) * (c.z[r] + aaff * c.dz[r]);
      blockSum<1>(sa, c.red);
      const double tauAff = tau + aaff * dtauA, kappaAff = kappa + aaff * dkappaA;
      const double muAff = (sa[0] + tauAff * kappaAff) / (double)(degree + 1);
      double sigma;
      if (mu > 0) {
        const double rt = fmax(muAff / mu, 0.0);
        sigma = fmin(fmax(rt * rt * rt, 0.0), 1.0);
      } else {
        sigma = 1.0;
      }
      if (trow && threadIdx.x == 0) { trow[5] = aaff; trow[6] = sigma; }
      // 7. combined step: lambda = W z; ds_comb = lambda o lambda + (W^-1 ds_aff) o (W dz_aff) - sigma mu e
      coneApply(c, kW, 0.0, c.z, c.lam);
      coneProduct(c, false, c.lam, c.lam, c.tm);           // lambda o lambda
      coneApply(c, kWinv, 0.0, c.ds, c.tm2);               // W^-1 ds_aff
      coneApply(c, kW, 0.0, c.dz, c.dcon);                 // W dz_aff (dcon as temp)
      coneProduct(c, false, c.tm2, c.dcon, c.rhs);         // corrector (rhs as temp, length m)
      FOR_T(r, m) c.tm2[r] = c.tm[r] + c.rhs[r] - sigma * mu * c.ev[r];
      __syncthreads();
      coneProduct(c, true, c.lam, c.tm2, c.tm);            // lambda \ ds_comb
      coneApply(c, kW, 0.0, c.tm, c.dcon);                 // ds_const = W (lambda \ ds_comb)
      FOR_T(j, n) c.rhs[j] = (1.0 - sigma) * c.rx[j];
      FOR_T(r, m) c.rhs[n + r] = c.dcon[r] - (1.0 - sigma) * c.rz[r];
      __syncthreads();
      kktSolve<FT, G>(c, st, fs, c.rhs, c.sol);
      if (!vecFinite(c, c.sol, N)) { status = 5; break; }
      pmul(c, c.sol, c.tn);
      tn3[0] = tn3[1] = tn3[2] = 0.0;
      FOR_T(j, n) {
        tn3[0] += c.qs[j] * c.sol[j];
        tn3[2] += (c.x[j] / tau) * c.tn[j];
      }
      FOR_T(r, m) tn3[1] += c.bs[r] * c.sol[n + r];
      blockSum<3>(tn3, c.red);
      const double dtrC = (1.0 - sigma) * rtau;
      const double dkrC = tau * kappa + dtauA * dkappaA - sigma * mu;
      const double tauNumC = dtrC - dkrC / tau + tn3[0] + tn3[1] + 2.0 * tn3[2];
      if (tauDen == 0.0 || !isfinite(tauNumC)) { status = 5; break; }
      const double dtau = tauNumC / tauDen;
      FOR_T(j, n) c.dx[j] = c.sol[j] + dtau * c.x1[j];
      FOR_T(r, m) c.dz[r] = c.sol[n + r] + dtau * c.z1[r];
      __syncthreads();
      coneApply(c, kHs, 0.0, c.dz, c.tm);
      FOR_T(r, m) c.ds[r] = -(c.tm[r] + c.dcon[r]);
      __syncthreads();
      const double dkappa = -(dkrC + kappa * dtau) / tau;
      {
        int bad = !finiteBits(dtau) || !finiteBits(dkappa);
        FOR_T(j, n) bad |= !finiteBits(c.dx[j]);
        FOR_T(r, m) bad |= !finiteBits(c.dz[r]) | !finiteBits(c.ds[r]);
        if (blockOrInt(bad, c.redi)) { status = 5; break; }
      }
      // 8. step length with the fraction-to-boundary factor
      double alpha = 1.0;
      if (dtau < 0) alpha = fmin(alpha, -tau / dtau);
      if (dkappa < 0) alpha = fmin(alpha, -kappa / dkappa);
      alpha = coneMaxStep(c, c.z, c.dz, alpha);
      alpha = coneMaxStep(c, c.s, c.ds, alpha);
      alpha *= st.max_step_fraction;
      if (trow && threadIdx.x == 0) { trow[7] = alpha; trow[10] = c.sc[SC_ITREL]; }
      if (!isfinite(alpha) || alpha <= 0.0) { status = 5; break; }
      // 9. update and rescale
      FOR_T(j, n) c.x[j] += alpha * c.dx[j];
      FOR_T(r, m) {
        c.s[r] += alpha * c.ds[r];
        c.z[r] += alpha * c.dz[r];
      }
      tau += alpha * dtau;
      kappa += alpha * dkappa;
      __syncthreads();
      const double scl = fmax(tau, kappa);
      if (scl > 1e8 || scl < 1e-8) {
        const double inv = 1.0 / scl;
        FOR_T(j, n) c.x[j] *= inv;
        FOR_T(r, m) {
          c.s[r] *= inv;
          c.z[r] *= inv;
        }
        tau *= inv;
        kappa *= inv;
        __syncthreads();
      }
    }
  }
  if (trow && threadIdx.x == 0) trow[10] = c.sc[SC_ITREL];  // the last row, whichever way it ended

  // finalizeSolution (solver_impl.cpp:342-365 of the reference numbering)
  const bool infeas = (status == 2 || status == 3);
  const double scale = infeas ? 1.0 / fmax(kappa, 1e-30) : 1.0 / fmax(tau, 1e-30);
  const double* dvec = a.dpool + D.dD;
  const double* evec = a.dpool + D.dE;
  const double cs = D.cscale;
  const bool eq = st.equilibrate != 0;
  FOR_T(j, n) a.x[D.vX + j] = c.x[j] * scale * (eq ? dvec[j] : 1.0);
  FOR_T(r, m) {
    a.s[D.vS + r] = eq ? (c.s[r] * scale) / evec[r] : c.s[r] * scale;
    a.z[D.vZ + r] = eq ? (c.z[r] * scale) * evec[r] / cs : c.z[r] * scale;
  }
  if (a.bwd) {
    // final factorisation (as FP64), scaling and normalised iterate for the adjoint
    double* Bs = a.bwd + D.bwdOff;
    const BwdLayout bl = bwdLayout(c.nr, n, m, c.nsoc);
    const int64_t rs = rootSize(c.nr);
    if (sizeof(FT) == 8) {
      const double* R = fs.use64 ? c.root64 : reinterpret_cast<const double*>(c.root);
      for (int64_t t = threadIdx.x; t < rs; t += blockDim.x) Bs[bl.root + t] = R[t];
    } else if (fs.use64) {
      const auto* R = rootHigh<FT>(c);
      for (int64_t t = threadIdx.x; t < rs; t += blockDim.x) Bs[bl.root + t] = (double)R[t];
    } else {
      const FT* R = rootT<FT>(c);
      for (int64_t t = threadIdx.x; t < rs; t += blockDim.x) Bs[bl.root + t] = (double)R[t];
    }
    FOR_T(r, m) {
      Bs[bl.cw + r] = c.cw[r];
      Bs[bl.cu + r] = c.cu[r];
      Bs[bl.zh + r] = c.z[r] / tau;
    }
    FOR_T(k, 8 * c.nsoc) Bs[bl.sp + k] = reinterpret_cast<const double*>(c.sp)[k];
    FOR_T(j, n) Bs[bl.xh + j] = c.x[j] / tau;
    if (threadIdx.x == 0) {
      Bs[bl.sc + 0] = fs.ea;
      Bs[bl.sc + 1] = fs.ep;
      Bs[bl.sc + 2] = (double)status;
      Bs[bl.sc + 3] = tau;
    }
  }
  double nr2[2] = {0.0, 0.0};
  FOR_T(j, n) nr2[0] += c.rx[j] * c.rx[j];
  FOR_T(r, m) nr2[1] += c.rz[r] * c.rz[r];
  blockSum<2>(nr2, c.red);
  if (status == 1 && st.warm_start && a.warmX) {
    FOR_T(j, n) a.warmX[D.vQ + j] = c.x[j];
    FOR_T(r, m) {
      a.warmS[D.vB + r] = c.s[r];
      a.warmZ[D.vB + r] = c.z[r];
    }
    if (threadIdx.x == 0 && a.haveWarm) a.haveWarm[inst] = 1;
  }
  if (threadIdx.x == 0) {
    DevResult R{};
    R.status = status;
    R.iterations = iterations;
    double pobj = (0.5 * dxPx / tau + dqx) / tau;
    double gap = dsz / (tau * tau);
    if (eq) {
      pobj /= cs;
      gap /= cs;
    }
    R.objective = pobj;
    R.duality_gap = gap;
    R.primal_residual = sqrt(nr2[1]) / fmax(tau, 1e-30);
    R.dual_residual = sqrt(nr2[0]) / fmax(tau, 1e-30);
    R.mu = (dsz + tau * kappa) / (double)(degree + 1);
    R.max_relres = c.sc[SC_MAXREL];
    R.fp64_fallbacks = (int)c.sc[SC_NFB];
    R.refine_steps = (int)c.sc[SC_RSTEPS];
    R.factor_attempts = (int)c.sc[SC_ATTEMPTS];
    R.escalations = (int)c.sc[SC_ESC];
    R.error_code = (G && reinterpret_cast<volatile GridCtl*>(c.grid)->error) ? 1 : 0;
    const long long tot = clock64() - tStart;
    R.cycles[0] = tot;
    if (st.record_timings) {
      unsigned long long wallEnd = 0;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(wallEnd));
      R.wall_ns[0] = (long long)wallStart;
      R.wall_ns[1] = (long long)wallEnd;
    }
    R.cycles[1] = timers(c)[TM_FACTOR];
    R.cycles[2] = timers(c)[TM_SOLVE];
    R.cycles[3] = tot - R.cycles[1] - R.cycles[2];
    R.cycles[4] = timers(c)[TM_ASSEMBLE];
    R.cycles[5] = timers(c)[TM_LDLT];
    R.cycles[6] = timers(c)[TM_DSOLVE];
    R.cycles[7] = timers(c)[TM_RESID];
    a.results[inst] = R;
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------------------
// kernel: persistent CTAs over an atomic instance queue
// ------------------------------------------------------------------------------------------
// Points the per-instance context at shared memory, the CTA's scratch and the pools (thread 0).
static __device__ void setupCtx(Ctx& c, const LaunchArgs& a, int inst, unsigned char* smem, double* scratch, int* sRedi) {
  const SmemLayout& L = a.lay;
  const InstanceDesc& D = a.desc[inst];
  c.D = &D;
  c.n = D.n; c.m = D.m; c.p = D.p; c.l = D.l; c.nsoc = D.nsoc; c.nr = D.nr; c.nUnits = D.nUnits;
  const int* I = a.ipool;
  c.psRow = I + D.iPsRow; c.psCol = I + D.iPsCol; c.pdiag = I + D.iPdiag;
  c.plowIdx = reinterpret_cast<const long long*>(I + D.iPlowIdx); c.plowSrc = I + D.iPlowSrc;
  c.ap = I + D.iAp; c.ai = I + D.iAi;
  c.arRow = I + D.iArRow; c.arCol = I + D.iArCol; c.arSrc = I + D.iArSrc;
  c.azIdx = reinterpret_cast<const long long*>(I + D.iAZIdx); c.azSrc = I + D.iAZSrc;
  c.socOff = I + D.iSocOff; c.socDim = I + D.iSocDim;
  c.unitAd = I + D.iUnitAd; c.unitSup = I + D.iUnitSup;
  c.tgtIdx = reinterpret_cast<const long long*>(I + D.iTgtIdx); c.tgtBeg = I + D.iTgtBeg; c.contrib = I + D.iContrib;
  // scratch carve-up for this instance (scaled P in user order, then its CSR-order copy)
  c.Pu = scratch + D.sPv;
  c.Pv = c.Pu + D.nnzPu;
  c.Av = scratch + D.sAv;
  c.Ad = scratch + D.sAd;
  c.T = scratch + D.sT;
  c.qs = scratch + D.sQ;
  c.bs = scratch + D.sB;
  c.root64 = L.root64InSmem ? reinterpret_cast<double*>(smem + L.rootOff) : scratch + D.sRoot64;
  // vectors: shared memory or scratch
  double* vb = L.vecInSmem ? reinterpret_cast<double*>(smem + L.vecOff) : scratch + D.sVec;
  const int nM = L.nMax, mM = L.mMax, NM = L.nMax + L.mMax, rM = rootTiles(L.nrMax) * kTile;
  double* q = vb;
  auto take = [&](int len) { double* r = q; q += (len + 1) & ~1; return r; };
  c.x = take(nM); c.rx = take(nM); c.x1 = take(nM); c.Px1 = take(nM); c.dx = take(nM); c.tn = take(nM);
  c.s = take(mM); c.z = take(mM); c.rz = take(mM); c.dz = take(mM); c.ds = take(mM);
  c.dcon = take(mM); c.lam = take(mM); c.tm = take(mM); c.tm2 = take(mM); c.cw = take(mM); c.cu = take(mM);
  c.rhs = take(NM); c.sol = take(NM); c.res = take(NM); c.cor = take(NM);
  c.rr = take(rM);
  c.sp = reinterpret_cast<SocScale*>(take(8 * L.nsocMax));
  // used once or twice per iteration: always in scratch (vecGlobalDoubles)
  c.ev = scratch + D.sVecG;
  c.z1 = c.ev + ((mM + 1) & ~1);
  c.root = L.rootInSmem ? reinterpret_cast<void*>(smem + L.rootOff) : reinterpret_cast<void*>(c.root64);
  c.red = reinterpret_cast<double*>(smem + L.redOff);
  c.sc = c.red + 128;
  c.kry = scratch + D.sKry;
  c.slices = reinterpret_cast<unsigned char*>(scratch + D.sSlice);
  c.redi = sRedi;
  c.grid = nullptr;
}

// ------------------------------------------------------------------------------------------
// kernel: persistent CTAs over an atomic instance queue
// ------------------------------------------------------------------------------------------
// kMaxThreads / kMinBlocks: the large-root form (up to 256 threads, registers for one CTA per
// SM) and the small-root form (up to 64 threads, at least 8 CTAs per SM: small instances are
// bound by FP64 latency, so more of them resident per SM is more throughput).

template <typename FT, int kMaxThreads, int kMinBlocks>
__global__ void __launch_bounds__(kMaxThreads, kMinBlocks) ipmKernel(LaunchArgs a) {
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
    solveInstance<FT>(c, a, inst);
  }
}

// Whole-GPU form for one large instance (a.grid set): a cooperative launch with one CTA per SM.
// CTA 0 runs the iteration, the other CTAs run the root jobs it posts (see gridSync); the
// vectors, the root and the solve vector are in CTA 0's scratch (global memory) so every CTA can
// reach them. A kernel of its own, so that the batched kernels keep their register allocation.
template <typename FT>
__global__ void __launch_bounds__(256, 1) ipmGridKernel(LaunchArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int sRedi[4];
  __shared__ Ctx c;
  GridCtl* g = a.grid;
  if (blockIdx.x == 0) {
    const int inst = a.order[0];
    if (threadIdx.x == 0) {
      setupCtx(c, a, inst, smem, a.scratch, sRedi);
      c.grid = g;
      g->ctx = c;
      g->stageOff = a.lay.rootOff;  // the root itself is in scratch in this form
    }
    __syncthreads();
    loadInstance(c, a);
    solveInstance<FT, true>(c, a, inst);
    if (threadIdx.x == 0) g->op = kGridOpExit;
    gridSync(g);
  } else {
    gridWorker<FT>(g, a.st);
  }
}

// ------------------------------------------------------------------------------------------
// adjoint (new; no reference counterpart): differentiate the KKT conditions at the solution
// with one extra solve through the saved final factorisation,
//   K [u; v] = [D dL/dx; 0],  dL/dq = -u, dL/db = v, dL/dP = -(u x' + x u'), dL/dA = -(z u' + v x'),
// all in the equilibrated space and mapped back through D, E, c (P^ = c D P D, q^ = c D q,
// A^ = E A D, b^ = E b, x = D x^).
// ------------------------------------------------------------------------------------------
static __device__ __noinline__ void adjointInstance(Ctx& c, const LaunchArgs& a) {
  const InstanceDesc& D = *c.D;
  const double* Bs = a.bwd + D.bwdOff;
  const BwdLayout bl = bwdLayout(c.nr, c.n, c.m, c.nsoc);
  const int n = c.n, m = c.m;
  const int status = (int)Bs[bl.sc + 2];
  if (threadIdx.x < SC_COUNT) c.sc[threadIdx.x] = 0.0;
  FOR_T(r, m) {
    c.cw[r] = Bs[bl.cw + r];
    c.cu[r] = Bs[bl.cu + r];
  }
  FOR_T(k, 8 * c.nsoc) reinterpret_cast<double*>(c.sp)[k] = Bs[bl.sp + k];
  if (a.lay.root64InSmem) {
    const int64_t rs = rootSize(c.nr);
    for (int64_t t = threadIdx.x; t < rs; t += blockDim.x) c.root64[t] = Bs[bl.root + t];
  } else if (threadIdx.x == 0) {
    c.root64 = const_cast<double*>(Bs + bl.root);
  }
  const double* dvec = a.dpool + D.dD;
  const double* evec = a.dpool + D.dE;
  const double cs = D.cscale;
  FOR_T(j, n) c.rhs[j] = dvec[j] * a.gx[D.vX + j];
  FOR_T(r, m) c.rhs[n + r] = 0.0;
  __syncthreads();
  const bool ok = status == 1;
  if (ok) {
    FactState fs{1, Bs[bl.sc + 1], Bs[bl.sc + 0]};
    kktSolve<double>(c, a.st, fs, c.rhs, c.sol);
  }
  const double* u = c.sol;
  const double* v = c.sol + n;
  const double* xh = Bs + bl.xh;
  const double* zh = Bs + bl.zh;
  const int* Pp = a.ipool + D.iPp;
  const int* Pi = a.ipool + D.iPi;
  FOR_T(j, n) {
    a.gq[D.vQ + j] = ok ? -u[j] * (cs * dvec[j]) : 0.0;
    for (int k = Pp[j]; k < Pp[j + 1]; ++k) {
      const int r = Pi[k];
      double g = 0.0;
      if (ok && r == j) g = -u[r] * xh[r];
      else if (ok && r < j) g = -(u[r] * xh[j] + u[j] * xh[r]);
      a.gP[D.vPx + k] = g * (cs * dvec[r] * dvec[j]);
    }
    for (int k = c.ap[j]; k < c.ap[j + 1]; ++k) {
      const int r = c.ai[k];
      a.gA[D.vAx + k] = ok ? -(zh[r] * u[j] + v[r] * xh[j]) * (evec[r] * dvec[j]) : 0.0;
    }
  }
  FOR_T(r, m) a.gb[D.vB + r] = ok ? v[r] * evec[r] : 0.0;
  __syncthreads();
}


// Host launchers of the kernels above, per root arithmetic FT (float: mixed precision, double:
// FP64) and launch form; explicitly instantiated in cxg_ipm_f32.cu, cxg_ipm_f32s.cu,
// cxg_ipm_f64.cu (batched forms) and cxg_ipm_gridf.cu, cxg_ipm_gridd.cu (whole-GPU form).
// Raises (never lowers) a kernel's dynamic shared-memory cap. The cap is one attribute of the
// function, while the size-bucket launches of one kernel form ask for different sizes: setting
// it to each launch's own size left the cap at the last bucket's, below what the earlier nodes of
// a captured graph carry, and a profiler replaying one of those nodes then failed to launch it.
// It also asks for the largest shared-memory carveout of the unified L1/shared array. An SM runs
// CTAs of different kernels side by side only while they share one carveout; with the driver's
// default choice the small-root forms (a few KB of shared memory) get a smaller carveout than the
// large ones, so the size buckets launched together could not share SMs and the small buckets
// started only once whole SMs had drained.
static inline cudaError_t raiseDynSmem(const void* k, size_t smem) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k);
  if (e != cudaSuccess) return e;
  if (fa.preferredShmemCarveout != (int)cudaSharedmemCarveoutMaxShared) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
  }
  if ((int)smem <= fa.maxDynamicSharedSizeBytes) return cudaSuccess;
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename FT, int kMaxThreads, int kMinBlocks>
cudaError_t launchIpmFormT(const LaunchArgs& a, int grid, int block, size_t smem, cudaStream_t stream) {
  void (*k)(LaunchArgs) = ipmKernel<FT, kMaxThreads, kMinBlocks>;
  cudaError_t e = raiseDynSmem((const void*)k, smem);
  if (e != cudaSuccess) return e;
  k<<<grid, block, smem, stream>>>(a);
  return cudaGetLastError();
}

template <typename FT, int kMaxThreads, int kMinBlocks>
cudaError_t ipmOccupancyFormT(int* blocksPerSM, int block, size_t smem) {
  void (*k)(LaunchArgs) = ipmKernel<FT, kMaxThreads, kMinBlocks>;
  cudaError_t e = raiseDynSmem((const void*)k, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, k, block, smem);
}

template <typename FT>
cudaError_t launchIpmGridT(const LaunchArgs& a, GridCtl* g, int grid, size_t smem, cudaStream_t stream) {
  void (*k)(LaunchArgs) = ipmGridKernel<FT>;
  cudaError_t e = raiseDynSmem((const void*)k, smem);
  if (e != cudaSuccess) return e;
  LaunchArgs av = a;
  av.grid = g;
  void* args[] = {(void*)&av};
  return cudaLaunchCooperativeKernel((const void*)k, dim3(grid), dim3(256), args, smem, stream);
}

template <typename FT>
cudaError_t ipmGridOccupancyT(int* blocksPerSM, size_t smem) {
  void (*k)(LaunchArgs) = ipmGridKernel<FT>;
  cudaError_t e = raiseDynSmem((const void*)k, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, k, 256, smem);
}

// Explicit instantiation (EXT empty) or declaration (EXT extern) of the launchers of one form.
#define CXG_IPM_FORM(EXT, FT, TH, MB)                                                            \
  EXT template cudaError_t launchIpmFormT<FT, TH, MB>(const LaunchArgs&, int, int, size_t, cudaStream_t); \
  EXT template cudaError_t ipmOccupancyFormT<FT, TH, MB>(int*, int, size_t);
#define CXG_IPM_GRID(EXT, FT)                                                                    \
  EXT template cudaError_t launchIpmGridT<FT>(const LaunchArgs&, GridCtl*, int, size_t, cudaStream_t); \
  EXT template cudaError_t ipmGridOccupancyT<FT>(int*, size_t);

}  // namespace cxg
