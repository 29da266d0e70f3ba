// Layout of one problem instance on the device, shared by the host planner (cxg_plan.cpp)
// and the interior-point kernel (cxg_ipm.cuh).
//
// The KKT system of ConicXX (src/conicxx/kkt/kkt_system.h:18-65)
//     K = [ P + epsP I      A'           ]
//         [ A              -(Hs + epsA I) ]
// is factorised here as a reduced system: the rows of every Nonnegative / SecondOrder cone
// block ("cone units": one unit per NN row, one per SOC block) are eliminated block by block
// in FP64 with G_u = (Hs_u + epsA I)^-1, leaving the dense quasi-definite root
//     M = [ P + epsP I + sum_u A_u' G_u A_u    A_Z'     ]     (rows: x, then Zero-cone rows)
//         [ A_Z                                -epsA I  ]
// which is factorised LDL' (FP32 or FP64) without pivoting. The root is stored packed-lower,
// column-major: entry (i, j), i >= j, at rootIdx(nr, i, j).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define CXG_HD __host__ __device__ __forceinline__
#else
#define CXG_HD inline
#endif

namespace cxg {

// The root is stored as the lower triangle of 32x32 tiles (T = ceil(nr/32) tile rows), tiles in
// column-major tile order, each tile column-major with leading dimension 33 (conflict-free row
// and column access in shared memory). Rows/columns beyond nr are identity padding.
// The upper half of a diagonal tile holds the transposed inverse of its unit-lower L block.
constexpr int kTile = 32;
constexpr int kTileLd = 33;
constexpr int kTileElems = kTile * kTileLd;

CXG_HD int rootTiles(int nr) { return (nr + kTile - 1) / kTile; }
CXG_HD int64_t tileBase(int T, int I, int J) {
  return ((int64_t)J * T - ((int64_t)J * (J - 1)) / 2 + (I - J)) * kTileElems;
}
// Element (i, j), i >= j, of the root.
CXG_HD int64_t rootIdx(int nr, int i, int j) {
  return tileBase(rootTiles(nr), i / kTile, j / kTile) + (int64_t)(j % kTile) * kTileLd + (i % kTile);
}
CXG_HD int64_t rootSize(int nr) {
  const int T = rootTiles(nr);
  return (int64_t)T * (T + 1) / 2 * kTileElems;
}

// Offsets are element offsets into the int pool (I*), the double pool (D*), or the
// concatenated user value arrays (V*). All int32 index data lives in the int pool.
struct InstanceDesc {
  int n, m, p, l, nsoc, nr;    // sizes: variables, constraints, Zero rows, NN rows, SOC blocks, root
  int nnzPu;                   // stored entries of the user's P (upper CSC)
  int nnzPs;                   // entries of the full symmetric P (CSR, both triangles)
  int nnzA;                    // stored entries of A
  int nPlow;                   // strictly-upper P entries scattered into the root
  int nAZ;                     // A entries in Zero-cone rows scattered into the root
  int nUnits;                  // cone units = l + nsoc
  int nAd;                     // entries of the densified per-unit A blocks (sum d_u * s_u)
  int nTgt;                    // root entries receiving cone-unit contributions
  int nContrib;                // contributions
  int pStoredNnz;              // P.nonZeros() of the user's P (the initial-point branch test)
  int pad0;
  // int pool offsets
  int64_t iPp, iPi;                   // the user's P pattern (upper CSC as given)
  int64_t iPsRow, iPsCol, iPsSrc;     // full symmetric P: CSR row ptr (n+1), cols, source index into Px
  int64_t iPdiag;                     // n: source index of P(i,i) in Px or -1
  int64_t iPlowIdx, iPlowSrc;         // nPlow: root index, Px source
  int64_t iAp, iAi;                   // A CSC: col ptr (n+1), row idx (nnzA)
  int64_t iArRow, iArCol, iArSrc;     // A CSR: row ptr (m+1), col idx, source index into Ax
  int64_t iAZIdx, iAZSrc;             // nAZ: root index, Ax source
  int64_t iSocOff, iSocDim;           // nsoc: row offset (within m) and dimension of each SOC block
  int64_t iUnitAd;                    // nUnits+1: offset of each unit's Ad block (d_u x s_u, col-major)
  int64_t iUnitSup;                   // nUnits+1: offset of each unit's support list
  int64_t iSup;                       // support lists (x column indices)
  int64_t iAdSrc;                     // nAd: Ax source index or -1 (structural zero)
  int64_t iTgtIdx, iTgtBeg;           // nTgt root indices; nTgt+1 contribution ranges
  int64_t iContrib;                   // 3*nContrib: (Ad column offset i, Ad column offset j, d)
  // double pool offsets (equilibration, src/conicxx/kkt/equilibration.h:45-54)
  int64_t dD, dE;                     // n, m
  double cscale;
  // offsets into the concatenated value arrays
  int64_t vPx, vQ, vAx, vB;           // user values (P upper CSC order, q, A CSC order, b)
  int64_t vX, vS, vZ;                 // outputs: x at vQ-like offset (n), s/z at vB-like offset (m)
  // per-instance FP64 scratch offsets (relative to the CTA's scratch base)
  int64_t sPv, sAv, sAd, sT, sQ, sB;  // scaled P (user order, then CSR order), scaled A, Ad, T, q, b
  int64_t sRoot64;                    // FP64 root (fallback / FP64 precision when not in SMEM)
  int64_t sVec;                       // FP64 vectors that do not fit in shared memory
  int64_t sVecG;                      // FP64 vectors always kept in scratch (vecGlobalDoubles)
  int64_t sKry;                       // whole-GPU form: the GMRES Krylov area (krylovDoubles)
  int64_t sSlice;                     // whole-GPU mixed form: the double-float panel slices (dfSliceBytes)
  int64_t scratchDoubles;             // total per-CTA scratch this instance needs
  int64_t bwdOff;                     // offset of this instance's saved final state (differentiable)
  double cost;                        // scheduling weight (~ nr^3)
};

// Saved final state of one instance for the adjoint (differentiable batches), in doubles:
// FP64 root factor, NN/SOC scaling (w, G eigenvalues / u, SOC parameters), normalised iterate
// x/tau and z/tau, and [bump_a, bump_p, status, tau].
struct BwdLayout {
  int64_t root, cw, cu, sp, xh, zh, sc, total;
};
CXG_HD BwdLayout bwdLayout(int nr, int n, int m, int nsoc) {
  BwdLayout b{};
  int64_t o = 0;
  b.root = o; o += rootSize(nr);
  b.cw = o; o += m;
  b.cu = o; o += m;
  b.sp = o; o += 8 * (int64_t)nsoc;
  b.xh = o; o += n;
  b.zh = o; o += m;
  b.sc = o; o += 4;
  b.total = (o + 1) & ~int64_t(1);
  return b;
}

// Kernel-side copy of the solver settings (cxg_settings) in the units the kernel uses.
struct DevSettings {
  double tol_feas, tol_gap_abs, tol_gap_rel, tol_infeas;
  double static_reg_P, static_reg_A, dynamic_reg_eps, dynamic_reg_delta;
  double refine_tol, max_step_fraction, mixed_fallback_tol;
  int max_iter, refine_max_iter, mixed_refine_max_iter, linear_solver;
  int equilibrate, warm_start, precision, record_timings;
  int fault_factor_failures, fault_nonfinite_solves;  // test-only fault injection (0 = off)
  int soc_ref_dense, pad0;  // SOC pivot test and Hs products in the reference's dense form
};

// Per-instance result written by the kernel (mirrors cxg_info plus internal counters).
struct DevResult {
  int status, iterations, fp64_fallbacks, refine_steps;
  double objective, primal_residual, dual_residual, duality_gap, mu, max_relres;
  int factor_attempts, error_code;  // error_code: 0 ok, else an internal diagnostic (bounds etc.)
  int escalations, pad1;            // refactorisations of escalateAndResolve (x1000 bumps)
  long long cycles[8];              // record_timings: total, factorisation, KKT solves, residual/cones,
                                    // assembly, dense LDL', dense triangular solves, KKT residuals
  long long wall_ns[2];             // record_timings: device global timer at the instance's start and end
};

}  // namespace cxg
