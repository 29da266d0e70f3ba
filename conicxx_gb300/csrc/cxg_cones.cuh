// Device-side cone algebra (FP64), one cone unit per call.
//
// Semantics follow src/conicxx/cones/{nonnegative_cone,second_order_cone,zero_cone}.cpp and
// cone_set.cpp; the Nesterov-Todd scaling of a second-order block is held in eigen-form rather
// than as the dense W = beta (2 v v' - J) the reference caches (second_order_cone.cpp:132-158):
// W acts as beta * I off the plane span{e0, (0, u)} (u = v1/|v1|) and as beta * B in it,
// B = [[2v0^2-1, 2 v0 |v1|], [2 v0 |v1|, 2|v1|^2+1]] with eigenvalues lambda, 1/lambda
// (det B = 2 v'Jv - 1 = 1). Every operator the interior-point method needs -- W, W^-1,
// Hs = W^2, Hs + eps I and (Hs + eps I)^-1 -- is then f(W) for a scalar f, applied in O(dim)
// along the eigenvectors. Applying these near-singular operators as dense matrices loses all
// accuracy once cond(Hs) approaches 1/eps_machine (Hs * (Hs+eps)^-1 - I reaches O(0.1) in FP64),
// whereas the eigen-form round trip stays at FP64 rounding.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace cxg {

constexpr double kTiny = 1e-12;                    // second_order_cone.cpp:23
constexpr double kDblMin = 2.2250738585072014e-308;
constexpr double kStepDegenerateEps = kDblMin * 1e4;  // second_order_cone.cpp:32
constexpr double kTinyRel = 1e-12;                 // second_order_cone.cpp:89
constexpr double kAbsFloor = kDblMin * 1e4;        // second_order_cone.cpp:90
constexpr double kBetaMax = 1e8;                   // second_order_cone.cpp:106
constexpr double kWMax = 1e8;                      // second_order_cone.cpp:152
// relative resolution of a dense FP64 Hs = W W (one ulp of its largest eigenvalue); see the
// reference dense form below
constexpr double kHsRes = 2.220446049250313e-16;

// Per-SOC-block scaling parameters (8 doubles in shared memory):
// [0] kind (0 identity fallback, 1 diagonal, 2 plane, 3 plane with the small eigenvalue of Hs held
// at the dense form's resolution, hsSmall), [1] beta, [2] lambda (plane) or
// a = 2v0^2-1 (diagonal), [3] q1c, [4] q1s (in-plane eigenvector of lambda), [5..7] the three
// eigenvalues of G = (Hs + eps I)^-1 prepared at factorisation time (socPrepareG).
// The unit vector u is kept in a row-indexed array at rows off+1 .. off+dim-1.
struct SocScale {
  double kind, beta, lam, qc, qs, r0, r1, r2;
};

// Computes the NT scaling of one SOC block from (s, z) (second_order_cone.cpp:70-159): the same
// clamps (margin floors, beta clamp, c floor, v0 floor) and the same identity fallback test on
// the entries of W = beta (2 v v' - J).
__device__ __forceinline__ void socUpdateScaling(const double* s, const double* z, int d,
                                                 SocScale& sc, double* u) {
  double s1sq = 0, z1sq = 0, sz = 0;
  for (int i = 1; i < d; ++i) {
    s1sq += s[i] * s[i];
    z1sq += z[i] * z[i];
  }
  for (int i = 0; i < d; ++i) sz += s[i] * z[i];
  const double s0 = s[0], z0 = z[0];
  const double a = sqrt(fmax(fmax(s0 * s0 - s1sq, kTinyRel * s0 * s0), kAbsFloor));
  const double b = sqrt(fmax(fmax(z0 * z0 - z1sq, kTinyRel * z0 * z0), kAbsFloor));
  const double beta = fmin(fmax(sqrt(a / b), 1.0 / kBetaMax), kBetaMax);
  const double c = sqrt(fmax((sz / (a * b) + 1.0) / 2.0, kTiny));
  // v = (s/a + J z / b) / (2c); v0 += 1; v0 = max(v0, tiny); v /= sqrt(2 v0)
  const double inv2c = 1.0 / (2.0 * c);
  double v0 = (z0 / b + s0 / a) / (2.0 * c);
  v0 += 1.0;
  v0 = fmax(v0, kTiny);
  const double nrm = sqrt(2.0 * v0);
  v0 /= nrm;
  double n1sq = 0.0, vmax1 = 0.0, vmax2 = 0.0, vdiagmax = 0.0;
  bool finite = isfinite(v0) && isfinite(beta);
  for (int i = 1; i < d; ++i) {
    const double vi = ((-z[i] / b + s[i] / a) / (2.0 * c)) / nrm;
    (void)inv2c;
    u[i] = vi;
    n1sq += vi * vi;
    const double av = fabs(vi);
    if (av > vmax1) { vmax2 = vmax1; vmax1 = av; } else if (av > vmax2) { vmax2 = av; }
    vdiagmax = fmax(vdiagmax, fabs(2.0 * vi * vi + 1.0));
    finite = finite && isfinite(vi);
  }
  // max |W_ij| / beta over the explicit W = beta (2 v v' - J)
  double wmax = fabs(2.0 * v0 * v0 - 1.0);
  wmax = fmax(wmax, vdiagmax);
  wmax = fmax(wmax, 2.0 * fabs(v0) * vmax1);
  if (d > 2) wmax = fmax(wmax, 2.0 * vmax1 * vmax2);
  wmax *= beta;
  // Hs = W W has entries up to ~dim * wmax^2: finite whenever W is finite and wmax <= 1e8.
  if (!finite || !(wmax <= kWMax)) {
    sc.kind = 0.0;
    sc.beta = 1.0;
    sc.lam = 1.0;
    sc.qc = 1.0;
    sc.qs = 0.0;
    return;
  }
  const double n1 = sqrt(n1sq);
  sc.beta = beta;
  if (n1 == 0.0 || d == 1) {
    sc.kind = 1.0;
    sc.lam = 2.0 * v0 * v0 - 1.0;
    sc.qc = 1.0;
    sc.qs = 0.0;
    for (int i = 1; i < d; ++i) u[i] = 0.0;
    return;
  }
  for (int i = 1; i < d; ++i) u[i] /= n1;
  const double A = 2.0 * v0 * v0 - 1.0, C = 2.0 * v0 * n1, E = 2.0 * n1 * n1 + 1.0;
  const double h = 0.5 * (A + E);
  const double r = hypot(0.5 * (A - E), C);
  const double l1 = h + r;
  double qa, qb;
  if (A >= E) { qa = l1 - E; qb = C; } else { qa = C; qb = l1 - A; }
  const double qn = hypot(qa, qb);
  sc.kind = 2.0;
  sc.lam = l1;
  sc.qc = qa / qn;
  sc.qs = qb / qn;
}

// Scalar functions of W used by the method.
enum WFun { kW = 0, kWinv = 1, kHs = 2, kHsEps = 3, kGinv = 4 };

__device__ __forceinline__ double wfun(int f, double w, double eps) {
  switch (f) {
    case kW: return w;
    case kWinv: return 1.0 / w;
    case kHs: return w * w;
    case kHsEps: return w * w + eps;
    default: return 1.0 / (w * w + eps);
  }
}

// Functions of Hs given one of its eigenvalues h (f = kHs, kHsEps, kGinv).
__device__ __forceinline__ double hsfun(int f, double h, double eps) {
  return f == kHs ? h : (f == kHsEps ? h + eps : 1.0 / (h + eps));
}

// The small in-plane eigenvalue of Hs of a kind-3 block: (beta / lambda)^2, held at no less than
// kHsRes (beta lambda)^2.
__device__ __forceinline__ double hsSmall(const SocScale& sc) {
  const double w1 = sc.beta * sc.lam, w2 = sc.beta / sc.lam;
  return fmax(w2 * w2, kHsRes * (w1 * w1));
}

// y = f(W) x for one SOC block (x, y may alias only if identical).
__device__ __forceinline__ void socApply(const SocScale& sc, const double* u, int d, int f, double eps,
                                         const double* x, double* y) {
  const int kind = (int)sc.kind;
  if (kind == 0) {
    const double g = wfun(f, 1.0, eps);
    for (int i = 0; i < d; ++i) y[i] = g * x[i];
    return;
  }
  if (kind == 1) {
    const double g0 = wfun(f, sc.beta * sc.lam, eps), g = wfun(f, sc.beta, eps);
    const double x0 = x[0];
    for (int i = 1; i < d; ++i) y[i] = g * x[i];
    y[0] = g0 * x0;
    return;
  }
  const double x0 = x[0];
  double xf = 0.0;
  for (int i = 1; i < d; ++i) xf += u[i] * x[i];
  const double c1 = sc.qc * x0 + sc.qs * xf;
  const double c2 = -sc.qs * x0 + sc.qc * xf;
  const double f1 = wfun(f, sc.beta * sc.lam, eps);
  const double f2 = (kind == 3 && f >= kHs) ? hsfun(f, hsSmall(sc), eps) : wfun(f, sc.beta / sc.lam, eps);
  const double f3 = wfun(f, sc.beta, eps);
  const double y0 = f1 * c1 * sc.qc - f2 * c2 * sc.qs;
  const double yF = f1 * c1 * sc.qs + f2 * c2 * sc.qc;
  for (int i = 1; i < d; ++i) y[i] = f3 * (x[i] - xf * u[i]) + yF * u[i];
  y[0] = y0;
}

// G = (Hs + eps I)^-1 of one SOC block as its three eigenvalues (stored in sc.r0..r2).
__device__ __forceinline__ void socPrepareG(SocScale& sc, double eps) {
  const int kind = (int)sc.kind;
  if (kind == 0) {
    const double g = 1.0 / (1.0 + eps);
    sc.r0 = sc.r1 = sc.r2 = g;
  } else if (kind == 1) {
    const double w0 = sc.beta * sc.lam, w = sc.beta;
    sc.r0 = 1.0 / (w0 * w0 + eps);
    sc.r1 = sc.r2 = 1.0 / (w * w + eps);
  } else {
    const double w1 = sc.beta * sc.lam, w2 = sc.beta / sc.lam, w3 = sc.beta;
    sc.r0 = 1.0 / (w1 * w1 + eps);
    sc.r1 = 1.0 / ((kind == 3 ? hsSmall(sc) : w2 * w2) + eps);
    sc.r2 = 1.0 / (w3 * w3 + eps);
  }
}

// y = G x with the eigenvalues prepared by socPrepareG (same structure as socApply).
__device__ __forceinline__ void socApplyG(const SocScale& sc, const double* u, int d, const double* x, double* y) {
  const int kind = (int)sc.kind;
  if (kind == 0) {
    for (int i = 0; i < d; ++i) y[i] = sc.r0 * x[i];
    return;
  }
  if (kind == 1) {
    const double x0 = x[0];
    for (int i = 1; i < d; ++i) y[i] = sc.r1 * x[i];
    y[0] = sc.r0 * x0;
    return;
  }
  const double x0 = x[0];
  double xf = 0.0;
  for (int i = 1; i < d; ++i) xf += u[i] * x[i];
  const double c1 = sc.qc * x0 + sc.qs * xf;
  const double c2 = -sc.qs * x0 + sc.qc * xf;
  const double y0 = sc.r0 * c1 * sc.qc - sc.r1 * c2 * sc.qs;
  const double yF = sc.r0 * c1 * sc.qs + sc.r1 * c2 * sc.qc;
  for (int i = 1; i < d; ++i) y[i] = sc.r2 * (x[i] - xf * u[i]) + yF * u[i];
  y[0] = y0;
}

// Jordan product (second_order_cone.cpp:43-48); out may alias neither u nor v.
__device__ __forceinline__ void socProduct(const double* u, const double* v, int d, double* out) {
  double dt = 0.0;
  for (int i = 0; i < d; ++i) dt += u[i] * v[i];
  const double u0 = u[0], v0 = v[0];
  for (int i = 1; i < d; ++i) out[i] = u0 * v[i] + v0 * u[i];
  out[0] = dt;
}

// Inverse Jordan product u \ w (second_order_cone.cpp:50-68).
__device__ __forceinline__ void socInverseProduct(const double* u, const double* w, int d, double* out) {
  double u0 = u[0];
  double u1sq = 0.0, nu = 0.0;
  for (int i = 1; i < d; ++i) {
    u1sq += u[i] * u[i];
    nu += u[i] * w[i];
  }
  double rho = u0 * u0 - u1sq;
  if (fabs(rho) < kTiny) rho = (rho >= 0 ? kTiny : -kTiny);
  if (fabs(u0) < kTiny) u0 = kTiny;
  const double w0 = w[0];
  const double k1 = (nu / u0 - w0), k2 = (rho / u0);
  for (int i = 1; i < d; ++i) out[i] = (k1 * u[i] + k2 * w[i]) / rho;
  out[0] = (u0 * w0 - nu) / rho;
}

// Largest step in [0, amax] keeping x + a dx in the closed SOC (second_order_cone.cpp:174-215).
__device__ __forceinline__ double socMaxStep(const double* x, const double* dx, int d, double amax) {
  const double p0 = x[0], d0 = dx[0];
  double d1sq = 0, p1d1 = 0, p1sq = 0;
  for (int i = 1; i < d; ++i) {
    d1sq += dx[i] * dx[i];
    p1d1 += x[i] * dx[i];
    p1sq += x[i] * x[i];
  }
  const double a = d0 * d0 - d1sq;
  const double b = 2.0 * (p0 * d0 - p1d1);
  const double c = p0 * p0 - p1sq;
  double alpha = amax;
  if (fabs(a) < kStepDegenerateEps) {
    if (fabs(b) > kStepDegenerateEps) {
      const double r = -c / b;
      if (r > 0 && (p0 + r * d0) >= 0) alpha = fmin(alpha, r);
    }
    return alpha;
  }
  const double disc = b * b - 4.0 * a * c;
  if (disc < 0) return alpha;
  const double sq = sqrt(disc);
  const double q = (b >= 0) ? -0.5 * (b + sq) : -0.5 * (b - sq);
  double r1, r2;
  if (fabs(q) > kStepDegenerateEps) {
    r1 = q / a;
    r2 = c / q;
  } else {
    r1 = r2 = -b / (2.0 * a);
  }
  if (r1 > 0 && (p0 + r1 * d0) >= 0) alpha = fmin(alpha, r1);
  if (r2 > 0 && (p0 + r2 * d0) >= 0) alpha = fmin(alpha, r2);
  return alpha;
}

// ---- a second-order block in the reference's dense FP64 form -----------------------------
// The reference keeps a block's Hs = W W as a dense FP64 matrix, W = beta (2 v v' - J) formed
// entry by entry (second_order_cone.cpp:132-158). Near the cone boundary the in-plane eigenvalues
// of Hs, beta^2 lambda^2 and beta^2 / lambda^2, lie more than 1/eps_machine apart, and the dense
// entries no longer carry the small one: it is replaced by rounding of the order of
// eps_machine * beta^2 lambda^2. The eigen-form held here is exact to rounding. Two of the
// reference's decisions depend on that rounding, and both are reproduced from the dense entries
// in the reference's arithmetic (its operation order, no fused multiply-adds) for blocks of up to
// kRefDenseMaxDim rows:
//  - the sparse LDL' of K (qdldl_ldlt.cpp:58-69) takes a block's rows before the x rows they
//    couple to (a block row has degree dim - 1 + the nonzeros of its A row), so the block
//    -(Hs + eps I) is factored on its own; its last pivot comes out zero or below
//    dynamic_reg_eps and factorizeWithRetry (kkt_system.cpp:242-264) fails the attempt and raises
//    the bump x10 until the bump survives the block's rounding (socRefLadderLevel);
//  - Hs itself: from the first iteration in which that pivot test fails, the instance holds the
//    small in-plane eigenvalue of Hs at no less than kHsRes times the large one (kind 3 in
//    SocScale: Hs, Hs + eps I and G; W and W^-1 stay exact), the resolution of the dense form.
//    With the exact small eigenvalue the iteration drives the complementarity of such blocks to
//    zero ahead of primal feasibility and then stalls (configuration 2's family from 3000
//    variables on; the reference's own iteration with exact Hs products slows from 26 to 76
//    iterations there); at the dense form's resolution it converges as the reference does.
constexpr int kRefDenseMaxDim = 8;
constexpr int kLadderLevels = 18;  // factorizeWithRetry's attempts (kkt_system.cpp:242-264)

// the bump of ladder attempt `level`: 0, delta, 10 delta, ... (kkt_system.cpp:258-259)
__host__ __device__ __forceinline__ double ladderBump(int level, double delta) {
  double e = 0.0;
  for (int k = 0; k < level; ++k) e = fmax(e * 10.0, delta);
  return e;
}

// Dense Hs of one block (row-major d x d, d <= kRefDenseMaxDim) in the reference's arithmetic;
// false for the identity fallback (W non-finite or max |W_ij| > 1e8), where Hs = I.
static __device__ __noinline__ bool socRefHs(const double* s, const double* z, int d, double* Hs) {
  double v[kRefDenseMaxDim];
  double s1sq = 0.0, z1sq = 0.0, sz = 0.0;
  for (int i = 1; i < d; ++i) {
    s1sq = __dadd_rn(s1sq, __dmul_rn(s[i], s[i]));
    z1sq = __dadd_rn(z1sq, __dmul_rn(z[i], z[i]));
  }
  for (int i = 0; i < d; ++i) sz = __dadd_rn(sz, __dmul_rn(s[i], z[i]));
  const double s0 = s[0], z0 = z[0];
  const double a =
      __dsqrt_rn(fmax(fmax(__dsub_rn(__dmul_rn(s0, s0), s1sq), __dmul_rn(__dmul_rn(kTinyRel, s0), s0)), kAbsFloor));
  const double b =
      __dsqrt_rn(fmax(fmax(__dsub_rn(__dmul_rn(z0, z0), z1sq), __dmul_rn(__dmul_rn(kTinyRel, z0), z0)), kAbsFloor));
  const double beta = fmin(fmax(__dsqrt_rn(__ddiv_rn(a, b)), __ddiv_rn(1.0, kBetaMax)), kBetaMax);
  const double c = __dsqrt_rn(fmax(__ddiv_rn(__dadd_rn(__ddiv_rn(sz, __dmul_rn(a, b)), 1.0), 2.0), kTiny));
  v[0] = __dadd_rn(__ddiv_rn(z0, b), __ddiv_rn(s0, a));
  for (int i = 1; i < d; ++i) v[i] = __dadd_rn(__ddiv_rn(-z[i], b), __ddiv_rn(s[i], a));
  const double c2 = __dmul_rn(2.0, c);
  for (int i = 0; i < d; ++i) v[i] = __ddiv_rn(v[i], c2);
  v[0] = fmax(__dadd_rn(v[0], 1.0), kTiny);
  const double nrm = __dsqrt_rn(__dmul_rn(2.0, v[0]));
  for (int i = 0; i < d; ++i) v[i] = __ddiv_rn(v[i], nrm);
  auto W = [&](int r, int cc) {
    double w = __dmul_rn(__dmul_rn(2.0, v[r]), v[cc]);
    if (r == cc) w = (r == 0) ? __dsub_rn(w, 1.0) : __dadd_rn(w, 1.0);
    return __dmul_rn(w, beta);
  };
  double wmax = 0.0;
  bool finite = true;
  for (int r = 0; r < d; ++r)
    for (int cc = 0; cc < d; ++cc) {
      const double w = W(r, cc);
      finite = finite && isfinite(w);
      wmax = fmax(wmax, fabs(w));
    }
  if (finite && wmax <= kWMax) {
    for (int r = 0; r < d; ++r)
      for (int cc = 0; cc < d; ++cc) {
        double acc = 0.0;
        for (int k = 0; k < d; ++k) acc = __dadd_rn(acc, __dmul_rn(W(r, k), W(k, cc)));
        finite = finite && isfinite(acc);
        Hs[r * d + cc] = acc;
      }
    if (finite) return true;
  }
  for (int r = 0; r < d; ++r)
    for (int cc = 0; cc < d; ++cc) Hs[r * d + cc] = (r == cc) ? 1.0 : 0.0;
  return false;
}

// The first ladder level (attempt index, 0..17) at which the block's dense pivots all pass, or
// 18 when none does; the search starts at startLevel (a block that passes there returns
// startLevel). Blocks of one row or above kRefDenseMaxDim rows: 0.
static __device__ __noinline__ int socRefLadderLevel(const double* s, const double* z, int d, double sregA,
                                                     double deps, double delta, int startLevel) {
  if (d > kRefDenseMaxDim || d < 2) return 0;
  double Hs[kRefDenseMaxDim * kRefDenseMaxDim];
  if (!socRefHs(s, z, d, Hs)) return 0;  // Hs = I: every pivot passes
  for (int level = startLevel; level < kLadderLevels; ++level) {
    const double ea = ladderBump(level, delta);
    // up-looking LDL' of -(Hs + sregA I) - ea I in natural order, QDLDL's operation order
    double L[kRefDenseMaxDim * kRefDenseMaxDim], Dinv[kRefDenseMaxDim], y[kRefDenseMaxDim];
    bool ok = true;
    for (int k = 0; k < d && ok; ++k) {
      double Dk = __dsub_rn(-Hs[k * d + k], sregA);
      if (ea != 0.0) Dk = __dsub_rn(Dk, ea);
      for (int r = 0; r < k; ++r) y[r] = -Hs[k * d + r];
      for (int cc = 0; cc < k; ++cc) {
        const double yc = y[cc];
        for (int r = cc + 1; r < k; ++r) y[r] = __dsub_rn(y[r], __dmul_rn(L[r * kRefDenseMaxDim + cc], yc));
        const double l = __dmul_rn(yc, Dinv[cc]);
        L[k * kRefDenseMaxDim + cc] = l;
        Dk = __dsub_rn(Dk, __dmul_rn(yc, l));
      }
      ok = isfinite(Dk) && fabs(Dk) > deps;
      Dinv[k] = __ddiv_rn(1.0, Dk);
    }
    if (ok) return level;
  }
  return kLadderLevels;
}

__device__ __forceinline__ double socMargin(const double* x, int d) {
  double t = 0.0;
  for (int i = 1; i < d; ++i) t += x[i] * x[i];
  return x[0] - sqrt(t);
}

}  // namespace cxg
