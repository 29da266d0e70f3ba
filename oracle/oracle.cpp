// ORACLE -- TEST INFRASTRUCTURE ONLY. Never linked into, loaded by, or called from the product
// path (conicxx_gb300/). Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
// it, and only as the checker / the timed CPU restatement of the reference.
//
// An FP64 CPU restatement of ConicXX's interior-point hot path, written from the reference's
// behaviour (file:line citations are relative to the ConicXX source tree):
//   * cones:            src/conicxx/cones/{zero_cone,nonnegative_cone,second_order_cone,cone_set}.cpp
//   * KKT system:       src/conicxx/kkt/kkt_system.cpp:22-311, sparsity_map.cpp:8-56
//   * LDL^T backends:   src/conicxx/kkt/qdldl_ldlt.cpp:22-75 (QDLDL semantics: fail on an exact
//                       zero pivot) and src/conicxx/kkt/regularized_ldlt.cpp:51-260 (per-pivot rule)
//   * equilibration:    src/conicxx/kkt/equilibration.cpp:8-139
//   * IPM driver:       src/conicxx/solver_impl.cpp:8-466
// Third-party pieces the reference links but that are absent here are re-derived from their
// published algorithms, not copied: the fill-reducing ordering is an exact minimum-degree
// ordering (the reference uses Eigen 3.4.0's AMDOrdering), the elimination tree / column counts
// and the up-looking LDL^T follow the textbook algorithms that qdldl v0.1.9 implements
// (T. Davis, "Direct Methods for Sparse Linear Systems", ch. 4), and the SOC W^-1 uses a partial
// pivoting LU (the reference uses Eigen::PartialPivLU). Different orderings change rounding only.
//
// Parity is pinned to the reference's own known-answer tests (test/solver/*, test/cones/*,
// test/kkt/*), re-expressed in tests/test_oracle_kats.py; the reference cannot be compiled in
// this environment (Eigen, qdldl and googletest are absent).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <thread>
#include <utility>
#include <vector>

#include "conicxx_gb300.h"

namespace orc {

using Vec = std::vector<double>;

static double dot(const double* a, const double* b, int n) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
static double norm2(const double* a, int n) { return std::sqrt(dot(a, a, n)); }
static bool allFinite(const Vec& v) {
  for (double x : v)
    if (!std::isfinite(x)) return false;
  return true;
}

struct Csc {
  int rows = 0, cols = 0;
  std::vector<int> p, i;
  Vec x;
  int nnz() const { return p.empty() ? 0 : p[(size_t)cols]; }
};

static Csc makeCsc(int rows, int cols, const int* p, const int* i, const double* x) {
  Csc c;
  c.rows = rows;
  c.cols = cols;
  c.p.assign(p, p + cols + 1);
  const int nz = p[cols];
  c.i.assign(i, i + nz);
  c.x.assign(x, x + nz);
  return c;
}

// y = P_sym * v, P given by its upper triangle (selfadjointView<Upper>, solver_impl.cpp:102);
// stored entries below the diagonal are ignored.
static void symUpperMul(const Csc& P, const double* v, double* y) {
  for (int r = 0; r < P.rows; ++r) y[r] = 0;
  for (int c = 0; c < P.cols; ++c) {
    for (int k = P.p[c]; k < P.p[c + 1]; ++k) {
      const int r = P.i[k];
      if (r > c) continue;
      const double a = P.x[k];
      y[r] += a * v[c];
      if (r != c) y[c] += a * v[r];
    }
  }
}

// ------------------------------------------------------------------------------------------
// Cones (cone_set.cpp, nonnegative_cone.cpp, second_order_cone.cpp, zero_cone.cpp)
// ------------------------------------------------------------------------------------------
enum BlockType { kZero = 0, kNonneg = 1, kSoc = 2 };
struct Block {
  int type, off, dim;
};

constexpr double kTiny = 1e-12;                                           // second_order_cone.cpp:23
constexpr double kStepDegenerateEps = std::numeric_limits<double>::min() * 1e4;  // :32
constexpr double kTinyRel = 1e-12;                                        // :89
constexpr double kAbsFloor = std::numeric_limits<double>::min() * 1e4;   // :90
constexpr double kBetaMax = 1e8;                                          // :106
constexpr double kWMax = 1e8;                                             // :152

// Dense d x d LU with partial pivoting (stand-in for Eigen::PartialPivLU, second_order_cone.cpp:158).
struct SmallLU {
  int d = 0;
  Vec lu;
  std::vector<int> piv;
  void compute(const Vec& A, int dim) {
    d = dim;
    lu = A;
    piv.resize((size_t)d);
    for (int k = 0; k < d; ++k) {
      int p = k;
      double best = std::abs(lu[(size_t)k * d + k]);
      for (int r = k + 1; r < d; ++r) {
        const double v = std::abs(lu[(size_t)r * d + k]);
        if (v > best) { best = v; p = r; }
      }
      piv[(size_t)k] = p;
      if (p != k)
        for (int c = 0; c < d; ++c) std::swap(lu[(size_t)k * d + c], lu[(size_t)p * d + c]);
      const double pv = lu[(size_t)k * d + k];
      if (pv == 0.0) continue;
      for (int r = k + 1; r < d; ++r) {
        const double f = lu[(size_t)r * d + k] / pv;
        lu[(size_t)r * d + k] = f;
        for (int c = k + 1; c < d; ++c) lu[(size_t)r * d + c] -= f * lu[(size_t)k * d + c];
      }
    }
  }
  void solve(const double* b, double* x) const {
    for (int i = 0; i < d; ++i) x[i] = b[i];
    for (int k = 0; k < d; ++k)
      if (piv[(size_t)k] != k) std::swap(x[k], x[piv[(size_t)k]]);
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < r; ++c) x[r] -= lu[(size_t)r * d + c] * x[c];
    for (int r = d - 1; r >= 0; --r) {
      for (int c = r + 1; c < d; ++c) x[r] -= lu[(size_t)r * d + c] * x[c];
      x[r] /= lu[(size_t)r * d + r];
    }
  }
};

class Cones {
 public:
  std::vector<Block> blocks;
  int m = 0, degree = 0;
  Vec e;
  // Scaling state. NN: w per row (stored at the row's offset), Hs = w^2. SOC: dense W, Hs, LU.
  Vec nn_w, nn_h;
  std::vector<Vec> W, Hs;
  std::vector<SmallLU> lu;

  void build(int zero, int nn, const std::vector<int>& soc) {
    blocks.clear();
    int off = 0;
    degree = 0;
    if (zero > 0) { blocks.push_back({kZero, off, zero}); off += zero; }
    if (nn > 0) { blocks.push_back({kNonneg, off, nn}); off += nn; degree += nn; }
    for (int d : soc) { blocks.push_back({kSoc, off, d}); off += d; degree += 1; }
    m = off;
    e.assign((size_t)m, 0.0);
    nn_w.assign((size_t)m, 1.0);
    nn_h.assign((size_t)m, 1.0);
    W.assign(blocks.size(), Vec());
    Hs.assign(blocks.size(), Vec());
    lu.assign(blocks.size(), SmallLU());
    for (size_t b = 0; b < blocks.size(); ++b) {
      const Block& B = blocks[b];
      if (B.type == kNonneg)
        for (int i = 0; i < B.dim; ++i) e[(size_t)(B.off + i)] = 1.0;
      if (B.type == kSoc) {
        e[(size_t)B.off] = 1.0;
        W[b].assign((size_t)B.dim * B.dim, 0.0);
        for (int i = 0; i < B.dim; ++i) W[b][(size_t)i * B.dim + i] = 1.0;
        Hs[b] = W[b];
        lu[b].compute(W[b], B.dim);
      }
    }
  }

  // nonnegative_cone.cpp:22-26, second_order_cone.cpp:70-159
  void updateScaling(const double* s, const double* z) {
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const Block& B = blocks[bi];
      if (B.type == kNonneg) {
        for (int i = B.off; i < B.off + B.dim; ++i) {
          const double w = std::sqrt(s[i] / z[i]);
          nn_w[(size_t)i] = w;
          nn_h[(size_t)i] = w * w;
        }
      } else if (B.type == kSoc) {
        socScaling(bi, s + B.off, z + B.off);
      }
    }
  }

  void socScaling(size_t bi, const double* s, const double* z) {
    const int d = blocks[bi].dim;
    double s1sq = 0, z1sq = 0, sz = 0;
    for (int i = 1; i < d; ++i) { s1sq += s[i] * s[i]; z1sq += z[i] * z[i]; }
    for (int i = 0; i < d; ++i) sz += s[i] * z[i];
    const double s0 = s[0], z0 = z[0];
    const double a = std::sqrt(std::max({s0 * s0 - s1sq, kTinyRel * s0 * s0, kAbsFloor}));
    const double b = std::sqrt(std::max({z0 * z0 - z1sq, kTinyRel * z0 * z0, kAbsFloor}));
    const double beta = std::min(std::max(std::sqrt(a / b), 1.0 / kBetaMax), kBetaMax);
    const double c = std::sqrt(std::max((sz / (a * b) + 1.0) / 2.0, kTiny));
    Vec v((size_t)d);
    v[0] = z0 / b;
    for (int i = 1; i < d; ++i) v[(size_t)i] = -z[i] / b;
    v[0] += s0 / a;
    for (int i = 1; i < d; ++i) v[(size_t)i] += s[i] / a;
    for (int i = 0; i < d; ++i) v[(size_t)i] /= (2.0 * c);
    v[0] += 1.0;
    v[0] = std::max(v[0], kTiny);
    const double nrm = std::sqrt(2.0 * v[0]);
    for (int i = 0; i < d; ++i) v[(size_t)i] /= nrm;
    Vec& Wb = W[bi];
    Vec& Hb = Hs[bi];
    Wb.assign((size_t)d * d, 0.0);
    for (int r = 0; r < d; ++r)
      for (int cc = 0; cc < d; ++cc) Wb[(size_t)r * d + cc] = 2.0 * v[(size_t)r] * v[(size_t)cc];
    Wb[0] -= 1.0;
    for (int i = 1; i < d; ++i) Wb[(size_t)i * d + i] += 1.0;
    for (double& w : Wb) w *= beta;
    Hb.assign((size_t)d * d, 0.0);
    for (int r = 0; r < d; ++r)
      for (int cc = 0; cc < d; ++cc) {
        double acc = 0;
        for (int k = 0; k < d; ++k) acc += Wb[(size_t)r * d + k] * Wb[(size_t)k * d + cc];
        Hb[(size_t)r * d + cc] = acc;
      }
    bool bad = false;
    double wmax = 0;
    for (double w : Wb) { if (!std::isfinite(w)) bad = true; wmax = std::max(wmax, std::abs(w)); }
    for (double h : Hb) if (!std::isfinite(h)) bad = true;
    if (bad || wmax > kWMax) {
      for (int r = 0; r < d; ++r)
        for (int cc = 0; cc < d; ++cc) {
          Wb[(size_t)r * d + cc] = (r == cc) ? 1.0 : 0.0;
          Hb[(size_t)r * d + cc] = (r == cc) ? 1.0 : 0.0;
        }
    }
    lu[bi].compute(Wb, d);
  }

  void product(const double* u, const double* v, double* out) const {
    for (const Block& B : blocks) {
      const int o = B.off, d = B.dim;
      if (B.type == kZero) {
        for (int i = 0; i < d; ++i) out[o + i] = 0;
      } else if (B.type == kNonneg) {
        for (int i = 0; i < d; ++i) out[o + i] = u[o + i] * v[o + i];
      } else {
        const double u0 = u[o], v0 = v[o];
        const double d0 = dot(u + o, v + o, d);
        for (int i = 1; i < d; ++i) out[o + i] = u0 * v[o + i] + v0 * u[o + i];
        out[o] = d0;
      }
    }
  }

  void inverseProduct(const double* u, const double* w, double* out) const {
    for (const Block& B : blocks) {
      const int o = B.off, d = B.dim;
      if (B.type == kZero) {
        for (int i = 0; i < d; ++i) out[o + i] = 0;
      } else if (B.type == kNonneg) {
        for (int i = 0; i < d; ++i) out[o + i] = w[o + i] / u[o + i];
      } else {
        double u0 = u[o];
        double u1sq = 0, nu = 0;
        for (int i = 1; i < d; ++i) { u1sq += u[o + i] * u[o + i]; nu += u[o + i] * w[o + i]; }
        double rho = u0 * u0 - u1sq;
        if (std::abs(rho) < kTiny) rho = (rho >= 0 ? kTiny : -kTiny);
        if (std::abs(u0) < kTiny) u0 = kTiny;
        const double w0 = w[o];
        Vec tmp((size_t)d);
        tmp[0] = (u0 * w0 - nu) / rho;
        for (int i = 1; i < d; ++i)
          tmp[(size_t)i] = ((nu / u0 - w0) * u[o + i] + (rho / u0) * w[o + i]) / rho;
        for (int i = 0; i < d; ++i) out[o + i] = tmp[(size_t)i];
      }
    }
  }

  void applyW(const double* x, double* out) const {
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const Block& B = blocks[bi];
      const int o = B.off, d = B.dim;
      if (B.type == kZero) {
        for (int i = 0; i < d; ++i) out[o + i] = 0;
      } else if (B.type == kNonneg) {
        for (int i = 0; i < d; ++i) out[o + i] = nn_w[(size_t)(o + i)] * x[o + i];
      } else {
        Vec tmp((size_t)d, 0.0);
        for (int r = 0; r < d; ++r) {
          double acc = 0;
          for (int c = 0; c < d; ++c) acc += W[bi][(size_t)r * d + c] * x[o + c];
          tmp[(size_t)r] = acc;
        }
        for (int i = 0; i < d; ++i) out[o + i] = tmp[(size_t)i];
      }
    }
  }

  void applyWInv(const double* x, double* out) const {
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const Block& B = blocks[bi];
      const int o = B.off, d = B.dim;
      if (B.type == kZero) {
        for (int i = 0; i < d; ++i) out[o + i] = 0;
      } else if (B.type == kNonneg) {
        for (int i = 0; i < d; ++i) out[o + i] = x[o + i] / nn_w[(size_t)(o + i)];
      } else {
        Vec in(x + o, x + o + d), tmp((size_t)d);
        lu[bi].solve(in.data(), tmp.data());
        for (int i = 0; i < d; ++i) out[o + i] = tmp[(size_t)i];
      }
    }
  }

  // cone_set.cpp:70-75: out = Hs * x block by block.
  void mulHs(const double* x, double* out) const {
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
      const Block& B = blocks[bi];
      const int o = B.off, d = B.dim;
      if (B.type == kZero) {
        for (int i = 0; i < d; ++i) out[o + i] = 0;
      } else if (B.type == kNonneg) {
        for (int i = 0; i < d; ++i) out[o + i] = nn_h[(size_t)(o + i)] * x[o + i];
      } else {
        Vec tmp((size_t)d, 0.0);
        for (int r = 0; r < d; ++r) {
          double acc = 0;
          for (int c = 0; c < d; ++c) acc += Hs[bi][(size_t)r * d + c] * x[o + c];
          tmp[(size_t)r] = acc;
        }
        for (int i = 0; i < d; ++i) out[o + i] = tmp[(size_t)i];
      }
    }
  }

  // cone_set.cpp:77-90 (NN margin is the block minimum, nonnegative_cone.h:29).
  std::pair<double, double> margins(const double* x) const {
    double mn = std::numeric_limits<double>::infinity(), pos = 0.0;
    for (const Block& B : blocks) {
      double mg;
      if (B.type == kZero) {
        mg = std::numeric_limits<double>::infinity();
      } else if (B.type == kNonneg) {
        mg = x[B.off];
        for (int i = 1; i < B.dim; ++i) mg = std::min(mg, x[B.off + i]);
      } else {
        double t = 0;
        for (int i = 1; i < B.dim; ++i) t += x[B.off + i] * x[B.off + i];
        mg = x[B.off] - std::sqrt(t);
      }
      if (std::isfinite(mg)) {
        mn = std::min(mn, mg);
        pos += std::max(mg, 0.0);
      }
    }
    if (!std::isfinite(mn)) mn = 0.0;
    return {mn, pos};
  }

  void scaledUnitShift(double* x, double alpha) const {
    for (const Block& B : blocks) {
      if (B.type == kNonneg)
        for (int i = 0; i < B.dim; ++i) x[B.off + i] += alpha;
      else if (B.type == kSoc)
        x[B.off] += alpha;
    }
  }

  void zeroPrimalZeroConeBlocks(double* s) const {
    for (const Block& B : blocks)
      if (B.type == kZero)
        for (int i = 0; i < B.dim; ++i) s[B.off + i] = 0.0;
  }

  static double socMaxStep(const double* x, const double* dx, int d, double alpha_max) {
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
    auto feasible = [&](double r) { return r > 0 && (p0 + r * d0) >= 0; };
    double alpha = alpha_max;
    if (std::abs(a) < kStepDegenerateEps) {
      if (std::abs(b) > kStepDegenerateEps) {
        const double r = -c / b;
        if (feasible(r)) alpha = std::min(alpha, r);
      }
      return alpha;
    }
    const double disc = b * b - 4.0 * a * c;
    if (disc < 0) return alpha;
    const double sq = std::sqrt(disc);
    const double q = (b >= 0) ? -0.5 * (b + sq) : -0.5 * (b - sq);
    double r1, r2;
    if (std::abs(q) > kStepDegenerateEps) {
      r1 = q / a;
      r2 = c / q;
    } else {
      r1 = r2 = -b / (2.0 * a);
    }
    if (feasible(r1)) alpha = std::min(alpha, r1);
    if (feasible(r2)) alpha = std::min(alpha, r2);
    return alpha;
  }

  // cone_set.cpp:108-115
  double maxStep(const double* x, const double* dx, double alpha_max) const {
    double alpha = alpha_max;
    for (const Block& B : blocks) {
      if (B.type == kNonneg) {
        for (int i = B.off; i < B.off + B.dim; ++i)
          if (dx[i] < 0) alpha = std::min(alpha, -x[i] / dx[i]);
      } else if (B.type == kSoc) {
        alpha = socMaxStep(x + B.off, dx + B.off, B.dim, alpha);
      }
    }
    return alpha;
  }
};

// ------------------------------------------------------------------------------------------
// Sparse LDL^T of the quasi-definite K (qdldl_ldlt.cpp / regularized_ldlt.cpp behaviour)
// ------------------------------------------------------------------------------------------

// Exact minimum-degree ordering of the symmetric pattern given by the lower CSC of K.
// perm[k] = original index eliminated k-th. Ties go to the smallest original index.
static std::vector<int> minimumDegree(int N, const std::vector<int>& Kp, const std::vector<int>& Ki) {
  std::vector<std::vector<int>> adj((size_t)N);
  for (int c = 0; c < N; ++c)
    for (int k = Kp[(size_t)c]; k < Kp[(size_t)c + 1]; ++k) {
      const int r = Ki[(size_t)k];
      if (r == c) continue;
      adj[(size_t)r].push_back(c);
      adj[(size_t)c].push_back(r);
    }
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  std::vector<char> done((size_t)N, 0);
  std::vector<int> perm;
  perm.reserve((size_t)N);
  std::vector<int> merged;
  for (int step = 0; step < N; ++step) {
    int best = -1;
    size_t bestDeg = std::numeric_limits<size_t>::max();
    for (int v = 0; v < N; ++v)
      if (!done[(size_t)v] && adj[(size_t)v].size() < bestDeg) {
        bestDeg = adj[(size_t)v].size();
        best = v;
      }
    const int v = best;
    done[(size_t)v] = 1;
    perm.push_back(v);
    const std::vector<int> nb = adj[(size_t)v];
    for (int u : nb) {
      std::vector<int>& au = adj[(size_t)u];
      merged.clear();
      merged.reserve(au.size() + nb.size());
      size_t i = 0, j = 0;
      while (i < au.size() || j < nb.size()) {
        int take;
        if (j >= nb.size() || (i < au.size() && au[i] < nb[j])) take = au[i++];
        else if (i >= au.size() || nb[j] < au[i]) take = nb[j++];
        else { take = au[i]; ++i; ++j; }
        if (take != v && take != u) merged.push_back(take);
      }
      au.swap(merged);
    }
    adj[(size_t)v].clear();
  }
  return perm;
}

class Ldl {
 public:
  int N = 0, nx = 0;
  bool regularized = false;
  double eps = 1e-14, delta = 1e-7;
  std::vector<int> perm, iperm;           // perm[k] = original at position k
  std::vector<int> Up, Ui;                // permuted upper CSC pattern
  std::vector<int> kmap;                  // K lower value index -> Up value index
  std::vector<int> etree, Lnz, Lp, Li;
  Vec Ux, Lx, D, Dinv;
  std::vector<double> sign;
  int nregularized = 0;
  bool ok = false;
  // work
  std::vector<int> yIdx, elim, nextSpace;
  std::vector<char> mark;
  Vec yVals;

  bool analyze(int dim, int nx_, const std::vector<int>& Kp, const std::vector<int>& Ki, bool reg,
               double eps_, double delta_) {
    N = dim;
    nx = nx_;
    regularized = reg;
    eps = eps_;
    delta = delta_;
    perm = minimumDegree(N, Kp, Ki);
    iperm.assign((size_t)N, 0);
    for (int k = 0; k < N; ++k) iperm[(size_t)perm[(size_t)k]] = k;
    sign.assign((size_t)N, 1.0);
    for (int k = 0; k < N; ++k) sign[(size_t)k] = (perm[(size_t)k] < nx) ? 1.0 : -1.0;
    // permuted upper pattern: entry (r,c) lower in K -> (min(pr,pc), max(pr,pc)) upper.
    const int nnz = Kp[(size_t)N];
    std::vector<int> cnt((size_t)N + 1, 0);
    for (int c = 0; c < N; ++c)
      for (int k = Kp[(size_t)c]; k < Kp[(size_t)c + 1]; ++k) {
        const int pr = iperm[(size_t)Ki[(size_t)k]], pc = iperm[(size_t)c];
        cnt[(size_t)std::max(pr, pc) + 1]++;
      }
    Up.assign((size_t)N + 1, 0);
    for (int c = 0; c < N; ++c) Up[(size_t)c + 1] = Up[(size_t)c] + cnt[(size_t)c + 1];
    std::vector<std::pair<int, int>> ent((size_t)nnz);  // (row, kidx) per upper column
    std::vector<int> fill(Up.begin(), Up.end() - 1);
    kmap.assign((size_t)nnz, 0);
    std::vector<int> rowOf((size_t)nnz), srcOf((size_t)nnz);
    for (int c = 0; c < N; ++c)
      for (int k = Kp[(size_t)c]; k < Kp[(size_t)c + 1]; ++k) {
        const int pr = iperm[(size_t)Ki[(size_t)k]], pc = iperm[(size_t)c];
        const int col = std::max(pr, pc), row = std::min(pr, pc);
        const int pos = fill[(size_t)col]++;
        rowOf[(size_t)pos] = row;
        srcOf[(size_t)pos] = k;
      }
    Ui.assign((size_t)nnz, 0);
    for (int c = 0; c < N; ++c) {
      std::vector<std::pair<int, int>> col;
      for (int pos = Up[(size_t)c]; pos < Up[(size_t)c + 1]; ++pos)
        col.push_back({rowOf[(size_t)pos], srcOf[(size_t)pos]});
      std::sort(col.begin(), col.end());
      for (size_t t = 0; t < col.size(); ++t) {
        const int pos = Up[(size_t)c] + (int)t;
        Ui[(size_t)pos] = col[t].first;
        kmap[(size_t)col[t].second] = pos;
      }
    }
    // elimination tree and column counts of L (up-looking symbolic pass)
    etree.assign((size_t)N, -1);
    Lnz.assign((size_t)N, 0);
    std::vector<int> flag((size_t)N, -1);
    for (int j = 0; j < N; ++j) {
      flag[(size_t)j] = j;
      for (int p = Up[(size_t)j]; p < Up[(size_t)j + 1]; ++p) {
        int i = Ui[(size_t)p];
        if (i >= j) continue;
        while (flag[(size_t)i] != j) {
          if (etree[(size_t)i] == -1) etree[(size_t)i] = j;
          Lnz[(size_t)i]++;
          flag[(size_t)i] = j;
          i = etree[(size_t)i];
        }
      }
    }
    Lp.assign((size_t)N + 1, 0);
    for (int i = 0; i < N; ++i) Lp[(size_t)i + 1] = Lp[(size_t)i] + Lnz[(size_t)i];
    Li.assign((size_t)Lp[(size_t)N], 0);
    Lx.assign((size_t)Lp[(size_t)N], 0.0);
    Ux.assign((size_t)nnz, 0.0);
    D.assign((size_t)N, 0.0);
    Dinv.assign((size_t)N, 0.0);
    yIdx.assign((size_t)N, 0);
    elim.assign((size_t)N, 0);
    nextSpace.assign((size_t)N, 0);
    mark.assign((size_t)N, 0);
    yVals.assign((size_t)N, 0.0);
    return true;
  }

  int nnzL() const { return Lp.empty() ? 0 : Lp[(size_t)N]; }

  // Per-pivot rule of regularized_ldlt.cpp:132-139.
  bool regularize(double& Dk, double sg) const {
    if (Dk * sg >= eps) return false;
    Dk += sg * delta;
    if (Dk * sg < eps) Dk = sg * delta;
    return true;
  }

  // Up-looking numeric factorisation (row k of L from a sparse triangular solve along the
  // elimination tree). QDLDL semantics: an exact zero pivot fails; RegularizedLdlt semantics:
  // correct the pivot, fail if more than 5% were corrected (regularized_ldlt.cpp:107,251).
  // Attribution: this loop follows the up-looking LDL^T of QDLDL (osqp/qdldl v0.1.9, Copyright
  // Paul Goulart and Bartolomeo Stellato, Apache License 2.0), which the reference's
  // src/conicxx/kkt/regularized_ldlt.cpp:166-243 also derives from (its header, :1-23): the
  // elimination-tree reach into a marker / elimination buffer, then the column updates with a
  // next-free-slot pointer per column of L.
  bool factor(const Vec& Kx_lower) {
    for (size_t k = 0; k < kmap.size(); ++k) Ux[(size_t)kmap[k]] = Kx_lower[k];
    for (int i = 0; i < N; ++i) {
      mark[(size_t)i] = 0;
      yVals[(size_t)i] = 0.0;
      D[(size_t)i] = 0.0;
      nextSpace[(size_t)i] = Lp[(size_t)i];
    }
    nregularized = 0;
    bool zeroPivot = false;
    for (int k = 0; k < N; ++k) {
      int nnzY = 0;
      for (int p = Up[(size_t)k]; p < Up[(size_t)k + 1]; ++p) {
        const int r = Ui[(size_t)p];
        if (r == k) { D[(size_t)k] = Ux[(size_t)p]; continue; }
        yVals[(size_t)r] = Ux[(size_t)p];
        int nxt = r;
        if (!mark[(size_t)nxt]) {
          mark[(size_t)nxt] = 1;
          elim[0] = nxt;
          int ne = 1;
          nxt = etree[(size_t)r];
          while (nxt != -1 && nxt < k) {
            if (mark[(size_t)nxt]) break;
            mark[(size_t)nxt] = 1;
            elim[(size_t)ne++] = nxt;
            nxt = etree[(size_t)nxt];
          }
          while (ne) yIdx[(size_t)nnzY++] = elim[(size_t)--ne];
        }
      }
      for (int t = nnzY - 1; t >= 0; --t) {
        const int c = yIdx[(size_t)t];
        const int end = nextSpace[(size_t)c];
        const double yc = yVals[(size_t)c];
        for (int p = Lp[(size_t)c]; p < end; ++p) yVals[(size_t)Li[(size_t)p]] -= Lx[(size_t)p] * yc;
        Li[(size_t)end] = k;
        Lx[(size_t)end] = yc * Dinv[(size_t)c];
        D[(size_t)k] -= yc * Lx[(size_t)end];
        nextSpace[(size_t)c]++;
        yVals[(size_t)c] = 0.0;
        mark[(size_t)c] = 0;
      }
      if (regularized) {
        if (regularize(D[(size_t)k], sign[(size_t)k])) nregularized++;
      } else if (D[(size_t)k] == 0.0) {
        zeroPivot = true;
      }
      Dinv[(size_t)k] = 1.0 / D[(size_t)k];
    }
    if (regularized) ok = !((double)nregularized > 0.05 * (double)N);
    else ok = !zeroPivot;
    return ok;
  }

  double minAbsD() const {
    if (N == 0) return 1.0;
    double mn = std::numeric_limits<double>::infinity();
    for (double d : D) {
      if (!std::isfinite(d)) return std::numeric_limits<double>::quiet_NaN();
      mn = std::min(mn, std::abs(d));
    }
    return mn;
  }

  // x <- K^-1 b (permute, L, D^-1, L', unpermute)
  void solve(const double* b, double* x) const {
    Vec y((size_t)N);
    for (int k = 0; k < N; ++k) y[(size_t)k] = b[perm[(size_t)k]];
    for (int i = 0; i < N; ++i)
      for (int p = Lp[(size_t)i]; p < Lp[(size_t)i + 1]; ++p) y[(size_t)Li[(size_t)p]] -= Lx[(size_t)p] * y[(size_t)i];
    for (int i = 0; i < N; ++i) y[(size_t)i] *= Dinv[(size_t)i];
    for (int i = N - 1; i >= 0; --i)
      for (int p = Lp[(size_t)i]; p < Lp[(size_t)i + 1]; ++p) y[(size_t)i] -= Lx[(size_t)p] * y[(size_t)Li[(size_t)p]];
    for (int k = 0; k < N; ++k) x[perm[(size_t)k]] = y[(size_t)k];
  }
};

// ------------------------------------------------------------------------------------------
// KKT system (kkt_system.cpp:22-311) with the SparsityMap mechanism (sparsity_map.cpp:8-56)
// ------------------------------------------------------------------------------------------
class Kkt {
 public:
  int n = 0, m = 0, N = 0;
  double sregP = 0, sregA = 0, deps = 0, ddelta = 0;
  int refineMax = 3;
  double refineTol = 1e-12;
  // K lower CSC
  std::vector<int> Kp, Ki;
  Vec Kx;
  std::vector<int> pDiagSlot;                 // value offset of K(i,i), i < n
  std::vector<int> pDiagSrc;                  // index into P.x of P(i,i) or -1
  std::vector<std::pair<int, int>> pOff;      // (K offset, P.x index) for P strict upper
  std::vector<std::pair<int, int>> aSlots;    // (K offset, A.x index)
  struct HsSlot { int block, a, b, koff; };
  std::vector<HsSlot> hsSlots;
  std::vector<int> coneDiagSlots;             // K offsets of the cone-block diagonal entries
  std::vector<int> pOuter, pInner, aOuter, aInner;
  Ldl ldl;
  bool factorized = false;
  double lastExtraP = 0, lastExtraA = 0;
  int attemptsLast = 0;

  static bool samePattern(const Csc& M, const std::vector<int>& outer, const std::vector<int>& inner) {
    if ((int)outer.size() != M.cols + 1) return false;
    if (!std::equal(M.p.begin(), M.p.end(), outer.begin())) return false;
    if ((int)inner.size() != M.nnz()) return false;
    return std::equal(M.i.begin(), M.i.begin() + M.nnz(), inner.begin());
  }

  bool setup(const Csc& P, const Csc& A, const Cones& cones, const cxg_settings& st) {
    n = P.rows;
    m = cones.m;
    N = n + m;
    sregP = st.static_reg_P;
    sregA = st.static_reg_A;
    deps = st.dynamic_reg_eps;
    ddelta = st.dynamic_reg_delta;
    refineMax = st.refine_max_iter;
    refineTol = st.refine_tol;
    factorized = false;
    const bool regularized = st.linear_solver == CXG_LINSOLVER_REGULARIZED;

    // Register slots in the reference's order (kkt_system.cpp:54-105).
    std::vector<std::pair<int, int>> entries;  // (row, col)
    std::vector<int> slotPdiag, slotPoff, slotA;
    struct HsReg { int block, a, b, slot; };
    std::vector<HsReg> hsReg;
    for (int i = 0; i < n; ++i) { slotPdiag.push_back((int)entries.size()); entries.push_back({i, i}); }
    std::vector<int> pOffSrc;
    for (int c = 0; c < P.cols; ++c)
      for (int k = P.p[(size_t)c]; k < P.p[(size_t)c + 1]; ++k) {
        const int r = P.i[(size_t)k];
        if (r >= c) continue;
        slotPoff.push_back((int)entries.size());
        pOffSrc.push_back(k);
        entries.push_back({c, r});
      }
    std::vector<int> aSrc;
    for (int c = 0; c < A.cols; ++c)
      for (int k = A.p[(size_t)c]; k < A.p[(size_t)c + 1]; ++k) {
        slotA.push_back((int)entries.size());
        aSrc.push_back(k);
        entries.push_back({n + A.i[(size_t)k], c});
      }
    for (size_t bi = 0; bi < cones.blocks.size(); ++bi) {
      const Block& B = cones.blocks[bi];
      if (B.type == kSoc) {
        for (int a = 0; a < B.dim; ++a)
          for (int b = 0; b <= a; ++b) {
            hsReg.push_back({(int)bi, a, b, (int)entries.size()});
            entries.push_back({n + B.off + a, n + B.off + b});
          }
      } else {
        for (int a = 0; a < B.dim; ++a) {
          hsReg.push_back({(int)bi, a, a, (int)entries.size()});
          entries.push_back({n + B.off + a, n + B.off + a});
        }
      }
    }
    // finalize: unique keys -> compressed CSC (rows sorted in each column)
    std::map<std::pair<int, int>, int> keyOff;
    {
      std::vector<std::pair<int, int>> keys;  // (col, row)
      for (auto& e : entries) keys.push_back({e.second, e.first});
      std::sort(keys.begin(), keys.end());
      keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
      Kp.assign((size_t)N + 1, 0);
      Ki.assign(keys.size(), 0);
      for (size_t t = 0; t < keys.size(); ++t) {
        Kp[(size_t)keys[t].first + 1]++;
        Ki[t] = keys[t].second;
        keyOff[{keys[t].second, keys[t].first}] = (int)t;
      }
      for (int c = 0; c < N; ++c) Kp[(size_t)c + 1] += Kp[(size_t)c];
      Kx.assign(keys.size(), 0.0);
    }
    auto off = [&](int slot) { return keyOff[entries[(size_t)slot]]; };
    pDiagSlot.clear();
    pDiagSrc.assign((size_t)n, -1);
    for (int i = 0; i < n; ++i) pDiagSlot.push_back(off(slotPdiag[(size_t)i]));
    for (int c = 0; c < P.cols; ++c)
      for (int k = P.p[(size_t)c]; k < P.p[(size_t)c + 1]; ++k)
        if (P.i[(size_t)k] == c && pDiagSrc[(size_t)c] < 0) pDiagSrc[(size_t)c] = k;
    pOff.clear();
    for (size_t t = 0; t < slotPoff.size(); ++t) pOff.push_back({off(slotPoff[t]), pOffSrc[t]});
    aSlots.clear();
    for (size_t t = 0; t < slotA.size(); ++t) aSlots.push_back({off(slotA[t]), aSrc[t]});
    hsSlots.clear();
    coneDiagSlots.clear();
    for (auto& h : hsReg) {
      hsSlots.push_back({h.block, h.a, h.b, off(h.slot)});
      if (h.a == h.b) coneDiagSlots.push_back(off(h.slot));
    }
    ldl.analyze(N, n, Kp, Ki, regularized, deps, ddelta);
    pOuter = P.p;
    pInner.assign(P.i.begin(), P.i.begin() + P.nnz());
    aOuter = A.p;
    aInner.assign(A.i.begin(), A.i.begin() + A.nnz());
    if (!updateData(&P, &A)) return false;
    return updateScalingAndFactorize(cones);
  }

  bool updateData(const Csc* P, const Csc* A) {
    if (P) {
      if (!samePattern(*P, pOuter, pInner)) return false;
      for (int i = 0; i < n; ++i) {
        const int src = pDiagSrc[(size_t)i];
        Kx[(size_t)pDiagSlot[(size_t)i]] = (src >= 0 ? P->x[(size_t)src] : 0.0) + sregP;
      }
      for (auto& po : pOff) Kx[(size_t)po.first] = P->x[(size_t)po.second];
    }
    if (A) {
      if (!samePattern(*A, aOuter, aInner)) return false;
      for (auto& as : aSlots) Kx[(size_t)as.first] = A->x[(size_t)as.second];
    }
    return factorizeWithRetry();
  }

  bool updateScalingAndFactorize(const Cones& cones) {
    for (auto& h : hsSlots) {
      const Block& B = cones.blocks[(size_t)h.block];
      double hv = 0.0;
      if (B.type == kNonneg) hv = cones.nn_h[(size_t)(B.off + h.a)];
      else if (B.type == kSoc) hv = cones.Hs[(size_t)h.block][(size_t)h.a * B.dim + h.b];
      double v = -hv;
      if (h.a == h.b) v -= sregA;
      Kx[(size_t)h.koff] = v;
    }
    return factorizeWithRetry();
  }

  // fault injection for tests (cxg_settings::fault_*): armed at the start of every solve
  int faultFactorLeft = 0, faultSolveLeft = 0;
  // attempts of factorizeWithRetry and refactorisations of escalateAndResolve since that start
  int attemptsTotal = 0, escalationsTotal = 0;

  // a solve with the factor; returns a non-finite vector while an injected fault is left
  void backendSolve(const double* rhs, double* x) {
    ldl.solve(rhs, x);
    if (faultSolveLeft > 0) {
      --faultSolveLeft;
      x[0] = std::numeric_limits<double>::quiet_NaN();
    }
  }

  bool tryFactorizeWithBump(double ep, double ea) {
    if (faultFactorLeft > 0) {
      --faultFactorLeft;
      return false;
    }
    if (ep != 0.0 || ea != 0.0) {
      Vec Kt = Kx;
      if (ep != 0.0)
        for (int s : pDiagSlot) Kt[(size_t)s] += ep;
      if (ea != 0.0)
        for (int s : coneDiagSlots) Kt[(size_t)s] -= ea;
      ldl.factor(Kt);
    } else {
      ldl.factor(Kx);
    }
    if (!ldl.ok) return false;
    const double mn = ldl.minAbsD();
    return std::isfinite(mn) && mn > deps;
  }

  bool factorizeWithRetry() {
    double ep = 0.0, ea = 0.0;
    for (int attempt = 0; attempt < 18; ++attempt) {
      ++attemptsTotal;
      if (tryFactorizeWithBump(ep, ea)) {
        factorized = true;
        lastExtraP = ep;
        lastExtraA = ea;
        attemptsLast = attempt + 1;
        return true;
      }
      ep = std::max(ep * 10.0, ddelta);
      ea = std::max(ea * 10.0, ddelta);
    }
    factorized = false;
    attemptsLast = 18;
    return false;
  }

  bool escalateAndResolve(const Vec& rhs, Vec& x) {
    double ep = lastExtraP, ea = lastExtraA;
    for (int attempt = 0; attempt < 10; ++attempt) {
      ep = std::max(ep * 1000.0, ddelta);
      ea = std::max(ea * 1000.0, ddelta);
      ++escalationsTotal;
      if (!tryFactorizeWithBump(ep, ea)) continue;
      backendSolve(rhs.data(), x.data());
      if (allFinite(x)) {
        lastExtraP = ep;
        lastExtraA = ea;
        return true;
      }
    }
    return false;
  }

  // y = K_sym * x from the lower CSC (selfadjointView<Lower>)
  void kmul(const double* x, double* y) const {
    for (int i = 0; i < N; ++i) y[i] = 0;
    for (int c = 0; c < N; ++c)
      for (int k = Kp[(size_t)c]; k < Kp[(size_t)c + 1]; ++k) {
        const int r = Ki[(size_t)k];
        const double v = Kx[(size_t)k];
        y[r] += v * x[c];
        if (r != c) y[c] += v * x[r];
      }
  }

  int lastRefineSteps = 0;
  double solve(const Vec& rhs, Vec& x) {
    x.assign((size_t)N, 0.0);
    backendSolve(rhs.data(), x.data());
    if (!allFinite(x)) escalateAndResolve(rhs, x);
    const double rn = std::max(norm2(rhs.data(), N), 1e-30);
    Vec Kxv((size_t)N), r((size_t)N), dx((size_t)N);
    kmul(x.data(), Kxv.data());
    for (int i = 0; i < N; ++i) r[(size_t)i] = rhs[(size_t)i] - Kxv[(size_t)i];
    double rel = norm2(r.data(), N) / rn;
    lastRefineSteps = 0;
    for (int it = 0; it < refineMax && rel > refineTol; ++it) {
      backendSolve(r.data(), dx.data());
      for (int i = 0; i < N; ++i) x[(size_t)i] += dx[(size_t)i];
      kmul(x.data(), Kxv.data());
      for (int i = 0; i < N; ++i) r[(size_t)i] = rhs[(size_t)i] - Kxv[(size_t)i];
      rel = norm2(r.data(), N) / rn;
      lastRefineSteps++;
    }
    return rel;
  }
};

// ------------------------------------------------------------------------------------------
// Equilibration (equilibration.cpp:8-139)
// ------------------------------------------------------------------------------------------
class Equil {
 public:
  Vec d, e;
  double c = 1.0;
  void compute(const Csc& P, const Csc& A, const Cones& cones, const cxg_settings& st) {
    const int n = P.rows, m = A.rows;
    d.assign((size_t)n, 1.0);
    e.assign((size_t)m, 1.0);
    c = 1.0;
    if (!st.equilibrate || n == 0) return;
    Csc Pw = P, Aw = A;
    const double minS = st.equilibrate_min_scale, maxS = st.equilibrate_max_scale;
    Vec nx((size_t)n), nz((size_t)m), dx((size_t)n), dz((size_t)m);
    for (int it = 0; it < st.equilibrate_max_iter; ++it) {
      std::fill(nx.begin(), nx.end(), 0.0);
      std::fill(nz.begin(), nz.end(), 0.0);
      for (int col = 0; col < Pw.cols; ++col)
        for (int k = Pw.p[(size_t)col]; k < Pw.p[(size_t)col + 1]; ++k) {
          const int r = Pw.i[(size_t)k];
          const double av = std::abs(Pw.x[(size_t)k]);
          nx[(size_t)r] = std::max(nx[(size_t)r], av);
          nx[(size_t)col] = std::max(nx[(size_t)col], av);
        }
      for (int col = 0; col < Aw.cols; ++col)
        for (int k = Aw.p[(size_t)col]; k < Aw.p[(size_t)col + 1]; ++k) {
          const int r = Aw.i[(size_t)k];
          const double av = std::abs(Aw.x[(size_t)k]);
          nx[(size_t)col] = std::max(nx[(size_t)col], av);
          nz[(size_t)r] = std::max(nz[(size_t)r], av);
        }
      for (const Block& B : cones.blocks) {
        if (B.type != kSoc) continue;
        double mx = nz[(size_t)B.off];
        for (int i = 1; i < B.dim; ++i) mx = std::max(mx, nz[(size_t)(B.off + i)]);
        for (int i = 0; i < B.dim; ++i) nz[(size_t)(B.off + i)] = mx;
      }
      for (int i = 0; i < n; ++i) dx[(size_t)i] = 1.0 / std::sqrt(nx[(size_t)i] > 0 ? nx[(size_t)i] : 1.0);
      for (int i = 0; i < m; ++i) dz[(size_t)i] = 1.0 / std::sqrt(nz[(size_t)i] > 0 ? nz[(size_t)i] : 1.0);
      for (int col = 0; col < Pw.cols; ++col)
        for (int k = Pw.p[(size_t)col]; k < Pw.p[(size_t)col + 1]; ++k)
          Pw.x[(size_t)k] *= dx[(size_t)Pw.i[(size_t)k]] * dx[(size_t)col];
      for (int col = 0; col < Aw.cols; ++col)
        for (int k = Aw.p[(size_t)col]; k < Aw.p[(size_t)col + 1]; ++k)
          Aw.x[(size_t)k] *= dz[(size_t)Aw.i[(size_t)k]] * dx[(size_t)col];
      for (int i = 0; i < n; ++i) d[(size_t)i] *= dx[(size_t)i];
      for (int i = 0; i < m; ++i) e[(size_t)i] *= dz[(size_t)i];
    }
    for (double& v : d) v = std::min(std::max(v, minS), maxS);
    for (double& v : e) v = std::min(std::max(v, minS), maxS);
    double sumAbs = 0.0;
    int count = 0;
    for (int k = 0; k < Pw.nnz(); ++k) { sumAbs += std::abs(Pw.x[(size_t)k]); ++count; }
    if (count > 0) {
      const double meanAbs = sumAbs / (double)count;
      if (meanAbs > 0) c = 1.0 / std::max(meanAbs, minS);
    }
    c = std::min(std::max(c, minS), maxS);
  }
  void scaleP(Csc& P) const {
    for (int col = 0; col < P.cols; ++col)
      for (int k = P.p[(size_t)col]; k < P.p[(size_t)col + 1]; ++k)
        P.x[(size_t)k] *= c * d[(size_t)P.i[(size_t)k]] * d[(size_t)col];
  }
  void scaleA(Csc& A) const {
    for (int col = 0; col < A.cols; ++col)
      for (int k = A.p[(size_t)col]; k < A.p[(size_t)col + 1]; ++k)
        A.x[(size_t)k] *= e[(size_t)A.i[(size_t)k]] * d[(size_t)col];
  }
  void scaleQ(Vec& q) const {
    for (size_t i = 0; i < q.size(); ++i) q[i] *= c * d[i];
  }
  void scaleB(Vec& b) const {
    for (size_t i = 0; i < b.size(); ++i) b[i] *= e[i];
  }
  void unscaleSolution(Vec& x, Vec& s, Vec& z) const {
    for (size_t i = 0; i < x.size(); ++i) x[i] *= d[i];
    for (size_t i = 0; i < z.size(); ++i) z[i] = z[i] * e[i] / c;
    for (size_t i = 0; i < s.size(); ++i) s[i] /= e[i];
  }
  void scaleSolution(Vec& x, Vec& s, Vec& z) const {
    for (size_t i = 0; i < x.size(); ++i) x[i] /= d[i];
    for (size_t i = 0; i < z.size(); ++i) z[i] = z[i] * c / e[i];
    for (size_t i = 0; i < s.size(); ++i) s[i] *= e[i];
  }
};

// ------------------------------------------------------------------------------------------
// IPM driver (solver_impl.cpp)
// ------------------------------------------------------------------------------------------
struct TraceRow {
  double mu, norm_rx, norm_rz, pobj, dobj, alpha_aff, sigma, alpha, tau, kappa, relres;
  double attempts;
};
constexpr int kTraceCols = 12;

class Solver {
 public:
  Csc P, A;
  Vec q, b;
  int n = 0, m = 0;
  Cones cones;
  cxg_settings st{};
  Equil eq;
  Kkt kkt;
  bool setupDone = false;
  Vec x, s, z;
  double tau = 1, kappa = 1;
  Vec Px, rx, rz;
  double rtau = 0, dqx = 0, dbz = 0, dsz = 0, dxPx = 0;
  Vec x1, z1, Px1;
  Vec dxa, dza, dsa, dx, dz, ds;
  double dtaua = 0, dkappaa = 0, dtau = 0, dkappa = 0;
  bool haveWarm = false;
  Vec wx, ws, wz;
  // solution
  int status = CXG_STATUS_UNSOLVED;
  Vec solx, sols, solz;
  double objective = 0;
  cxg_info info{};
  std::vector<TraceRow> trace;
  double maxRel = 0;
  int refineSteps = 0;

  bool setup(const cxg_problem& pr, const cxg_settings& settings) {
    setupDone = false;
    if (pr.zero_dim < 0 || pr.nonneg_dim < 0 || pr.n_soc < 0) return false;
    std::vector<int> socd;
    for (int i = 0; i < pr.n_soc; ++i) {
      if (pr.soc_dims[i] < 1) return false;
      socd.push_back(pr.soc_dims[i]);
    }
    n = pr.n;
    int mm = pr.zero_dim + pr.nonneg_dim;
    for (int d : socd) mm += d;
    m = mm;
    if (pr.m != m || n < 0) return false;
    st = settings;
    cones.build(pr.zero_dim, pr.nonneg_dim, socd);
    P = makeCsc(n, n, pr.Pp, pr.Pi, pr.Px);
    A = makeCsc(m, n, pr.Ap, pr.Ai, pr.Ax);
    q.assign(pr.q, pr.q + n);
    b.assign(pr.b, pr.b + m);
    eq = Equil();
    eq.d.assign((size_t)n, 1.0);
    eq.e.assign((size_t)m, 1.0);
    if (st.equilibrate) {
      eq.compute(P, A, cones, st);
      eq.scaleP(P);
      eq.scaleA(A);
      eq.scaleQ(q);
      eq.scaleB(b);
    }
    if (!kkt.setup(P, A, cones, st)) return false;
    x.assign((size_t)n, 0.0); s.assign((size_t)m, 0.0); z.assign((size_t)m, 0.0);
    Px = rx = x1 = Px1 = dxa = dx = x;
    rz = z1 = dza = dsa = dz = ds = s;
    haveWarm = false;
    status = CXG_STATUS_UNSOLVED;
    setupDone = true;
    return true;
  }

  bool updateData(const Csc* Pn, const Vec* qn, const Csc* An, const Vec* bn) {
    if (!setupDone) return false;
    Csc Ps, As;
    Vec qs, bs;
    if (Pn) {
      if (Pn->rows != n || Pn->cols != n) return false;
      Ps = *Pn;
      if (st.equilibrate) eq.scaleP(Ps);
    }
    if (An) {
      if (An->rows != m || An->cols != n) return false;
      As = *An;
      if (st.equilibrate) eq.scaleA(As);
    }
    if (qn) {
      if ((int)qn->size() != n) return false;
      qs = *qn;
      if (st.equilibrate) eq.scaleQ(qs);
    }
    if (bn) {
      if ((int)bn->size() != m) return false;
      bs = *bn;
      if (st.equilibrate) eq.scaleB(bs);
    }
    if (!kkt.updateData(Pn ? &Ps : nullptr, An ? &As : nullptr)) return false;
    if (Pn) P = Ps;
    if (An) A = As;
    if (qn) q = qs;
    if (bn) b = bs;
    return true;
  }

  void setWarmStart(const double* xw, const double* sw, const double* zw) {
    if (!setupDone) return;
    wx.assign(xw, xw + n);
    ws.assign(sw, sw + m);
    wz.assign(zw, zw + m);
    if (st.equilibrate) eq.scaleSolution(wx, ws, wz);
    haveWarm = true;
  }

  void pmul(const double* v, double* y) const { symUpperMul(P, v, y); }

  void shiftToInteriorCold(Vec& v) const {
    auto mg = cones.margins(v.data());
    const double deg = (double)std::max(cones.degree, 1);
    const double target = std::max(1.0, 0.1 * mg.second / deg);
    if (mg.first <= 0.0) {
      cones.scaledUnitShift(v.data(), -mg.first);
      cones.scaledUnitShift(v.data(), target);
    } else if (mg.first < target) {
      cones.scaledUnitShift(v.data(), target - mg.first);
    } else {
      cones.scaledUnitShift(v.data(), 0.0);
    }
  }

  void ensureStrictlyInteriorWarm(Vec& v) const {
    auto mg = cones.margins(v.data());
    if (mg.first <= 1e-8) cones.scaledUnitShift(v.data(), -mg.first + 1e-6);
  }

  double iterRel = 0;
  double kktSolve(const Vec& rhs, Vec& sol) {
    const double rel = kkt.solve(rhs, sol);
    if (rel > maxRel || !std::isfinite(rel)) maxRel = rel;
    if (rel > iterRel || !std::isfinite(rel)) iterRel = rel;
    refineSteps += kkt.lastRefineSteps;
    return rel;
  }

  bool computeInitialPoint() {
    cones.updateScaling(cones.e.data(), cones.e.data());
    if (!kkt.updateScalingAndFactorize(cones)) return false;
    Vec rhs((size_t)(n + m)), sol;
    if (P.nnz() == 0) {
      for (int i = 0; i < n; ++i) rhs[(size_t)i] = 0;
      for (int i = 0; i < m; ++i) rhs[(size_t)(n + i)] = b[(size_t)i];
      kktSolve(rhs, sol);
      for (int i = 0; i < n; ++i) x[(size_t)i] = sol[(size_t)i];
      for (int i = 0; i < m; ++i) s[(size_t)i] = -sol[(size_t)(n + i)];
      for (int i = 0; i < n; ++i) rhs[(size_t)i] = -q[(size_t)i];
      for (int i = 0; i < m; ++i) rhs[(size_t)(n + i)] = 0;
      kktSolve(rhs, sol);
      for (int i = 0; i < m; ++i) z[(size_t)i] = sol[(size_t)(n + i)];
    } else {
      for (int i = 0; i < n; ++i) rhs[(size_t)i] = -q[(size_t)i];
      for (int i = 0; i < m; ++i) rhs[(size_t)(n + i)] = b[(size_t)i];
      kktSolve(rhs, sol);
      for (int i = 0; i < n; ++i) x[(size_t)i] = sol[(size_t)i];
      for (int i = 0; i < m; ++i) { z[(size_t)i] = sol[(size_t)(n + i)]; s[(size_t)i] = -z[(size_t)i]; }
    }
    cones.zeroPrimalZeroConeBlocks(s.data());
    shiftToInteriorCold(s);
    shiftToInteriorCold(z);
    tau = 1.0;
    kappa = 1.0;
    return allFinite(x) && allFinite(s) && allFinite(z);
  }

  bool refactorize() {
    cones.updateScaling(s.data(), z.data());
    return kkt.updateScalingAndFactorize(cones);
  }

  bool constantSolve() {
    Vec rhs((size_t)(n + m)), sol;
    for (int i = 0; i < n; ++i) rhs[(size_t)i] = -q[(size_t)i];
    for (int i = 0; i < m; ++i) rhs[(size_t)(n + i)] = b[(size_t)i];
    kktSolve(rhs, sol);
    x1.assign(sol.begin(), sol.begin() + n);
    z1.assign(sol.begin() + n, sol.end());
    pmul(x1.data(), Px1.data());
    return allFinite(x1) && allFinite(z1);
  }

  void residuals() {
    pmul(x.data(), Px.data());
    Vec Atz((size_t)n, 0.0), Ax((size_t)m, 0.0);
    for (int c = 0; c < A.cols; ++c)
      for (int k = A.p[(size_t)c]; k < A.p[(size_t)c + 1]; ++k) {
        Atz[(size_t)c] += A.x[(size_t)k] * z[(size_t)A.i[(size_t)k]];
        Ax[(size_t)A.i[(size_t)k]] += A.x[(size_t)k] * x[(size_t)c];
      }
    for (int i = 0; i < n; ++i) rx[(size_t)i] = -Atz[(size_t)i] - Px[(size_t)i] - tau * q[(size_t)i];
    for (int i = 0; i < m; ++i) rz[(size_t)i] = Ax[(size_t)i] + s[(size_t)i] - tau * b[(size_t)i];
    dqx = dot(q.data(), x.data(), n);
    dbz = dot(b.data(), z.data(), m);
    dsz = dot(s.data(), z.data(), m);
    dxPx = dot(x.data(), Px.data(), n);
    rtau = dqx + dbz + kappa + dxPx / tau;
  }

  double mu() const { return (dsz + tau * kappa) / (double)(cones.degree + 1); }

  // Shared tau-elimination of the affine and combined steps (solver_impl.cpp:201-217,260-272).
  bool tauElim(const Vec& sol, double dtau_rhs, double dkappa_rhs, double& dt, Vec& dxo, Vec& dzo) {
    Vec xv(sol.begin(), sol.begin() + n), zv(sol.begin() + n, sol.end());
    if (!allFinite(xv) || !allFinite(zv)) return false;
    Vec xi((size_t)n), Pxv((size_t)n), xm((size_t)n), Pxm((size_t)n);
    for (int i = 0; i < n; ++i) xi[(size_t)i] = x[(size_t)i] / tau;
    pmul(xv.data(), Pxv.data());
    const double tau_num = dtau_rhs - dkappa_rhs / tau + dot(q.data(), xv.data(), n) +
                           dot(b.data(), zv.data(), m) + 2.0 * dot(xi.data(), Pxv.data(), n);
    for (int i = 0; i < n; ++i) xm[(size_t)i] = xi[(size_t)i] - x1[(size_t)i];
    pmul(xm.data(), Pxm.data());
    const double tau_den = kappa / tau - dot(q.data(), x1.data(), n) - dot(b.data(), z1.data(), m) +
                           dot(xm.data(), Pxm.data(), n) - dot(x1.data(), Px1.data(), n);
    if (tau_den == 0.0 || !std::isfinite(tau_num) || !std::isfinite(tau_den)) return false;
    dt = tau_num / tau_den;
    for (int i = 0; i < n; ++i) dxo[(size_t)i] = xv[(size_t)i] + dt * x1[(size_t)i];
    for (int i = 0; i < m; ++i) dzo[(size_t)i] = zv[(size_t)i] + dt * z1[(size_t)i];
    return true;
  }

  bool affineStep() {
    Vec rhs((size_t)(n + m)), sol;
    for (int i = 0; i < n; ++i) rhs[(size_t)i] = rx[(size_t)i];
    for (int i = 0; i < m; ++i) rhs[(size_t)(n + i)] = s[(size_t)i] - rz[(size_t)i];
    kktSolve(rhs, sol);
    const double dkrhs = tau * kappa;
    if (!tauElim(sol, rtau, dkrhs, dtaua, dxa, dza)) return false;
    Vec Hz((size_t)m);
    cones.mulHs(dza.data(), Hz.data());
    for (int i = 0; i < m; ++i) dsa[(size_t)i] = -(Hz[(size_t)i] + s[(size_t)i]);
    dkappaa = -(dkrhs + kappa * dtaua) / tau;
    return std::isfinite(dtaua) && std::isfinite(dkappaa) && allFinite(dxa) && allFinite(dza) &&
           allFinite(dsa);
  }

  bool combinedStep(double sigma, double muv) {
    Vec lambda((size_t)m), lp((size_t)m), wi((size_t)m), wd((size_t)m), corr((size_t)m),
        dsc((size_t)m), lid((size_t)m), dconst((size_t)m);
    cones.applyW(z.data(), lambda.data());
    cones.product(lambda.data(), lambda.data(), lp.data());
    cones.applyWInv(dsa.data(), wi.data());
    cones.applyW(dza.data(), wd.data());
    cones.product(wi.data(), wd.data(), corr.data());
    for (int i = 0; i < m; ++i) dsc[(size_t)i] = lp[(size_t)i] + corr[(size_t)i] - sigma * muv * cones.e[(size_t)i];
    cones.inverseProduct(lambda.data(), dsc.data(), lid.data());
    cones.applyW(lid.data(), dconst.data());
    Vec rhs((size_t)(n + m)), sol;
    for (int i = 0; i < n; ++i) rhs[(size_t)i] = (1.0 - sigma) * rx[(size_t)i];
    for (int i = 0; i < m; ++i) rhs[(size_t)(n + i)] = dconst[(size_t)i] - (1.0 - sigma) * rz[(size_t)i];
    kktSolve(rhs, sol);
    const double dtrhs = (1.0 - sigma) * rtau;
    const double dkrhs = tau * kappa + dtaua * dkappaa - sigma * muv;
    if (!tauElim(sol, dtrhs, dkrhs, dtau, dx, dz)) return false;
    Vec Hz((size_t)m);
    cones.mulHs(dz.data(), Hz.data());
    for (int i = 0; i < m; ++i) ds[(size_t)i] = -(Hz[(size_t)i] + dconst[(size_t)i]);
    dkappa = -(dkrhs + kappa * dtau) / tau;
    return std::isfinite(dtau) && std::isfinite(dkappa) && allFinite(dx) && allFinite(dz) && allFinite(ds);
  }

  double stepLength(const Vec& dsv, const Vec& dzv, double dt, double dk) const {
    double alpha = 1.0;
    if (dt < 0) alpha = std::min(alpha, -tau / dt);
    if (dk < 0) alpha = std::min(alpha, -kappa / dk);
    alpha = cones.maxStep(z.data(), dzv.data(), alpha);
    alpha = cones.maxStep(s.data(), dsv.data(), alpha);
    return alpha;
  }

  void finalize() {
    const bool infeas = status == CXG_STATUS_PRIMAL_INFEASIBLE || status == CXG_STATUS_DUAL_INFEASIBLE;
    const double scale = infeas ? 1.0 / std::max(kappa, 1e-30) : 1.0 / std::max(tau, 1e-30);
    solx = x; sols = s; solz = z;
    for (double& v : solx) v *= scale;
    for (double& v : sols) v *= scale;
    for (double& v : solz) v *= scale;
    if (st.equilibrate) eq.unscaleSolution(solx, sols, solz);
    double pobj = (0.5 * dxPx / tau + dqx) / tau;
    if (st.equilibrate) pobj /= eq.c;
    objective = pobj;
    double gap = dsz / (tau * tau);
    if (st.equilibrate) gap /= eq.c;
    info.duality_gap = gap;
    info.primal_residual = norm2(rz.data(), m) / std::max(tau, 1e-30);
    info.dual_residual = norm2(rx.data(), n) / std::max(tau, 1e-30);
    info.mu = mu();
  }

  // Adjoint of the KKT conditions at the last solution (new; no reference counterpart): one
  // extra KKT solve with the final factorisation and NT scaling,
  //   K [u; v] = [D dL/dx; 0]   (equilibrated space),
  // then dL/dq = -u, dL/db = v, dL/dP = -(u x' + x u'), dL/dA = -(z u' + v x'), mapped back
  // through the equilibration (x = D xh, P^ = c D P D, q^ = c D q, A^ = E A D, b^ = E b).
  bool adjoint(const double* dldx, double* dq, double* db, double* dPx, double* dAx) {
    if (status != CXG_STATUS_SOLVED) return false;
    const double* d = eq.d.data();
    const double* e = eq.e.data();
    const double cs = eq.c;
    Vec rhs((size_t)(n + m), 0.0), sol;
    for (int j = 0; j < n; ++j) rhs[(size_t)j] = d[j] * dldx[j];
    kkt.solve(rhs, sol);
    const double* u = sol.data();
    const double* v = sol.data() + n;
    Vec xh((size_t)n), zh((size_t)m);
    for (int j = 0; j < n; ++j) xh[(size_t)j] = x[(size_t)j] / tau;
    for (int r = 0; r < m; ++r) zh[(size_t)r] = z[(size_t)r] / tau;
    if (dq) for (int j = 0; j < n; ++j) dq[j] = -u[j] * (cs * d[j]);
    if (db) for (int r = 0; r < m; ++r) db[r] = v[r] * e[r];
    if (dPx) {
      for (int col = 0; col < P.cols; ++col)
        for (int k = P.p[(size_t)col]; k < P.p[(size_t)col + 1]; ++k) {
          const int r = P.i[(size_t)k];
          double g = 0.0;
          if (r == col) g = -u[r] * xh[(size_t)r];
          else if (r < col) g = -(u[r] * xh[(size_t)col] + u[col] * xh[(size_t)r]);
          dPx[k] = g * (cs * d[r] * d[col]);
        }
    }
    if (dAx) {
      for (int col = 0; col < A.cols; ++col)
        for (int k = A.p[(size_t)col]; k < A.p[(size_t)col + 1]; ++k) {
          const int r = A.i[(size_t)k];
          dAx[k] = -(zh[(size_t)r] * u[col] + v[r] * xh[(size_t)col]) * (e[r] * d[col]);
        }
    }
    return true;
  }

  void solve() {
    info = cxg_info{};
    trace.clear();
    kkt.faultFactorLeft = std::max(st.fault_factor_failures, 0);
    kkt.faultSolveLeft = std::max(st.fault_nonfinite_solves, 0);
    kkt.attemptsTotal = 0;
    kkt.escalationsTotal = 0;
    maxRel = 0;
    refineSteps = 0;
    status = CXG_STATUS_UNSOLVED;
    if (!setupDone) {
      status = CXG_STATUS_NUMERICAL_ERROR;
      info.status = status;
      return;
    }
    const bool useWarm = st.warm_start && haveWarm;
    if (useWarm) {
      x = wx; s = ws; z = wz;
      tau = 1.0; kappa = 1.0;
      cones.zeroPrimalZeroConeBlocks(s.data());
      ensureStrictlyInteriorWarm(s);
      ensureStrictlyInteriorWarm(z);
    } else if (!computeInitialPoint()) {
      status = CXG_STATUS_NUMERICAL_ERROR;
      finalize();
      info.status = status;
      info.objective = objective;
      info.factor_attempts = kkt.attemptsTotal;
      info.escalations = kkt.escalationsTotal;
      return;
    }
    int fin = CXG_STATUS_MAX_ITERATIONS;
    int iterations = 0;
    for (int iter = 0; iter < st.max_iter; ++iter) {
      iterations = iter + 1;
      TraceRow tr{};
      iterRel = 0;
      if (!refactorize() || !constantSolve()) { fin = CXG_STATUS_NUMERICAL_ERROR; tr.relres = iterRel; trace.push_back(tr); break; }
      tr.attempts = kkt.attemptsLast;
      residuals();
      const double muv = mu();
      const double nrx = norm2(rx.data(), n) / tau;
      const double nrz = norm2(rz.data(), m) / tau;
      const double pobj = (0.5 * dxPx / tau + dqx) / tau;
      const double dobj = (-0.5 * dxPx / tau - dbz) / tau;
      tr.mu = muv; tr.norm_rx = nrx; tr.norm_rz = nrz; tr.pobj = pobj; tr.dobj = dobj;
      tr.tau = tau; tr.kappa = kappa;
      const double gapAbs = std::abs(pobj - dobj);
      const double gapTol = st.tol_gap_abs + st.tol_gap_rel * std::max(std::abs(pobj), std::abs(dobj));
      if (nrx < st.tol_feas && nrz < st.tol_feas && gapAbs < gapTol && tau > 1e-6) {
        fin = CXG_STATUS_SOLVED;
        tr.relres = iterRel;
        trace.push_back(tr);
        break;
      }
      const double ratio = tau / std::max(kappa, 1e-30);
      if (ratio <= st.tol_infeas) {
        if (dbz < -st.tol_infeas * std::max(1.0, norm2(z.data(), m))) {
          fin = CXG_STATUS_PRIMAL_INFEASIBLE;
          status = fin;
          tr.relres = iterRel; trace.push_back(tr);
          break;
        }
        if (dqx < -st.tol_infeas * std::max(1.0, norm2(x.data(), n))) {
          fin = CXG_STATUS_DUAL_INFEASIBLE;
          status = fin;
          tr.relres = iterRel; trace.push_back(tr);
          break;
        }
      }
      if (!affineStep()) { fin = CXG_STATUS_NUMERICAL_ERROR; tr.relres = iterRel; trace.push_back(tr); break; }
      const double aaff = stepLength(dsa, dza, dtaua, dkappaa);
      double szaff = 0;
      for (int i = 0; i < m; ++i) szaff += (s[(size_t)i] + aaff * dsa[(size_t)i]) * (z[(size_t)i] + aaff * dza[(size_t)i]);
      const double taff = tau + aaff * dtaua, kaff = kappa + aaff * dkappaa;
      const double muaff = (szaff + taff * kaff) / (double)(cones.degree + 1);
      double sigma;
      if (muv > 0) {
        const double r = std::max(muaff / muv, 0.0);
        sigma = std::min(std::max(r * r * r, 0.0), 1.0);
      } else {
        sigma = 1.0;
      }
      tr.alpha_aff = aaff; tr.sigma = sigma;
      if (!combinedStep(sigma, muv)) { fin = CXG_STATUS_NUMERICAL_ERROR; tr.relres = iterRel; trace.push_back(tr); break; }
      const double alpha = stepLength(ds, dz, dtau, dkappa) * st.max_step_fraction;
      tr.alpha = alpha;
      tr.relres = iterRel;
      trace.push_back(tr);
      if (!std::isfinite(alpha) || alpha <= 0.0) { fin = CXG_STATUS_NUMERICAL_ERROR; break; }
      for (int i = 0; i < n; ++i) x[(size_t)i] += alpha * dx[(size_t)i];
      for (int i = 0; i < m; ++i) { s[(size_t)i] += alpha * ds[(size_t)i]; z[(size_t)i] += alpha * dz[(size_t)i]; }
      tau += alpha * dtau;
      kappa += alpha * dkappa;
      const double sc = std::max(tau, kappa);
      if (sc > 1e8 || sc < 1e-8) {
        const double inv = 1.0 / sc;
        for (double& v : x) v *= inv;
        for (double& v : s) v *= inv;
        for (double& v : z) v *= inv;
        tau *= inv;
        kappa *= inv;
      }
    }
    status = fin;
    info.iterations = iterations;
    finalize();
    info.status = status;
    info.objective = objective;
    info.max_relres = maxRel;
    info.refine_steps = refineSteps;
    info.factor_attempts = kkt.attemptsTotal;
    info.escalations = kkt.escalationsTotal;
    if (fin == CXG_STATUS_SOLVED && st.warm_start) {
      wx = x; ws = s; wz = z;
      haveWarm = true;
    }
  }
};

}  // namespace orc

// ==========================================================================================
// C API (ctypes)
// ==========================================================================================
extern "C" {

void* orc_create(void) { return new orc::Solver(); }
void orc_destroy(void* h) { delete static_cast<orc::Solver*>(h); }

int orc_setup(void* h, const cxg_problem* pr, const cxg_settings* st) {
  return static_cast<orc::Solver*>(h)->setup(*pr, *st) ? 1 : 0;
}

int orc_update(void* h, const int* Pp, const int* Pi, const double* Px, const double* q,
               const int* Ap, const int* Ai, const double* Ax, const double* b) {
  auto* S = static_cast<orc::Solver*>(h);
  if (!S->setupDone) return 0;
  orc::Csc P, A;
  orc::Vec qv, bv;
  if (Px) P = orc::makeCsc(S->n, S->n, Pp, Pi, Px);
  if (Ax) A = orc::makeCsc(S->m, S->n, Ap, Ai, Ax);
  if (q) qv.assign(q, q + S->n);
  if (b) bv.assign(b, b + S->m);
  return S->updateData(Px ? &P : nullptr, q ? &qv : nullptr, Ax ? &A : nullptr, b ? &bv : nullptr) ? 1 : 0;
}

void orc_set_warm_start(void* h, const double* x, const double* s, const double* z) {
  static_cast<orc::Solver*>(h)->setWarmStart(x, s, z);
}

int orc_solve(void* h, double* x, double* s, double* z, cxg_info* info) {
  auto* S = static_cast<orc::Solver*>(h);
  S->solve();
  if (x && !S->solx.empty()) std::memcpy(x, S->solx.data(), sizeof(double) * S->solx.size());
  if (s && !S->sols.empty()) std::memcpy(s, S->sols.data(), sizeof(double) * S->sols.size());
  if (z && !S->solz.empty()) std::memcpy(z, S->solz.data(), sizeof(double) * S->solz.size());
  if (info) *info = S->info;
  return S->status;
}

int orc_adjoint(void* h, const double* dldx, double* dq, double* db, double* dPx, double* dAx) {
  return static_cast<orc::Solver*>(h)->adjoint(dldx, dq, db, dPx, dAx) ? 1 : 0;
}

int orc_trace_len(void* h) { return (int)static_cast<orc::Solver*>(h)->trace.size(); }
int orc_trace_cols(void) { return orc::kTraceCols; }
void orc_trace(void* h, double* out) {
  auto* S = static_cast<orc::Solver*>(h);
  for (size_t t = 0; t < S->trace.size(); ++t) std::memcpy(out + t * orc::kTraceCols, &S->trace[t], sizeof(orc::TraceRow));
}

// Equilibrated (scaled) problem data and scaling factors, for host-logic parity tests.
void orc_equilibration(void* h, double* d, double* e, double* c) {
  auto* S = static_cast<orc::Solver*>(h);
  if (d) std::memcpy(d, S->eq.d.data(), sizeof(double) * S->eq.d.size());
  if (e) std::memcpy(e, S->eq.e.data(), sizeof(double) * S->eq.e.size());
  if (c) *c = S->eq.c;
}

int orc_nnz_l(void* h) { return static_cast<orc::Solver*>(h)->kkt.ldl.nnzL(); }

// --- KKT layer (kkt_system.cpp), for the reference's KKT known-answer tests ----------------
// Sets up the KKT of (P, A, cones) with equilibration off, optionally rescales with (s, z),
// then solves K x = rhs with refinement. Returns the relative residual, or -1 on failure.
double orc_kkt_solve(const cxg_problem* pr, const cxg_settings* st, const double* s, const double* z,
                     const double* rhs, double* out) {
  orc::Cones cones;
  std::vector<int> socd(pr->soc_dims, pr->soc_dims + pr->n_soc);
  cones.build(pr->zero_dim, pr->nonneg_dim, socd);
  orc::Csc P = orc::makeCsc(pr->n, pr->n, pr->Pp, pr->Pi, pr->Px);
  orc::Csc A = orc::makeCsc(pr->m, pr->n, pr->Ap, pr->Ai, pr->Ax);
  orc::Kkt kkt;
  if (!kkt.setup(P, A, cones, *st)) return -1.0;
  if (s && z) {
    cones.updateScaling(s, z);
    if (!kkt.updateScalingAndFactorize(cones)) return -1.0;
  }
  orc::Vec r(rhs, rhs + pr->n + pr->m), x;
  const double rel = kkt.solve(r, x);
  std::memcpy(out, x.data(), sizeof(double) * x.size());
  return rel;
}

// --- cone layer (cone_set.cpp and the three cone classes) ---------------------------------
void* orc_cones_create(int zero, int nn, int nsoc, const int* dims) {
  auto* C = new orc::Cones();
  C->build(zero, nn, std::vector<int>(dims, dims + nsoc));
  return C;
}
void orc_cones_destroy(void* h) { delete static_cast<orc::Cones*>(h); }
int orc_cones_dim(void* h) { return static_cast<orc::Cones*>(h)->m; }
int orc_cones_degree(void* h) { return static_cast<orc::Cones*>(h)->degree; }
void orc_cones_identity(void* h, double* out) {
  auto* C = static_cast<orc::Cones*>(h);
  std::memcpy(out, C->e.data(), sizeof(double) * C->e.size());
}
void orc_cones_update_scaling(void* h, const double* s, const double* z) {
  static_cast<orc::Cones*>(h)->updateScaling(s, z);
}
// op: 0 product(u,v), 1 inverseProduct(u,v), 2 applyW(u), 3 applyWInv(u), 4 mulHs(u)
void orc_cones_apply(void* h, int op, const double* u, const double* v, double* out) {
  auto* C = static_cast<orc::Cones*>(h);
  switch (op) {
    case 0: C->product(u, v, out); break;
    case 1: C->inverseProduct(u, v, out); break;
    case 2: C->applyW(u, out); break;
    case 3: C->applyWInv(u, out); break;
    default: C->mulHs(u, out); break;
  }
}
double orc_cones_max_step(void* h, const double* x, const double* dx, double amax) {
  return static_cast<orc::Cones*>(h)->maxStep(x, dx, amax);
}
void orc_cones_margins(void* h, const double* x, double* mn, double* pos) {
  auto r = static_cast<orc::Cones*>(h)->margins(x);
  *mn = r.first;
  *pos = r.second;
}
void orc_cones_shift(void* h, double* x, double alpha) { static_cast<orc::Cones*>(h)->scaledUnitShift(x, alpha); }
// Dense W and Hs of every SOC block, concatenated (dim*dim each, row-major); NN w per row.
void orc_cones_scaling(void* h, double* nn_w, double* soc_W, double* soc_Hs) {
  auto* C = static_cast<orc::Cones*>(h);
  if (nn_w) std::memcpy(nn_w, C->nn_w.data(), sizeof(double) * C->nn_w.size());
  size_t off = 0;
  for (size_t b = 0; b < C->blocks.size(); ++b) {
    if (C->blocks[b].type != orc::kSoc) continue;
    const size_t dd = (size_t)C->blocks[b].dim * C->blocks[b].dim;
    if (soc_W) std::memcpy(soc_W + off, C->W[b].data(), sizeof(double) * dd);
    if (soc_Hs) std::memcpy(soc_Hs + off, C->Hs[b].data(), sizeof(double) * dd);
    off += dd;
  }
}

// --- CPU baseline: solve `count` independent instances with `nthreads` threads (one solver
// per instance, instances handed out by an atomic counter). Setup happens before the timed
// region. Returns the wall time of the solve phase in seconds.
double orc_batch_solve_x(int count, const cxg_problem* problems, const cxg_settings* st, int nthreads,
                         int* statuses, int* iterations, double* x, double* s, double* z);

double orc_batch_solve(int count, const cxg_problem* problems, const cxg_settings* st, int nthreads,
                       int* statuses, int* iterations) {
  return orc_batch_solve_x(count, problems, st, nthreads, statuses, iterations, nullptr, nullptr, nullptr);
}

// As orc_batch_solve, and (outside the timed region) the solutions concatenated in instance order
// into x (sum of n), s and z (sum of m) when those are non-null.
double orc_batch_solve_x(int count, const cxg_problem* problems, const cxg_settings* st, int nthreads,
                         int* statuses, int* iterations, double* x, double* s, double* z) {
  std::vector<std::unique_ptr<orc::Solver>> solvers((size_t)count);
  for (int i = 0; i < count; ++i) {
    solvers[(size_t)i] = std::make_unique<orc::Solver>();
    if (!solvers[(size_t)i]->setup(problems[i], *st)) solvers[(size_t)i].reset();
  }
  std::atomic<int> next{0};
  auto work = [&]() {
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= count) break;
      if (!solvers[(size_t)i]) { if (statuses) statuses[i] = -1; continue; }
      solvers[(size_t)i]->solve();
      if (statuses) statuses[i] = solvers[(size_t)i]->status;
      if (iterations) iterations[i] = solvers[(size_t)i]->info.iterations;
    }
  };
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  for (int t = 0; t < std::max(1, nthreads); ++t) th.emplace_back(work);
  for (auto& t : th) t.join();
  const auto t1 = std::chrono::steady_clock::now();
  if (x && s && z) {
    size_t on = 0, om = 0;
    for (int i = 0; i < count; ++i) {
      const size_t n = (size_t)problems[i].n, m = (size_t)problems[i].m;
      const orc::Solver* S = solvers[(size_t)i].get();
      if (S && S->solx.size() == n && S->sols.size() == m && S->solz.size() == m) {
        std::memcpy(x + on, S->solx.data(), sizeof(double) * n);
        std::memcpy(s + om, S->sols.data(), sizeof(double) * m);
        std::memcpy(z + om, S->solz.data(), sizeof(double) * m);
      }
      on += n;
      om += m;
    }
  }
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
