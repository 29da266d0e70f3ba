// conicxx_gb300.hpp -- C++ API of the GB300 interior-point path with ConicXX's names, so that
// code written against ConicXX's Solver (include/conicxx/solver.h:33-95), ConeSpec
// (include/conicxx/cone_spec.h:15-33), Settings (include/conicxx/settings.h:21-62) and Solution
// (include/conicxx/solution.h:9-39) compiles against this header and links
// libconicxx_gb300.so instead.
//
// Header-only; everything goes through the C-ABI in conicxx_gb300.h. No exception is thrown by
// the solver calls: setup()/updateData() return false on any error (cxg_last_error() has the
// message) and solve() always returns a Solution with a definite Status, NumericalError when
// called before a successful setup() -- as the reference does (src/conicxx/solver_impl.cpp:367-372).
//
// Types. ConicXX uses Eigen (include/conicxx/types.h:8-19). Define CONICXX_GB300_WITH_EIGEN
// before including this header to use Eigen's types under the same names. Otherwise small
// stand-ins are provided. Each carries the Eigen members this API reads: SparseMat
// (rows/cols/nonZeros/outerIndexPtr/innerIndexPtr/valuePtr, setFromTriplets), Vec
// (size/data/operator[]/operator()) and Mat (rows/cols/operator()(i, j)), so caller code that uses
// only those members compiles unchanged with either.
#ifndef CONICXX_GB300_HPP
#define CONICXX_GB300_HPP

#include <cmath>
#include <cstdio>
#include <initializer_list>
#include <map>
#include <utility>
#include <vector>

#include "conicxx_gb300.h"

#ifdef CONICXX_GB300_WITH_EIGEN
#include <Eigen/Core>
#include <Eigen/SparseCore>
#endif

namespace conicxx {

using Scalar = double;
using Index = int;

#ifdef CONICXX_GB300_WITH_EIGEN
using Vec = Eigen::VectorXd;
using Mat = Eigen::MatrixXd;
using SparseMat = Eigen::SparseMatrix<Scalar, Eigen::ColMajor, Index>;
using Triplet = Eigen::Triplet<Scalar, Index>;
#else
class Vec {
 public:
  Vec() = default;
  explicit Vec(Index n) : v_((size_t)n, 0.0) {}
  Vec(std::initializer_list<Scalar> init) : v_(init) {}
  Index size() const { return (Index)v_.size(); }
  void resize(Index n) { v_.assign((size_t)n, 0.0); }
  Scalar* data() { return v_.data(); }
  const Scalar* data() const { return v_.data(); }
  Scalar& operator[](Index i) { return v_[(size_t)i]; }
  Scalar operator[](Index i) const { return v_[(size_t)i]; }
  Scalar& operator()(Index i) { return v_[(size_t)i]; }
  Scalar operator()(Index i) const { return v_[(size_t)i]; }
  static Vec Zero(Index n) { return Vec(n); }

 private:
  std::vector<Scalar> v_;
};

// Dense column-major matrix.
class Mat {
 public:
  Mat() = default;
  Mat(Index rows, Index cols) : r_(rows), c_(cols), v_((size_t)rows * (size_t)cols, 0.0) {}
  Index rows() const { return r_; }
  Index cols() const { return c_; }
  Scalar& operator()(Index i, Index j) { return v_[(size_t)j * (size_t)r_ + (size_t)i]; }
  Scalar operator()(Index i, Index j) const { return v_[(size_t)j * (size_t)r_ + (size_t)i]; }
  static Mat Zero(Index rows, Index cols) { return Mat(rows, cols); }

 private:
  Index r_ = 0, c_ = 0;
  std::vector<Scalar> v_;
};

struct Triplet {
  Triplet(Index r, Index c, Scalar v) : r_(r), c_(c), v_(v) {}
  Index row() const { return r_; }
  Index col() const { return c_; }
  Scalar value() const { return v_; }
  Index r_, c_;
  Scalar v_;
};

// Compressed sparse column matrix with 32-bit indices, rows sorted within each column.
class SparseMat {
 public:
  SparseMat() = default;
  SparseMat(Index rows, Index cols) : r_(rows), c_(cols), p_((size_t)cols + 1, 0) {}
  Index rows() const { return r_; }
  Index cols() const { return c_; }
  Index nonZeros() const { return (Index)x_.size(); }
  bool isCompressed() const { return true; }
  const Index* outerIndexPtr() const { return p_.data(); }
  const Index* innerIndexPtr() const { return i_.data(); }
  const Scalar* valuePtr() const { return x_.data(); }
  Index* outerIndexPtr() { return p_.data(); }
  Index* innerIndexPtr() { return i_.data(); }
  Scalar* valuePtr() { return x_.data(); }
  // Duplicates are summed (Eigen's setFromTriplets semantics).
  template <typename It>
  void setFromTriplets(It begin, It end) {
    std::map<std::pair<Index, Index>, Scalar> acc;  // (col, row) -> value
    for (It t = begin; t != end; ++t) acc[{t->col(), t->row()}] += t->value();
    p_.assign((size_t)c_ + 1, 0);
    i_.clear();
    x_.clear();
    for (const auto& kv : acc) {
      ++p_[(size_t)kv.first.first + 1];
      i_.push_back(kv.first.second);
      x_.push_back(kv.second);
    }
    for (Index j = 0; j < c_; ++j) p_[(size_t)j + 1] += p_[(size_t)j];
  }

 private:
  Index r_ = 0, c_ = 0;
  std::vector<Index> p_{0}, i_;
  std::vector<Scalar> x_;
};
#endif

// ConeSpec (include/conicxx/cone_spec.h:15-33): Zero rows, then Nonnegative, then SOC blocks.
struct ConeSpec {
  Index zero_dim = 0;
  Index nonneg_dim = 0;
  std::vector<Index> soc_dims;
  Index totalDim() const {
    Index t = zero_dim + nonneg_dim;
    for (Index d : soc_dims) t += d;
    return t;
  }
  bool isValid() const {
    if (zero_dim < 0 || nonneg_dim < 0) return false;
    for (Index d : soc_dims)
      if (d < 1) return false;
    return true;
  }
};

// LinearSolverBackend (include/conicxx/settings.h:8-18). On the device all three select the
// same factorisation; RegularizedLdlt adds the per-pivot correction rule.
enum class LinearSolverBackend { Eigen, Qdldl, RegularizedLdlt };

// Arithmetic of the KKT factorisation (GB300 addition).
enum class Precision { FP64, Mixed };

// Settings (include/conicxx/settings.h:21-62): same fields and defaults, then the GB300 additions.
struct Settings {
  Scalar tol_feas = 1e-8;
  Scalar tol_gap_abs = 1e-8;
  Scalar tol_gap_rel = 1e-8;
  Scalar tol_infeas = 1e-7;
  int max_iter = 200;
  Scalar static_reg_P = 1e-8;
  Scalar static_reg_A = 1e-8;
  Scalar dynamic_reg_eps = 1e-14;
  Scalar dynamic_reg_delta = 1e-7;
  int refine_max_iter = 3;
  Scalar refine_tol = 1e-12;
  Scalar max_step_fraction = 0.99;
  bool equilibrate = true;
  int equilibrate_max_iter = 10;
  Scalar equilibrate_min_scale = 1e-4;
  Scalar equilibrate_max_scale = 1e4;
  bool warm_start = true;
  int verbose = 0;
  bool record_timings = false;
  bool validate_inputs = true;
  LinearSolverBackend linear_solver = LinearSolverBackend::Qdldl;
  // ---- GB300 additions ----
  Precision precision = Precision::FP64;
  int mixed_refine_max_iter = 4;
  Scalar mixed_fallback_tol = 1e-10;
  int threads_per_instance = 0;
  bool differentiable = true;  // keep the final factorisation for backward()
  int whole_gpu_root = 0;      // 0 automatic (roots above 512 rows use every SM), 1 always, -1 never
  bool soc_reference_dense = true;  // SOC pivot test and Hs products in the reference's dense form
};

// Status / Info / Solution (include/conicxx/solution.h:9-39).
enum class Status { Unsolved, Solved, PrimalInfeasible, DualInfeasible, MaxIterations, NumericalError };

inline const char* toString(Status s) { return cxg_status_string((int)s); }

struct Info {
  int iterations = 0;
  Scalar primal_residual = 0;
  Scalar dual_residual = 0;
  Scalar duality_gap = 0;
  Scalar mu = 0;
  Scalar setup_time_s = 0;
  Scalar solve_time_s = 0;
  // ---- GB300 additions ----
  int fp64_fallbacks = 0;
  int refine_steps = 0;
  Scalar max_relres = 0;
};

struct Solution {
  Status status = Status::Unsolved;
  Vec x;
  Vec s;
  Vec z;
  Scalar objective = 0;
  Info info;
  bool ok() const { return status == Status::Solved; }
};

// dL/d(problem data) from Solver::backward (GB300 addition): dq (n), db (m), and the gradients
// with respect to the stored values of P (upper, setup CSC order) and of A (setup CSC order).
struct Gradients {
  Vec dq, db, dP, dA;
};

// Last error message of the calling thread (the C-ABI's cxg_last_error).
inline const char* lastError() { return cxg_last_error(); }

// Dense -> CSC keeping every entry, including exact zeros, so the pattern never depends on the
// values (conicxx::toSparse, include/conicxx/convert.h:12-30).
inline SparseMat toSparse(const Mat& dense, const char* name = nullptr, bool warn = true) {
  static bool warned = false;
  if (warn && !warned) {
    std::fprintf(stderr, "conicxx_gb300: dense %s converted to sparse (every entry kept)\n", name ? name : "matrix");
    warned = true;
  }
  std::vector<Triplet> t;
  for (Index j = 0; j < dense.cols(); ++j)
    for (Index i = 0; i < dense.rows(); ++i) t.emplace_back(i, j, dense(i, j));
  SparseMat S(dense.rows(), dense.cols());
  S.setFromTriplets(t.begin(), t.end());
  return S;
}

// Upper triangle (with the diagonal) of a dense symmetric matrix (toSparseUpperTriangular,
// include/conicxx/convert.h:32-40).
inline SparseMat toSparseUpperTriangular(const Mat& sym, const char* name = nullptr, bool warn = true) {
  static bool warned = false;
  if (warn && !warned) {
    std::fprintf(stderr, "conicxx_gb300: dense %s converted to sparse upper triangle\n", name ? name : "matrix");
    warned = true;
  }
  std::vector<Triplet> t;
  for (Index j = 0; j < sym.cols(); ++j)
    for (Index i = 0; i <= j && i < sym.rows(); ++i) t.emplace_back(i, j, sym(i, j));
  SparseMat S(sym.rows(), sym.cols());
  S.setFromTriplets(t.begin(), t.end());
  return S;
}

namespace detail {
inline cxg_settings toC(const Settings& s) {
  cxg_settings c;
  cxg_default_settings(&c);
  c.tol_feas = s.tol_feas;
  c.tol_gap_abs = s.tol_gap_abs;
  c.tol_gap_rel = s.tol_gap_rel;
  c.tol_infeas = s.tol_infeas;
  c.max_iter = s.max_iter;
  c.static_reg_P = s.static_reg_P;
  c.static_reg_A = s.static_reg_A;
  c.dynamic_reg_eps = s.dynamic_reg_eps;
  c.dynamic_reg_delta = s.dynamic_reg_delta;
  c.refine_max_iter = s.refine_max_iter;
  c.refine_tol = s.refine_tol;
  c.max_step_fraction = s.max_step_fraction;
  c.equilibrate = s.equilibrate ? 1 : 0;
  c.equilibrate_max_iter = s.equilibrate_max_iter;
  c.equilibrate_min_scale = s.equilibrate_min_scale;
  c.equilibrate_max_scale = s.equilibrate_max_scale;
  c.warm_start = s.warm_start ? 1 : 0;
  c.verbose = s.verbose;
  c.record_timings = s.record_timings ? 1 : 0;
  c.validate_inputs = s.validate_inputs ? 1 : 0;
  c.linear_solver = s.linear_solver == LinearSolverBackend::Eigen       ? CXG_LINSOLVER_EIGEN
                    : s.linear_solver == LinearSolverBackend::Qdldl     ? CXG_LINSOLVER_QDLDL
                                                                        : CXG_LINSOLVER_REGULARIZED;
  c.precision = s.precision == Precision::Mixed ? CXG_PRECISION_MIXED : CXG_PRECISION_FP64;
  c.mixed_refine_max_iter = s.mixed_refine_max_iter;
  c.mixed_fallback_tol = s.mixed_fallback_tol;
  c.threads_per_instance = s.threads_per_instance;
  c.differentiable = s.differentiable ? 1 : 0;
  c.whole_gpu_root = s.whole_gpu_root;
  c.fault_factor_failures = 0;
  c.fault_nonfinite_solves = 0;
  c.soc_reference_dense = s.soc_reference_dense ? 1 : 0;
  return c;
}
}  // namespace detail

// Solver (include/conicxx/solver.h:33-95): owns copies of all data (on the device), move-only,
// not thread-safe; independent instances may be used from different host threads.
class Solver {
 public:
  Solver() { cxg_solver_create(&h_); }
  ~Solver() {
    if (h_) cxg_solver_destroy(h_);
  }
  Solver(Solver&& o) noexcept { swap(o); }
  Solver& operator=(Solver&& o) noexcept {
    if (this != &o) {
      Solver tmp(std::move(o));
      swap(tmp);
    }
    return *this;
  }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  // Structural setup; false on invalid input or a device error (never throws).
  bool setup(const SparseMat& P, const Vec& q, const SparseMat& A, const Vec& b, const ConeSpec& cone,
             const Settings& settings = Settings{}) {
    if (!h_) return false;
    ok_ = false;
    settings_ = settings;
    if (!cone.isValid() || P.rows() != P.cols() || A.cols() != P.cols() || q.size() != P.cols() ||
        b.size() != A.rows() || cone.totalDim() != A.rows())
      return false;
    cxg_problem pr{};
    pr.n = (int)P.cols();
    pr.m = (int)A.rows();
    pr.Pp = P.outerIndexPtr();
    pr.Pi = P.innerIndexPtr();
    pr.Px = P.valuePtr();
    pr.q = q.data();
    pr.Ap = A.outerIndexPtr();
    pr.Ai = A.innerIndexPtr();
    pr.Ax = A.valuePtr();
    pr.b = b.data();
    pr.zero_dim = cone.zero_dim;
    pr.nonneg_dim = cone.nonneg_dim;
    pr.n_soc = (int)cone.soc_dims.size();
    pr.soc_dims = cone.soc_dims.empty() ? nullptr : cone.soc_dims.data();
    const cxg_settings cs = detail::toC(settings);
    if (cxg_solver_setup(h_, &pr, &cs) != CXG_OK) return false;
    n_ = pr.n;
    m_ = pr.m;
    nnzP_ = P.nonZeros();
    nnzA_ = A.nonZeros();
    ok_ = true;
    return true;
  }
  bool setup(const Mat& P, const Vec& q, const SparseMat& A, const Vec& b, const ConeSpec& cone,
             const Settings& settings = Settings{}) {
    return setup(toSparseUpperTriangular(P, "P"), q, A, b, cone, settings);
  }
  bool setup(const SparseMat& P, const Vec& q, const Mat& A, const Vec& b, const ConeSpec& cone,
             const Settings& settings = Settings{}) {
    return setup(P, q, toSparse(A, "A"), b, cone, settings);
  }
  bool setup(const Mat& P, const Vec& q, const Mat& A, const Vec& b, const ConeSpec& cone,
             const Settings& settings = Settings{}) {
    return setup(toSparseUpperTriangular(P, "P"), q, toSparse(A, "A"), b, cone, settings);
  }

  // Values-only update; nullptr = unchanged. false if a pattern differs from setup() (the caller
  // then calls setup() again) or on any other error.
  bool updateData(const SparseMat* P, const Vec* q, const SparseMat* A, const Vec* b) {
    if (!h_ || !ok_) return false;
    if ((q && q->size() != n_) || (b && b->size() != m_)) return false;
    return cxg_solver_update_data(h_, P ? P->outerIndexPtr() : nullptr, P ? P->innerIndexPtr() : nullptr,
                                  P ? P->valuePtr() : nullptr, q ? q->data() : nullptr,
                                  A ? A->outerIndexPtr() : nullptr, A ? A->innerIndexPtr() : nullptr,
                                  A ? A->valuePtr() : nullptr, b ? b->data() : nullptr) == CXG_OK;
  }

  // Seed the next solve() with (x, s, z) in original problem units; after setup().
  void setWarmStart(const Vec& x, const Vec& s, const Vec& z) {
    if (h_ && ok_ && x.size() == n_ && s.size() == m_ && z.size() == m_)
      cxg_solver_set_warm_start(h_, x.data(), s.data(), z.data());
  }

  void setSettings(const Settings& settings) {
    settings_ = settings;
    if (h_) {
      const cxg_settings cs = detail::toC(settings);
      cxg_solver_set_settings(h_, &cs);
    }
  }
  const Settings& settings() const { return settings_; }

  const Solution& solve() {
    sol_ = Solution{};
    if (!h_ || !ok_) {
      sol_.status = Status::NumericalError;
      return sol_;
    }
    sol_.x.resize(n_);
    sol_.s.resize(m_);
    sol_.z.resize(m_);
    cxg_info info{};
    if (cxg_solver_solve(h_, sol_.x.data(), sol_.s.data(), sol_.z.data(), &info) != CXG_OK) {
      sol_.status = Status::NumericalError;
      return sol_;
    }
    sol_.status = (Status)info.status;
    sol_.objective = info.objective;
    sol_.info.iterations = info.iterations;
    sol_.info.primal_residual = info.primal_residual;
    sol_.info.dual_residual = info.dual_residual;
    sol_.info.duality_gap = info.duality_gap;
    sol_.info.mu = info.mu;
    sol_.info.setup_time_s = info.setup_time_s;
    sol_.info.solve_time_s = info.solve_time_s;
    sol_.info.fp64_fallbacks = info.fp64_fallbacks;
    sol_.info.refine_steps = info.refine_steps;
    sol_.info.max_relres = info.max_relres;
    return sol_;
  }
  const Solution& solution() const { return sol_; }

  // GB300 addition: dL/d(q, b, values of P, values of A) at the last Solved solution, by one
  // extra KKT solve with the final factorisation. Needs Settings::differentiable (default on).
  bool backward(const Vec& dL_dx, Gradients* out) {
    if (!h_ || !ok_ || !out || dL_dx.size() != n_) return false;
    out->dq.resize(n_);
    out->db.resize(m_);
    out->dP.resize(nnzP_);
    out->dA.resize(nnzA_);
    return cxg_solver_backward(h_, dL_dx.data(), out->dq.data(), out->db.data(), out->dP.data(),
                               out->dA.data()) == CXG_OK;
  }

 private:
  void swap(Solver& o) noexcept {
    std::swap(h_, o.h_);
    std::swap(ok_, o.ok_);
    std::swap(n_, o.n_);
    std::swap(m_, o.m_);
    std::swap(nnzP_, o.nnzP_);
    std::swap(nnzA_, o.nnzA_);
    std::swap(settings_, o.settings_);
    std::swap(sol_, o.sol_);
  }
  cxg_solver* h_ = nullptr;
  bool ok_ = false;
  Index n_ = 0, m_ = 0, nnzP_ = 0, nnzA_ = 0;
  Settings settings_;
  Solution sol_;
};

}  // namespace conicxx

#endif  // CONICXX_GB300_HPP
