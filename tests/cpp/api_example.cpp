// Caller-side program written against ConicXX's C++ API names (include/conicxx/solver.h), built
// against conicxx_gb300.hpp and libconicxx_gb300.so by tests/test_cpp_api.py.
//   api_example host  -- checks that need no GPU: defaults, ConeSpec, invalid input, solve before setup
//   api_example gpu   -- the README example (README.md:84-123 of ConicXX), updateData, warm start, backward
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "conicxx_gb300.hpp"

using namespace conicxx;

static int failures = 0;
#define CHECK(cond)                                                   \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::printf("CHECK failed line %d: %s\n", __LINE__, #cond);     \
      ++failures;                                                     \
    }                                                                 \
  } while (0)

static SparseMat sparse(Index r, Index c, const std::vector<Triplet>& t) {
  SparseMat S(r, c);
  S.setFromTriplets(t.begin(), t.end());
  return S;
}

// ConicXX's README example (README.md:84-123): min 1/2|x|^2 - x0 - x1 - 0.3 t subject to
// x0 + x1 = 1 (Zero), t >= 0 (Nonnegative), ||(x0, x1)|| <= t (SOC of dimension 3);
// solution x = (0.5, 0.5, sqrt(0.5)).
static void readme_problem(SparseMat& P, Vec& q, SparseMat& A, Vec& b, ConeSpec& cone) {
  P = sparse(3, 3, {Triplet(0, 0, 1.0), Triplet(1, 1, 1.0), Triplet(2, 2, 1.0)});
  q = Vec{-1.0, -1.0, -0.3};
  A = sparse(5, 3, {Triplet(0, 0, 1.0), Triplet(0, 1, 1.0), Triplet(1, 2, -1.0), Triplet(2, 2, -1.0),
                    Triplet(3, 0, -1.0), Triplet(4, 1, -1.0)});
  b = Vec{1.0, 0.0, 0.0, 0.0, 0.0};
  cone = ConeSpec{};
  cone.zero_dim = 1;
  cone.nonneg_dim = 1;
  cone.soc_dims = {3};
}

static int host_checks() {
  Settings st;
  CHECK(st.tol_feas == 1e-8 && st.tol_gap_abs == 1e-8 && st.tol_gap_rel == 1e-8 && st.tol_infeas == 1e-7);
  CHECK(st.max_iter == 200 && st.refine_max_iter == 3 && st.refine_tol == 1e-12);
  CHECK(st.static_reg_P == 1e-8 && st.static_reg_A == 1e-8 && st.dynamic_reg_eps == 1e-14 &&
        st.dynamic_reg_delta == 1e-7);
  CHECK(st.max_step_fraction == 0.99 && st.equilibrate && st.equilibrate_max_iter == 10 && st.warm_start);
  CHECK(st.linear_solver == LinearSolverBackend::Qdldl);
  ConeSpec bad;
  bad.soc_dims = {3, 0};
  CHECK(!bad.isValid());
  ConeSpec good;
  good.zero_dim = 2;
  good.nonneg_dim = 3;
  good.soc_dims = {3, 4};
  CHECK(good.isValid() && good.totalDim() == 12);
  CHECK(std::strcmp(toString(Status::Solved), "Solved") == 0);
  CHECK(std::strcmp(toString(Status::MaxIterations), "MaxIterations") == 0);
  Solver s;
  CHECK(s.solve().status == Status::NumericalError);  // before setup
  SparseMat P, A;
  Vec q, b;
  ConeSpec cone;
  readme_problem(P, q, A, b, cone);
  Vec shortb{1.0, 0.0};
  CHECK(!s.setup(P, q, A, shortb, cone));  // dimension mismatch: false, never throws
  CHECK(s.solve().status == Status::NumericalError);
  Solver moved(std::move(s));
  CHECK(moved.solve().status == Status::NumericalError);
  return failures;
}

static int gpu_checks() {
  SparseMat P, A;
  Vec q, b;
  ConeSpec cone;
  readme_problem(P, q, A, b, cone);
  Solver solver;
  CHECK(solver.setup(P, q, A, b, cone));
  const Solution& sol = solver.solve();
  CHECK(sol.ok());
  CHECK(std::fabs(sol.x[0] - 0.5) < 1e-6 && std::fabs(sol.x[1] - 0.5) < 1e-6 &&
        std::fabs(sol.x[2] - std::sqrt(0.5)) < 1e-6);
  CHECK(std::fabs(sol.objective - (0.5 - 1.0 - 0.3 * std::sqrt(0.5))) < 1e-6);
  // values-only update keeps the pattern: b0 = 2 -> x = (1, 1), t = sqrt(2)
  Vec b2{2.0, 0.0, 0.0, 0.0, 0.0};
  CHECK(solver.updateData(nullptr, nullptr, nullptr, &b2));
  const Solution& sol2 = solver.solve();
  CHECK(sol2.ok() && std::fabs(sol2.x[2] - std::sqrt(2.0)) < 1e-6);
  // a different pattern of A is refused
  SparseMat A2 = sparse(5, 3, {Triplet(0, 0, 1.0), Triplet(1, 2, -1.0), Triplet(2, 2, -1.0), Triplet(3, 0, -1.0),
                               Triplet(4, 1, -1.0)});
  CHECK(!solver.updateData(nullptr, nullptr, &A2, nullptr));
  // warm start from the solution converges in no more iterations than a cold start
  const int cold = sol2.info.iterations;
  solver.setWarmStart(sol2.x, sol2.s, sol2.z);
  const Solution& sol3 = solver.solve();
  CHECK(sol3.ok() && sol3.info.iterations <= cold);
  // backward for L = t: t* = b0 / sqrt(2) on the active cone, so dL/db0 = 1/sqrt(2)
  Vec g{0.0, 0.0, 1.0};
  Gradients gr;
  CHECK(solver.backward(g, &gr));
  CHECK(gr.db.size() == 5 && std::fabs(gr.db[0] - 1.0 / std::sqrt(2.0)) < 1e-2);
  // the dense overloads give the same solution
  Mat Pd(3, 3), Ad(5, 3);
  Pd(0, 0) = Pd(1, 1) = Pd(2, 2) = 1.0;
  Ad(0, 0) = Ad(0, 1) = 1.0;
  Ad(1, 2) = Ad(2, 2) = Ad(3, 0) = Ad(4, 1) = -1.0;
  Solver dense;
  CHECK(dense.setup(Pd, q, Ad, b, cone));
  const Solution& sd = dense.solve();
  CHECK(sd.ok() && std::fabs(sd.x[2] - std::sqrt(0.5)) < 1e-6);
  return failures;
}

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  const int f = gpu ? gpu_checks() : host_checks();
  std::printf("%s: %d failure(s)\n", gpu ? "gpu" : "host", f);
  return f == 0 ? 0 : 1;
}
