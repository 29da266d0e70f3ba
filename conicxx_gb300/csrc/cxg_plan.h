// Host-side symbolic set-up of one instance: validation, equilibration, and the device plan
// (index arrays that stay fixed while only values change, the role SparsityMap + KktSystem::setup
// play in the reference: src/conicxx/kkt/sparsity_map.cpp:8-56, kkt_system.cpp:22-117).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "conicxx_gb300.h"
#include "cxg_layout.h"

namespace cxg {

struct Pools {
  std::vector<int> ipool;
  std::vector<double> dpool;
  std::vector<InstanceDesc> desc;
  int64_t totPx = 0, totQ = 0, totAx = 0, totB = 0;  // lengths of the concatenated value arrays
};

// Structural validation of one problem (cone spec as ConeSpec::isValid, cone_spec.h:25-31,
// dimensions as SolverImpl::setup, solver_impl.cpp:11-16, plus CSC well-formedness, which the
// device path needs to index safely). Returns an empty string when valid.
std::string validateProblem(const cxg_problem& pr);

// A size the device plan cannot index (reported as CXG_E_UNSUPPORTED, not as an allocation failure).
struct LimitError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// The plan's per-instance counts that the device indexes with 32-bit ints, computed exactly from
// the input pattern before any plan array is built: entries of the full symmetric P (both
// triangles of the stored upper part), of the densified per-unit A blocks (sum of d_u * s_u over
// cone units, s_u the number of distinct columns in the unit's rows), and three ints per cone-unit
// contribution (sum of s_u (s_u + 1) / 2). Returns an empty string when all fit in INT32_MAX.
std::string checkPlanCounts(const cxg_problem& pr);

// Ruiz equilibration (src/conicxx/kkt/equilibration.cpp:8-100) of the RAW data.
void computeEquilibration(const cxg_problem& pr, const cxg_settings& st, std::vector<double>& d,
                          std::vector<double>& e, double& c);

// Appends the plan of `pr` to `pools` (values are NOT copied; see packValues).
void planInstance(const cxg_problem& pr, const cxg_settings& st, Pools& pools);

// Appends the plans of `src` (planned on their own) to `dst`, shifting every pool and value
// offset of src's instances by what dst already holds.
void appendPools(Pools& dst, const Pools& src);

// Whether P's upper-CSC pattern / A's CSC pattern equal the instance's (updateData check,
// kkt_system.cpp:10-19).
bool samePattern(const std::vector<int>& p_ref, const std::vector<int>& i_ref, int cols,
                 const int* p, const int* i);

}  // namespace cxg
