// exhaustive.hpp -- exhaustive::solve on the GPU.
//
// Mirrors include/exhaustive/exhaustive.hpp of quantumz-io/oneSolver:
// solve(queue, model) returns the minimum energy and the smallest minimising
// state (exhaustive.hpp:29-167), through os_exhaustive_run (Gray-code
// enumeration, exact for integer coefficients). The reference's 32-variable
// limit (exhaustive.hpp:67, ulong_to_vec.hpp:24-26) is lifted to 50.
// solve_all additionally returns every degenerate minimiser.
#ifndef ONESOLVER_EXHAUSTIVE_HPP_
#define ONESOLVER_EXHAUSTIVE_HPP_

#include <cstdint>
#include <vector>

#include "onesolver.h"
#include "onesolver/devices.hpp"
#include "onesolver/qubo.hpp"
#include "onesolver/qubo_helpers.hpp"
#include "onesolver/solution.hpp"

namespace helpers {

// ulong_to_vec (include/helpers/ulong_to_vec.hpp:23-32): bit i = variable i.
inline std::vector<char> ulong_to_vec(unsigned long long val, unsigned n_bits) {
  std::vector<char> state;
  for (unsigned i = 0; i < n_bits; ++i) state.push_back((val >> i) & 1ull);
  return state;
}

}  // namespace helpers

namespace exhaustive {

struct AllMinimisers {
  double energy;
  std::vector<uint64_t> states;  // ascending
  unsigned long long count;
};

template <class NodeType, class CoefType>
AllMinimisers solve_all(os::Queue &q, qubo::QUBOModel<NodeType, CoefType> &qubos,
                        unsigned long long max_minimisers = 1u << 16) {
  const int n = (int)qubos.get_nodes();
  std::vector<double> flat = helpers::flatten_qubo(qubos);
  os_qubo_dense dq{n, flat.data()};
  os_exh_params p{};
  p.max_minimisers = max_minimisers;
  std::vector<uint64_t> states(max_minimisers ? max_minimisers : 1);
  os_exh_result r{};
  r.states = states.data();
  os::check(os_exhaustive_run(q.ctx(), &dq, &p, &r));
  states.resize(r.count < max_minimisers ? r.count : max_minimisers);
  return AllMinimisers{r.energy, states, r.count};
}

template <class NodeType, class CoefType>
qubo::Solution solve(os::Queue &q, qubo::QUBOModel<NodeType, CoefType> &qubos) {
  const int n = (int)qubos.get_nodes();
  std::vector<double> flat = helpers::flatten_qubo(qubos);
  os_qubo_dense dq{n, flat.data()};
  os_exh_params p{};
  os_exh_result r{};
  os::check(os_exhaustive_run(q.ctx(), &dq, &p, &r));
  auto result = helpers::ulong_to_vec(r.state, n);
  return qubo::Solution(result.begin(), result.end(), r.energy);
}

}  // namespace exhaustive

#endif  // ONESOLVER_EXHAUSTIVE_HPP_
