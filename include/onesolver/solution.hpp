// solution.hpp -- qubo::Solution, the result type of both solvers.
//
// Mirrors include/model/solution.hpp of quantumz-io/oneSolver: a 0/1 state
// vector plus its energy, serialised by save() as a two-line CSV (variable
// indices then "energy"; values then the energy at the stream's default
// precision of 6 significant digits), byte for byte as solution.hpp:58-67.
#ifndef ONESOLVER_SOLUTION_HPP_
#define ONESOLVER_SOLUTION_HPP_

#include <ostream>
#include <vector>

namespace qubo {

class Solution {
public:
  std::vector<char> state;
  double energy;

  template <typename InputIt>
  Solution(InputIt begin, InputIt end, double energy)
      : state(begin, end), energy(energy) {}

  void save(std::ostream &stream) {
    for (size_t var_index = 0; var_index < state.size(); var_index++) {
      stream << var_index << ',';
    }
    stream << "energy" << std::endl;
    for (auto &bit : state) {
      stream << int(bit) << ",";
    }
    stream << energy << std::endl;
  }
};

}  // namespace qubo

#endif  // ONESOLVER_SOLUTION_HPP_
