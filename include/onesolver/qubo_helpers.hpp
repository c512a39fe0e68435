// qubo_helpers.hpp -- dense staging of a QUBO model.
//
// Mirrors helpers::flatten_qubo (include/helpers/qubo_helpers.hpp:26-44 of
// quantumz-io/oneSolver): an n*n row-major symmetric matrix whose diagonal
// holds the linear terms and whose (i,j) and (j,i) entries both hold the
// coupling of i<j. This is the layout the C ABI (os_qubo_dense) takes.
#ifndef ONESOLVER_QUBO_HELPERS_HPP_
#define ONESOLVER_QUBO_HELPERS_HPP_

#include <algorithm>
#include <vector>

#include "onesolver/qubo.hpp"

namespace helpers {

// The same layout written into a caller's buffer of n * n values.
template <class CoeffType>
void flatten_qubo_into(const qubo::QUBOModel<int, CoeffType> &instance, CoeffType *result) {
  const size_t n = instance.get_nodes();
  std::fill(result, result + n * n, CoeffType(0));
  for (auto &kv : instance.linear_terms()) {
    if (kv.first >= 0 && (size_t)kv.first < n)
      result[(size_t)kv.first * n + kv.first] = kv.second;
  }
  // Only keys with i < j contribute (get_connection of (i,j), i > j, finds
  // no key and adds 0); both triangles receive the value.
  for (auto &kv : instance.quadratic_terms()) {
    int i = kv.first.first, j = kv.first.second;
    if (i < 0 || j < 0 || (size_t)i >= n || (size_t)j >= n || i >= j) continue;
    result[(size_t)i + (size_t)j * n] += kv.second;
    result[(size_t)j + (size_t)i * n] += kv.second;
  }
}

template <class CoeffType>
std::vector<CoeffType> flatten_qubo(const qubo::QUBOModel<int, CoeffType> &instance) {
  const size_t n = instance.get_nodes();
  std::vector<CoeffType> result(n * n);
  flatten_qubo_into(instance, result.data());
  return result;
}

}  // namespace helpers

#endif  // ONESOLVER_QUBO_HELPERS_HPP_
