// tempering.hpp -- parallel tempering and population annealing on the GPU
// from a QUBO model.
//
// No counterpart in quantumz-io/oneSolver: its annealing benchmark names
// parallel tempering as the next solver (benchmarks/annealing/
// performance.md:52-59). pt::temper takes the same model and queue as
// sa::anneal and returns the same qubo::Solution (the lowest-energy state any
// replica visited, FP64 energy from the reference's energy function); it runs
// through os_pt_run_sparse on the model's couplings in CSR form. pa::anneal
// does the same through os_pa_run_sparse.
#ifndef ONESOLVER_TEMPERING_HPP_
#define ONESOLVER_TEMPERING_HPP_

#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

#include "onesolver.h"
#include "onesolver/devices.hpp"
#include "onesolver/qubo.hpp"
#include "onesolver/solution.hpp"

namespace pt {

struct Options {
  unsigned num_chains = 32;      // independent replica chains
  int num_rounds = 1000;         // exchange rounds
  int sweeps_per_round = 5;      // sweeps of every replica per round
  unsigned long long seed = 1234;
  int resync_every = 100;        // rounds between FP64 field resyncs
};

// The model's couplings as symmetric CSR (both triangles, columns ascending)
// and its linear terms, in the layout os_qubo_csr takes. Only i < j keys
// count, as in the reference's flatten (include/helpers/qubo_helpers.hpp:26-44).
struct Csr {
  int n = 0;
  std::vector<int32_t> row_ptr, col;
  std::vector<double> val, diag;
};

template <typename T> Csr to_csr(const qubo::QUBOModel<int, T> &m) {
  Csr c;
  c.n = (int)m.get_nodes();
  const size_t n = (size_t)c.n;
  c.diag.assign(n, 0.0);
  for (auto &kv : m.linear_terms())
    if (kv.first >= 0 && (size_t)kv.first < n) c.diag[kv.first] = (double)kv.second;
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  for (auto &kv : m.quadratic_terms()) {
    const int i = kv.first.first, j = kv.first.second;
    if (i < 0 || j < 0 || (size_t)i >= n || (size_t)j >= n || i >= j || kv.second == 0) continue;
    rows[i].push_back({j, (double)kv.second});
    rows[j].push_back({i, (double)kv.second});
  }
  c.row_ptr.assign(n + 1, 0);
  for (size_t i = 0; i < n; ++i) {
    std::sort(rows[i].begin(), rows[i].end());
    c.row_ptr[i + 1] = c.row_ptr[i] + (int32_t)rows[i].size();
    for (auto &e : rows[i]) {
      c.col.push_back(e.first);
      c.val.push_back(e.second);
    }
  }
  return c;
}

// Inverse temperatures beta_min * (beta_max / beta_min)^(k / (num_temps - 1)).
inline std::vector<double> geometric_ladder(double beta_min, double beta_max, int num_temps) {
  std::vector<double> b(num_temps);
  for (int k = 0; k < num_temps; ++k)
    b[k] = num_temps == 1 ? beta_min : beta_min * std::pow(beta_max / beta_min, k / (double)(num_temps - 1));
  return b;
}

template <typename T>
qubo::Solution temper(const qubo::QUBOModel<int, T> &instance, os::Queue &q, const std::vector<double> &beta,
                      const Options &opt = Options()) {
  const Csr c = to_csr(instance);
  os_qubo_csr qc{c.n, c.row_ptr.data(), c.col.data(), c.val.data(), c.diag.data()};
  os_pt_params p{};
  p.beta = beta.data();
  p.num_temps = (int32_t)beta.size();
  p.num_chains = opt.num_chains;
  p.num_rounds = opt.num_rounds;
  p.sweeps_per_round = opt.sweeps_per_round;
  p.seed = opt.seed;
  p.resync_every = opt.resync_every;
  std::vector<char> state(c.n);
  os_pt_result r{};
  r.state = state.data();
  os::check(os_pt_run_sparse(q.ctx(), &qc, &p, &r));
  return qubo::Solution(state.begin(), state.end(), r.energy);
}

}  // namespace pt

namespace pa {

// Population annealing (os_pa_run_sparse): resampling between consecutive
// inverse temperatures of the schedule, sweeps_per_beta sweeps per step.
struct Options {
  unsigned population = 16384;
  int sweeps_per_beta = 5;
  unsigned long long seed = 1234;
  int resync_every = 100;        // steps between FP64 field resyncs
};

template <typename T>
qubo::Solution anneal(const qubo::QUBOModel<int, T> &instance, os::Queue &q, const std::vector<double> &beta,
                      const Options &opt = Options()) {
  const pt::Csr c = pt::to_csr(instance);
  os_qubo_csr qc{c.n, c.row_ptr.data(), c.col.data(), c.val.data(), c.diag.data()};
  os_pa_params p{};
  p.beta = beta.data();
  p.num_steps = (int32_t)beta.size();
  p.sweeps_per_beta = opt.sweeps_per_beta;
  p.population = opt.population;
  p.seed = opt.seed;
  p.resync_every = opt.resync_every;
  std::vector<char> state(c.n);
  os_pa_result r{};
  r.state = state.data();
  os::check(os_pa_run_sparse(q.ctx(), &qc, &p, &r));
  return qubo::Solution(state.begin(), state.end(), r.energy);
}

}  // namespace pa

#endif  // ONESOLVER_TEMPERING_HPP_
