// annealing.hpp -- sa::anneal on the GPU.
//
// Mirrors include/simulated_annealing/annealing.hpp of quantumz-io/oneSolver:
// sa::anneal(instance, queue, beta schedule, num_iter, num_tries,
// sweeps_per_beta) returns the lowest-energy state over num_tries
// trajectories (annealing.hpp:55-140). It runs through os_sa_run: FP32 local
// fields on the GPU, Philox randoms, FP64 re-score of every trajectory's best
// state with the reference's energy function, first minimum on the host
// (annealing.hpp:134-139). With the default options the dynamics are the
// reference's: one random site per step and exp((E - E') / beta) > u.
#ifndef ONESOLVER_ANNEALING_HPP_
#define ONESOLVER_ANNEALING_HPP_

#include <cmath>
#include <vector>

#include "onesolver.h"
#include "onesolver/devices.hpp"
#include "onesolver/qubo.hpp"
#include "onesolver/qubo_helpers.hpp"
#include "onesolver/solution.hpp"

namespace sa {

// Options beyond the reference's signature (all default to its behaviour).
struct Options {
  unsigned long long seed = 1234;            // the reference's engine seed
  int acceptance = OS_ACCEPT_REFERENCE;
  int site_order = OS_SITES_RANDOM;
  int resync_every = 0;
  const std::vector<float> *init_prob = nullptr;  // warm start, P(x_i = 1)
};

template <typename T>
qubo::Solution anneal(qubo::QUBOModel<int, T> instance, os::Queue &q,
                      std::vector<double> &h_beta_schedule, int num_iter,
                      unsigned int num_tries, int sweeps_per_beta = 1,
                      const Options &opt = Options()) {
  const int n = (int)instance.get_nodes();
  std::vector<double> flat = helpers::flatten_qubo(instance);
  os_qubo_dense dq{n, flat.data()};
  os_sa_params p{};
  p.beta = h_beta_schedule.data();
  p.num_iter = num_iter;
  p.sweeps_per_beta = sweeps_per_beta;
  p.num_tries = num_tries;
  p.seed = opt.seed;
  p.acceptance = opt.acceptance;
  p.site_order = opt.site_order;
  p.resync_every = opt.resync_every;
  p.init_prob = opt.init_prob ? opt.init_prob->data() : nullptr;
  std::vector<char> state(n);
  os_sa_result r{};
  r.state = state.data();
  os::check(os_sa_run(q.ctx(), &dq, &p, &r));
  return qubo::Solution(state.begin(), state.end(), r.energy);
}

// The CLI's schedules (app/one-solver-anneal.cpp:23-39), reproduced exactly:
// the linear one ends at beta_min + beta_max.
inline void construct_linear_beta_schedule(std::vector<double> &schedule, double beta_min,
                                           double beta_max, unsigned num_iter) {
  for (unsigned i = 0; i < num_iter; i++)
    schedule[i] = beta_min + beta_max * i / static_cast<double>(num_iter - 1);
}

inline void construct_geometric_beta_schedule(std::vector<double> &schedule, double beta_min,
                                              double beta_max, unsigned num_iter) {
  schedule[0] = beta_min;
  auto alpha = std::pow(beta_max / beta_min, 1.0 / (num_iter - 1));
  for (unsigned i = 1; i < num_iter; i++) schedule[i] = schedule[i - 1] * alpha;
}

}  // namespace sa

#endif  // ONESOLVER_ANNEALING_HPP_
