// oracle.cpp -- CPU restatement of oneSolver's two hot paths.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: the pytest suite, the
// smoke check and the CPU-baseline leg of bench.py load it (through
// liboracle.so) to verify the GPU library and to time the reference's
// algorithm on host cores. The product (libonesolver.so) never links or
// calls it.
//
// Every function restates the reference algorithm it cites (paths are
// relative to the quantumz-io/oneSolver project root). The reference itself
// cannot be compiled here (it needs a SYCL compiler, Boost and oneMKL), so
// parity is pinned by checking this restatement against the reference's own
// known-answer tests (tests/exhaustive_test.cpp, tests/qubo_helpers_test.cpp).
//
// Conventions shared with the GPU library:
//   * a QUBO of n variables is staged as the reference's flat matrix
//     F (n*n doubles, row-major, symmetric, diagonal = linear terms),
//     produced by orc_flatten (helpers::flatten_qubo);
//   * a state is n chars, one 0/1 value per variable, variable 0 first;
//     exhaustive-search states are uint64 with bit i = variable i
//     (helpers::ulong_to_vec, include/helpers/ulong_to_vec.hpp:23-32).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

namespace {

// sa::energy, include/simulated_annealing/annealing.hpp:31-40.
// E(x) = sum_{i<=j} F[i*n+j] * x_i * x_j, accumulated in FP64 in row-major
// order over the upper triangle. Multiplying by 0/1 chars is exact, so the
// value equals the ordered sum of F[i][j] over the pairs with both bits set.
double energy_ref(const double *flat, const char *state, int n) {
  double result = 0.0;
  for (int i = 0; i < n; i++) {
    for (int j = i; j < n; j++) {
      result += flat[(size_t)i * n + j] * state[i] * state[j];
    }
  }
  return result;
}

// Inner loop of exhaustive::solve, include/exhaustive/exhaustive.hpp:112-129:
// the same ordered FP64 sum, written over the bits of a state integer.
double energy_state_bits(const double *flat, int n, uint64_t state) {
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    for (int j = i; j < n; ++j) {
      if (i == j) {
        if ((state >> i) & 1ull) e += flat[(size_t)i * n + i];
      } else {
        if (((state >> i) & 1ull) && ((state >> j) & 1ull))
          e += flat[(size_t)i * n + j];
      }
    }
  }
  return e;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11). Restated from the published round function; the
// GPU library carries its own implementation and the tests compare the two.
inline void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                   uint32_t out[4]) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(M0, c0, hi0, lo0);
    mulhilo32(M1, c2, hi1, lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += W0; k1 += W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Small host RNG for the free-running oracle anneal (splitmix64 seeding a
// xoshiro256** stream, both published generators by Vigna). The oracle's
// free-running stream is independent of the GPU's Philox stream: the two are
// compared statistically, never draw by draw.
struct HostRng {
  uint64_t s[4];
  static uint64_t splitmix(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  explicit HostRng(uint64_t seed) {
    for (int i = 0; i < 4; ++i) s[i] = splitmix(seed);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
  int below(int n) { return (int)(((next() >> 32) * (uint64_t)n) >> 32); }
};

}  // namespace

extern "C" {

// helpers::flatten_qubo, include/helpers/qubo_helpers.hpp:26-44.
// Inputs are the model's coefficient maps as parallel arrays (linear
// i -> v; quadratic (i,j) -> v with i<j, as QUBOBuilder::add_element stores
// them, include/model/qubo.hpp:304-318). A key missing from a map reads as 0
// (QUBOModel::get_variable / get_connection, qubo.hpp:216-240), and
// get_connection(i,j) with i>j finds no key, so only i<j pairs contribute.
void orc_flatten(int n, int nlin, const int *lin_i, const double *lin_v,
                 int nquad, const int *quad_i, const int *quad_j,
                 const double *quad_v, double *out) {
  std::vector<double> lin(n, 0.0);
  for (int k = 0; k < nlin; ++k)
    if (lin_i[k] >= 0 && lin_i[k] < n) lin[lin_i[k]] = lin_v[k];
  std::vector<double> quad((size_t)n * n, 0.0);
  std::vector<char> present((size_t)n * n, 0);
  for (int k = 0; k < nquad; ++k) {
    int i = quad_i[k], j = quad_j[k];
    if (i >= 0 && j >= 0 && i < n && j < n) {
      quad[(size_t)i * n + j] = quad_v[k];
      present[(size_t)i * n + j] = 1;
    }
  }
  std::fill(out, out + (size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) {
      if (i == j) {
        out[(size_t)i + (size_t)j * n] = lin[i];
      } else {
        double c = (i < j && present[(size_t)i * n + j]) ? quad[(size_t)i * n + j] : 0.0;
        out[(size_t)i + (size_t)j * n] += c;
        out[(size_t)j + (size_t)i * n] += c;
      }
    }
  }
}

double orc_energy(const double *flat, const char *state, int n) {
  return energy_ref(flat, state, n);
}

// Batch re-score: energies of m states (m x n chars).
void orc_energy_batch(const double *flat, const char *states, int n, int m,
                      double *out) {
  for (int t = 0; t < m; ++t) out[t] = energy_ref(flat, states + (size_t)t * n, n);
}

double orc_energy_bits(const double *flat, int n, uint64_t state) {
  return energy_state_bits(flat, n, state);
}

// Beta schedules of app/one-solver-anneal.cpp:23-39, reproduced exactly:
// linear beta_i = beta_min + beta_max * i / (n-1) (ends at beta_min+beta_max),
// geometric as a running FP64 product with alpha = (max/min)^(1/(n-1)).
void orc_schedule_linear(double *out, double beta_min, double beta_max,
                         unsigned num_iter) {
  for (unsigned i = 0; i < num_iter; i++)
    out[i] = beta_min + beta_max * i / static_cast<double>(num_iter - 1);
}

void orc_schedule_geometric(double *out, double beta_min, double beta_max,
                            unsigned num_iter) {
  out[0] = beta_min;
  double alpha = std::pow(beta_max / beta_min, 1.0 / (num_iter - 1));
  for (unsigned i = 1; i < num_iter; i++) out[i] = out[i - 1] * alpha;
}

// Exhaustive search over the state range [begin, end) exactly as the
// reference's work-item loop (exhaustive.hpp:106-134): FP64 energy per state,
// keep the first strict minimum. Ranges are split over nthreads host threads
// the way the reference splits over compute units (exhaustive.hpp:63-90, with
// the 64-bit shift repaired), and the per-range results are reduced with the
// first-minimum rule of std::min_element (exhaustive.hpp:158-159). The tie
// rule therefore returns the smallest state integer among exact minima.
void orc_exhaustive(const double *flat, int n, uint64_t begin, uint64_t end,
                    int nthreads, double *e_out, uint64_t *state_out) {
  if (nthreads < 1) nthreads = 1;
  uint64_t total = end - begin;
  std::vector<double> e_best(nthreads, std::numeric_limits<double>::max());
  std::vector<uint64_t> s_best(nthreads, 0);
  uint64_t per = total / nthreads, rem = total % nthreads;
  std::vector<std::thread> pool;
  uint64_t cursor = begin;
  for (int t = 0; t < nthreads; ++t) {
    uint64_t lo = cursor;
    cursor += per + ((uint64_t)t < rem ? 1 : 0);
    uint64_t hi = cursor;
    pool.emplace_back([&, t, lo, hi]() {
      double eb = std::numeric_limits<double>::max();
      uint64_t sb = 0;
      for (uint64_t s = lo; s < hi; ++s) {
        double e = energy_state_bits(flat, n, s);
        if (e < eb) { eb = e; sb = s; }
      }
      e_best[t] = eb;
      s_best[t] = sb;
    });
  }
  for (auto &th : pool) th.join();
  int best = (int)(std::min_element(e_best.begin(), e_best.end()) - e_best.begin());
  *e_out = e_best[best];
  *state_out = s_best[best];
}

// All exact minimisers over [begin, end) under the reference's FP64 energy
// function: the degenerate ground-state set that the reference's strict-min
// scan would pick from. Writes up to cap states in ascending order and returns
// the total count.
uint64_t orc_exhaustive_all(const double *flat, int n, uint64_t begin,
                            uint64_t end, int nthreads, double *e_out,
                            uint64_t *states, uint64_t cap) {
  if (nthreads < 1) nthreads = 1;
  double emin;
  uint64_t smin;
  orc_exhaustive(flat, n, begin, end, nthreads, &emin, &smin);
  uint64_t total = end - begin;
  std::vector<std::vector<uint64_t>> found(nthreads);
  uint64_t per = total / nthreads, rem = total % nthreads;
  std::vector<std::thread> pool;
  uint64_t cursor = begin;
  for (int t = 0; t < nthreads; ++t) {
    uint64_t lo = cursor;
    cursor += per + ((uint64_t)t < rem ? 1 : 0);
    uint64_t hi = cursor;
    pool.emplace_back([&, t, lo, hi]() {
      for (uint64_t s = lo; s < hi; ++s)
        if (energy_state_bits(flat, n, s) == emin) found[t].push_back(s);
    });
  }
  for (auto &th : pool) th.join();
  uint64_t count = 0;
  for (auto &v : found)
    for (uint64_t s : v) {
      if (count < cap) states[count] = s;
      ++count;
    }
  *e_out = emin;
  return count;
}

// All exact minimisers over [begin, end) of an integer-coefficient QUBO, for
// state spaces too large for the O(n^2)-per-state loop of orc_exhaustive_all
// (2^36 states at n = 36). Every state's energy is still evaluated on its
// own, as the reference's work-item loop does (exhaustive.hpp:110-129):
//   E(s) = sum_{i set} ( Q_ii + sum_{j > i, j set} Q_ij ),
// with the inner sum over j read a byte of the state at a time from per-row
// tables U_i[b][v] = sum of Q_ij over the set bits j of byte value v in byte
// b (j > i only). With integer coefficients every partial sum is an integer
// far below 2^53, so the int64 value equals the reference's FP64 sum in any
// order. Returns the total number of minimisers (up to cap of them written
// to states in ascending order) and the minimum in *e_out; returns -1 when a
// coefficient on or above the diagonal is not an integer of magnitude below
// 2^40. Threads take blocks of 2^16 states from a shared counter.
int64_t orc_exhaustive_int_all(const double *flat, int n, uint64_t begin, uint64_t end, int nthreads,
                               int64_t *e_out, uint64_t *states, uint64_t cap) {
  if (n < 1 || n > 63 || end <= begin) return -1;
  if (nthreads < 1) nthreads = 1;
  const int nb = (n + 7) / 8;
  std::vector<int64_t> diag(n);
  std::vector<int64_t> tab((size_t)n * nb * 256, 0);
  for (int i = 0; i < n; ++i) {
    for (int j = i; j < n; ++j) {
      const double v = flat[(size_t)i * n + j];
      if (!(std::fabs(v) < 0x1.0p40) || v != std::floor(v)) return -1;
    }
    diag[i] = (int64_t)flat[(size_t)i * n + i];
    for (int b = 0; b < nb; ++b)
      for (int v = 0; v < 256; ++v) {
        int64_t s = 0;
        for (int k = 0; k < 8; ++k) {
          const int j = 8 * b + k;
          if (j > i && j < n && ((v >> k) & 1)) s += (int64_t)flat[(size_t)i * n + j];
        }
        tab[((size_t)i * nb + b) * 256 + v] = s;
      }
  }
  const uint64_t block = 1ull << 16;
  std::atomic<uint64_t> next{begin};
  std::vector<int64_t> emin(nthreads, std::numeric_limits<int64_t>::max());
  std::vector<std::vector<uint64_t>> found(nthreads);
  auto worker = [&](int t) {
    int64_t em = std::numeric_limits<int64_t>::max();
    std::vector<uint64_t> &f = found[t];
    for (;;) {
      const uint64_t lo = next.fetch_add(block);
      if (lo >= end) break;
      const uint64_t hi = std::min(end, lo + block);
      for (uint64_t s = lo; s < hi; ++s) {
        int64_t e = 0;
        for (uint64_t m = s; m; m &= m - 1) {
          const int i = __builtin_ctzll(m);
          const int64_t *row = &tab[(size_t)i * nb * 256];
          int64_t r = diag[i];
          for (int b = i >> 3; b < nb; ++b) r += row[b * 256 + ((s >> (8 * b)) & 255)];
          e += r;
        }
        if (e < em) {
          em = e;
          f.clear();
        }
        if (e == em) f.push_back(s);
      }
    }
    emin[t] = em;
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker, t);
  for (auto &th : pool) th.join();
  const int64_t best = *std::min_element(emin.begin(), emin.end());
  std::vector<uint64_t> all;
  for (int t = 0; t < nthreads; ++t)
    if (emin[t] == best) all.insert(all.end(), found[t].begin(), found[t].end());
  std::sort(all.begin(), all.end());
  for (uint64_t k = 0; k < all.size() && k < cap; ++k) states[k] = all[k];
  *e_out = best;
  return (int64_t)all.size();
}

// Deterministic verification transcription of sa::anneal's kernel body,
// include/simulated_annealing/annealing.hpp:87-125, for one trajectory per
// row of the precomputed arrays.
//
// The reference draws from oneMKL philox4x32x10 (annealing.hpp:87), which
// is not reproducible here. Verification mode instead consumes caller-given
// arrays: init[t*n + i] (the bit() draws of annealing.hpp:91-93),
// site[t*steps + a] (bit_index(), :101) and u[t*steps + a] (uniform(),
// :108), with steps = num_iter * sweeps_per_beta. One (site, u) pair is
// consumed per attempt unconditionally, so the array index of attempt a is
// fixed; the reference only draws u when new_energy >= current_energy (the
// short-circuit at :106-108), which leaves the decisions unchanged.
//
// acceptance 0 = the reference rule exp((E_cur - E_new) / beta) > u
// (:106-108); acceptance 1 = the physical Metropolis rule
// exp(-beta * (E_new - E_cur)) > u. Energies are full FP64 recomputations
// per attempt as in the reference (:104).
//
// Outputs: best_states/best_energies (the kernel's best_states /
// best_energies_acc, :115-121,124), final_states/final_energies (the
// current_states at exit), and accept_count per trajectory.
void orc_anneal_verify(const double *flat, int n, const double *beta,
                       int num_iter, int num_tries, int sweeps_per_beta,
                       const char *init, const int *site, const double *u,
                       int acceptance, char *best_states,
                       double *best_energies, char *final_states,
                       double *final_energies, int64_t *accept_count) {
  const int64_t steps = (int64_t)num_iter * sweeps_per_beta;
  for (int t = 0; t < num_tries; ++t) {
    std::vector<char> cur(init + (size_t)t * n, init + (size_t)(t + 1) * n);
    std::vector<char> best = cur;
    double best_energy = energy_ref(flat, cur.data(), n);
    double current_energy = best_energy;
    int64_t acc = 0;
    for (int iter = 0; iter < num_iter; iter++) {
      double b = beta[iter];
      for (int sweep = 0; sweep < sweeps_per_beta; sweep++) {
        int64_t a = (int64_t)iter * sweeps_per_beta + sweep;
        int k = site[(size_t)t * steps + a];
        double uu = u[(size_t)t * steps + a];
        cur[k] = 1 - cur[k];
        double new_energy = energy_ref(flat, cur.data(), n);
        bool accept;
        if (new_energy < current_energy) {
          accept = true;
        } else if (acceptance == 0) {
          accept = std::exp((current_energy - new_energy) / b) > uu;
        } else {
          accept = std::exp(-b * (new_energy - current_energy)) > uu;
        }
        if (accept) {
          current_energy = new_energy;
          ++acc;
        } else {
          cur[k] = 1 - cur[k];
        }
        if (current_energy < best_energy) {
          best_energy = current_energy;
          best = cur;
        }
      }
    }
    std::memcpy(best_states + (size_t)t * n, best.data(), n);
    best_energies[t] = best_energy;
    if (final_states) std::memcpy(final_states + (size_t)t * n, cur.data(), n);
    if (final_energies) final_energies[t] = current_energy;
    if (accept_count) accept_count[t] = acc;
  }
}

// Replay transcription of sa::anneal's kernel body
// (include/simulated_annealing/annealing.hpp:97-123) in a given site order,
// for checking the GPU sweep kernels' replay mode bit for bit.
//
// Trajectory t starts from init[t*n ..] (:91-93). Step a = iter *
// sweeps_per_beta + sweep runs at beta[iter] (:97-99) and is
//   mode 0: one attempt at site[t*S + a] (:101), u = u[t*S + a];
//   mode 1, 2: one attempt at every site in order[0 .. n) (a sequential
//           sweep), u = u[(t*S + a)*n + k] for site k;
// with S = num_iter * sweeps_per_beta. An attempt flips the site, takes the
// energy of the flipped state, keeps the flip when new_energy <
// current_energy or the acceptance test passes, else flips back (:102-113):
// acceptance 0 is exp((current_energy - new_energy) / beta) > u, 1 is
// exp(-beta * (new_energy - current_energy)) > u. The best state and energy
// are updated when current_energy < best_energy (:115-121) after every
// attempt (modes 0 and 1), or after the last attempt of every sweep only
// (mode 2: the sparse kernel's bookkeeping).
//
// full_energy 1 evaluates every new_energy from scratch with the
// reference's energy function (:104); 0 keeps FP64 local fields
// h_k = sum_{j != k} F[k][j] x_j, new_energy = current_energy +
// (1 - 2 x_k)(F[k][k] + h_k), which equals it exactly when the
// coefficients are integers (every partial sum an integer below 2^53) and
// costs O(n) per accepted flip instead of O(n^2) per attempt.
//
// Outputs per trajectory: final and best states, final and best energies,
// accepted flips. Trajectories are spread over nthreads host threads.
void orc_sa_replay(const double *flat, int n, const double *beta, int num_iter, int sweeps_per_beta,
                   int num_tries, int acceptance, int mode, const int *order, const char *init,
                   const int *site, const double *u, int full_energy, int nthreads, char *final_states,
                   char *best_states, double *final_energies, double *best_energies,
                   int64_t *accept_count) {
  if (nthreads < 1) nthreads = 1;
  const int64_t S = (int64_t)num_iter * sweeps_per_beta;
  std::atomic<int> next{0};
  auto worker = [&]() {
    std::vector<char> cur(n), best(n);
    std::vector<double> h(n);
    for (;;) {
      const int t = next.fetch_add(1);
      if (t >= num_tries) break;
      for (int i = 0; i < n; ++i) cur[i] = init[(size_t)t * n + i] ? 1 : 0;
      best = cur;
      for (int k = 0; k < n; ++k) {
        double acc = 0.0;
        for (int j = 0; j < n; ++j)
          if (j != k && cur[j]) acc += j < k ? flat[(size_t)j * n + k] : flat[(size_t)k * n + j];
        h[k] = acc;
      }
      double best_energy = energy_ref(flat, cur.data(), n);
      double current_energy = best_energy;
      int64_t acc = 0;
      auto attempt = [&](int k, double b, double uu) {
        cur[k] = 1 - cur[k];
        double new_energy;
        if (full_energy) {
          new_energy = energy_ref(flat, cur.data(), n);
        } else {
          const double loc = flat[(size_t)k * n + k] + h[k];
          new_energy = current_energy + (cur[k] ? loc : -loc);
        }
        bool keep = new_energy < current_energy;
        if (!keep)
          keep = acceptance == 0 ? std::exp((current_energy - new_energy) / b) > uu
                                 : std::exp(-b * (new_energy - current_energy)) > uu;
        if (keep) {
          current_energy = new_energy;
          ++acc;
          if (!full_energy) {
            const double sgn = cur[k] ? 1.0 : -1.0;
            for (int j = 0; j < n; ++j)
              if (j != k) h[j] += sgn * (j < k ? flat[(size_t)j * n + k] : flat[(size_t)k * n + j]);
          }
        } else {
          cur[k] = 1 - cur[k];
        }
      };
      for (int iter = 0; iter < num_iter; iter++) {
        const double b = beta[iter];
        for (int sweep = 0; sweep < sweeps_per_beta; sweep++) {
          const int64_t a = (int64_t)iter * sweeps_per_beta + sweep;
          if (mode == 0) {
            attempt(site[(size_t)t * S + a], b, u[(size_t)t * S + a]);
          } else {
            const double *ua = u + ((size_t)t * S + a) * n;
            for (int m = 0; m < n; ++m) {
              const int k = order[m];
              attempt(k, b, ua[k]);
              if (mode == 1 && current_energy < best_energy) {
                best_energy = current_energy;
                best = cur;
              }
            }
          }
          if (mode != 1 && current_energy < best_energy) {
            best_energy = current_energy;
            best = cur;
          }
        }
      }
      std::memcpy(final_states + (size_t)t * n, cur.data(), n);
      std::memcpy(best_states + (size_t)t * n, best.data(), n);
      final_energies[t] = current_energy;
      best_energies[t] = best_energy;
      accept_count[t] = acc;
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < nthreads; ++i) pool.emplace_back(worker);
  for (auto &th : pool) th.join();
}

// Free-running CPU anneal with the reference algorithm (full FP64 energy
// recomputation per attempt, annealing.hpp:97-123) and a host RNG, threaded
// over trajectories the way the SYCL cpu device runs work-items. Used as the
// statistical reference (KS tests) and as the timed CPU baseline.
//
// site_order 0 = one uniformly random site per step (the reference);
// site_order 1 = one step is a sequential pass over sites 0..n-1 (n
// attempts), the physics "sweep". Returns total attempts performed.
int64_t orc_anneal_free(const double *flat, int n, const double *beta,
                        int num_iter, int num_tries, int sweeps_per_beta,
                        uint64_t seed, int acceptance, int site_order,
                        int nthreads, char *best_states,
                        double *best_energies) {
  if (nthreads < 1) nthreads = 1;
  std::atomic<int> next{0};
  std::atomic<int64_t> attempts{0};
  auto worker = [&]() {
    for (;;) {
      int t = next.fetch_add(1);
      if (t >= num_tries) break;
      HostRng rng(seed * 0x9E3779B97F4A7C15ull + (uint64_t)t * 0xD1B54A32D192ED03ull + 1);
      std::vector<char> cur(n), best(n);
      for (int i = 0; i < n; ++i) cur[i] = (char)(rng.next() >> 63);
      best = cur;
      double best_energy = energy_ref(flat, cur.data(), n);
      double current_energy = best_energy;
      int64_t local = 0;
      for (int iter = 0; iter < num_iter; iter++) {
        double b = beta[iter];
        for (int sweep = 0; sweep < sweeps_per_beta; sweep++) {
          int inner = site_order == 1 ? n : 1;
          for (int s = 0; s < inner; ++s) {
            int k = site_order == 1 ? s : rng.below(n);
            cur[k] = 1 - cur[k];
            double new_energy = energy_ref(flat, cur.data(), n);
            bool accept;
            if (new_energy < current_energy) {
              accept = true;
            } else {
              double uu = rng.uniform();
              accept = acceptance == 0
                           ? std::exp((current_energy - new_energy) / b) > uu
                           : std::exp(-b * (new_energy - current_energy)) > uu;
            }
            if (accept) current_energy = new_energy;
            else cur[k] = 1 - cur[k];
            if (current_energy < best_energy) {
              best_energy = current_energy;
              best = cur;
            }
            ++local;
          }
        }
      }
      std::memcpy(best_states + (size_t)t * n, best.data(), n);
      best_energies[t] = best_energy;
      attempts += local;
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < nthreads; ++i) pool.emplace_back(worker);
  for (auto &th : pool) th.join();
  return attempts.load();
}

// The free-running anneal of orc_anneal_free (same host RNG stream, same
// draws in the same order: the initial bits, then per attempt the site in
// random order and the uniform only when new_energy >= current_energy, the
// short-circuit of annealing.hpp:106-108), with two changes for large
// instances:
//   * energies are kept in FP64 local fields over the nonzero couplings,
//     new_energy = current_energy + (1 - 2 x_k)(F[k][k] + h_k), which equals
//     the reference's per-attempt recomputation (:104) exactly for integer
//     coefficients and to rounding otherwise, at O(degree) per accepted flip;
//   * a sequential sweep visits order[0 .. n) (NULL: 0 .. n-1), so the chain
//     can be the one a GPU kernel runs in its own site order.
// best_at_sweep_end = 1 checks the best state at the end of every step only
// (the sparse kernel's bookkeeping) instead of after every attempt
// (:115-121). With order = NULL and best_at_sweep_end = 0 the output on an
// integer instance is orc_anneal_free's, bit for bit. Returns the attempts.
int64_t orc_anneal_free_fields(const double *flat, int n, const double *beta, int num_iter, int sweeps_per_beta,
                               int num_tries, uint64_t seed, int acceptance, int site_order, const int *order,
                               int best_at_sweep_end, int nthreads, char *best_states, double *best_energies) {
  if (nthreads < 1) nthreads = 1;
  // Nonzero couplings of every site (upper triangle mirrored).
  std::vector<int> ptr(n + 1, 0), nb;
  std::vector<double> cv;
  for (int k = 0; k < n; ++k) {
    for (int j = 0; j < n; ++j) {
      if (j == k) continue;
      const double c = j < k ? flat[(size_t)j * n + k] : flat[(size_t)k * n + j];
      if (c != 0.0) {
        nb.push_back(j);
        cv.push_back(c);
      }
    }
    ptr[k + 1] = (int)nb.size();
  }
  std::atomic<int> next{0};
  std::atomic<int64_t> attempts{0};
  auto worker = [&]() {
    std::vector<char> cur(n), best(n);
    std::vector<double> h(n);
    for (;;) {
      const int t = next.fetch_add(1);
      if (t >= num_tries) break;
      HostRng rng(seed * 0x9E3779B97F4A7C15ull + (uint64_t)t * 0xD1B54A32D192ED03ull + 1);
      for (int i = 0; i < n; ++i) cur[i] = (char)(rng.next() >> 63);
      best = cur;
      for (int k = 0; k < n; ++k) {
        double acc = 0.0;
        for (int e = ptr[k]; e < ptr[k + 1]; ++e)
          if (cur[nb[e]]) acc += cv[e];
        h[k] = acc;
      }
      double best_energy = energy_ref(flat, cur.data(), n);
      double current_energy = best_energy;
      int64_t local = 0;
      for (int iter = 0; iter < num_iter; iter++) {
        const double b = beta[iter];
        for (int sweep = 0; sweep < sweeps_per_beta; sweep++) {
          const int inner = site_order == 1 ? n : 1;
          for (int s = 0; s < inner; ++s) {
            const int k = site_order == 1 ? (order ? order[s] : s) : rng.below(n);
            const double loc = flat[(size_t)k * n + k] + h[k];
            const double new_energy = current_energy + (cur[k] ? -loc : loc);
            bool accept;
            if (new_energy < current_energy) {
              accept = true;
            } else {
              const double uu = rng.uniform();
              accept = acceptance == 0 ? std::exp((current_energy - new_energy) / b) > uu
                                       : std::exp(-b * (new_energy - current_energy)) > uu;
            }
            if (accept) {
              cur[k] = 1 - cur[k];
              current_energy = new_energy;
              const double sgn = cur[k] ? 1.0 : -1.0;
              for (int e = ptr[k]; e < ptr[k + 1]; ++e) h[nb[e]] += sgn * cv[e];
            }
            if (!best_at_sweep_end && current_energy < best_energy) {
              best_energy = current_energy;
              best = cur;
            }
            ++local;
          }
          if (best_at_sweep_end && current_energy < best_energy) {
            best_energy = current_energy;
            best = cur;
          }
        }
      }
      std::memcpy(best_states + (size_t)t * n, best.data(), n);
      best_energies[t] = best_energy;
      attempts += local;
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < nthreads; ++i) pool.emplace_back(worker);
  for (auto &th : pool) th.join();
  return attempts.load();
}

// Host-side argmin over trajectories, annealing.hpp:134-139 (first minimum).
int orc_argmin(const double *e, int m) {
  return (int)(std::min_element(e, e + m) - e);
}

void orc_philox4x32_10(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
  philox4x32_10(ctr, key, out);
}

// qubo::Solution::save, include/model/solution.hpp:58-67: the header row of
// variable indices followed by "energy", then the 0/1 values and the energy
// at the default ostream precision (6 significant digits, "%g"). Returns the
// number of bytes written (excluding the terminator) or -1 if cap is short.
int orc_solution_csv(const char *state, int n, double energy, char *out, int cap) {
  std::string s;
  for (int i = 0; i < n; ++i) s += std::to_string(i) + ",";
  s += "energy\n";
  for (int i = 0; i < n; ++i) s += std::to_string((int)state[i]) + ",";
  char buf[64];
  std::snprintf(buf, sizeof buf, "%g", energy);
  s += buf;
  s += "\n";
  if ((int)s.size() + 1 > cap) return -1;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return (int)s.size();
}


// Replica-exchange step of parallel tempering (Swendsen and Wang, PRL 57
// (1986); Hukushima and Nemoto, J. Phys. Soc. Jpn. 65 (1996)). Not in the
// reference: its annealing benchmark recommends parallel tempering as the
// next solver (benchmarks/annealing/performance.md:52-59), so this is the
// project's own statement of the rule the GPU library implements, written
// independently of it. Chains of nt replicas; temps[c*nt + r] is the
// temperature index of replica r of chain c. Round `round` tries the adjacent
// pairs (k, k+1), k = round mod 2, k+2, ...; with `hot` the replica at k and
// `cold` the one at k+1, d = (beta[k+1] - beta[k]) * (E_cold - E_hot), and the
// pair swaps when d >= 0 or ln u < d, u = (w + 1/2) 2^-32 with w the first
// word of Philox4x32-10 at counter (k, round, c, 4 << 28) and key (seed low,
// seed high). Energies are held fixed; swaps[k] counts accepted exchanges.
void orc_pt_exchange(int chains, int nt, const double *beta, const double *e, uint64_t seed, int round0,
                     int rounds, int *temps, uint64_t *swaps) {
  std::vector<int> at((size_t)chains * nt);
  for (int c = 0; c < chains; ++c)
    for (int r = 0; r < nt; ++r) at[(size_t)c * nt + temps[(size_t)c * nt + r]] = c * nt + r;
  for (int k = 0; k + 1 < nt; ++k) swaps[k] = 0;
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (int c = 0; c < chains; ++c) {
    int *a = &at[(size_t)c * nt];
    for (int round = round0; round < round0 + rounds; ++round)
      for (int k = round % 2; k + 1 < nt; k += 2) {
        const int hot = a[k], cold = a[k + 1];
        const double d = (beta[k + 1] - beta[k]) * (e[cold] - e[hot]);
        bool swap = d >= 0.0;
        if (!swap) {
          const uint32_t ctr[4] = {(uint32_t)k, (uint32_t)round, (uint32_t)c, 4u << 28};
          uint32_t w[4];
          philox4x32_10(ctr, key, w);
          swap = std::log(((double)w[0] + 0.5) * 0x1.0p-32) < d;
        }
        if (swap) {
          std::swap(a[k], a[k + 1]);
          temps[cold] = k;
          temps[hot] = k + 1;
          ++swaps[k];
        }
      }
  }
}


// Systematic resampling step of population annealing (Hukushima and Iba,
// 2003; Machta, PRE 82 (2010)). Not in the reference (its annealing benchmark
// names population annealing as a next solver,
// benchmarks/annealing/performance.md:52-59): the project's own statement of
// the rule the GPU library implements. Weights w_i = exp(-dbeta (E_i - E_min));
// cumulative sums in 1024 blocks of L = ceil(R / 1024) consecutive replicas
// (running sum inside a block, plus the block's offset: the block totals form
// 32 groups of 32, each group summed in order, the group totals summed in
// order; offset = earlier groups' sum + earlier blocks of the group);
// W = the sum of the group totals; u = (w + 1/2) 2^-32 from
// the first word of Philox4x32-10 at counter (step, 0, 0, 5 << 28); slot j
// takes the first i (at most R - 1) with cum_i > (u + j) (W / R);
// ln Q = (-dbeta E_min) + ln(W / R).
// Built without floating-point contraction so that every product and sum
// rounds on its own, as the device code does (__dmul_rn / __dadd_rn there).
__attribute__((optimize("fp-contract=off")))
void orc_pa_resample(int R, const double *e, double dbeta, uint64_t seed, int step, int *parent, double *log_q) {
  const int B = 1024;
  const int L = (R + B - 1) / B;
  double emin = INFINITY;
  for (int i = 0; i < R; ++i) emin = std::fmin(emin, e[i]);
  std::vector<double> cum(R), tot(B, 0.0);
  for (int b = 0; b < B; ++b) {
    double run = 0.0;
    for (int i = b * L; i < std::min(R, (b + 1) * L); ++i) {
      const double x = -dbeta * (e[i] - emin);
      run += std::exp(x);
      cum[i] = run;
    }
    tot[b] = run;
  }
  // Offsets: 32 groups of 32 block totals, each summed in order, then the
  // group totals in order.
  std::vector<double> pre(B), goff(32);
  for (int g = 0; g < 32; ++g) {
    double run = 0.0;
    for (int k = 0; k < 32; ++k) {
      pre[32 * g + k] = run;
      run += tot[32 * g + k];
    }
    goff[g] = run;
  }
  double acc = 0.0;
  for (int g = 0; g < 32; ++g) {
    const double v = goff[g];
    goff[g] = acc;
    acc += v;
  }
  for (int b = 0; b < B; ++b) {
    const double off = goff[b / 32] + pre[b];
    for (int i = b * L; i < std::min(R, (b + 1) * L); ++i) cum[i] = off + cum[i];
  }
  const double m = -dbeta * emin;
  const double lg = std::log(acc / R);
  *log_q = m + lg;
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  const uint32_t ctr[4] = {(uint32_t)step, 0u, 0u, 5u << 28};
  uint32_t w[4];
  philox4x32_10(ctr, key, w);
  const double u = ((double)w[0] + 0.5) * 0x1.0p-32;
  const double stride = acc / R;
  for (int j = 0; j < R; ++j) {
    const double target = (u + j) * stride;
    const int i = (int)(std::upper_bound(cum.begin(), cum.end(), target) - cum.begin());
    parent[j] = std::min(i, R - 1);
  }
}

}  // extern "C"
