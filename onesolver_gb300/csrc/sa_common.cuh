// sa_common.cuh -- staging and shared pieces of the simulated-annealing
// kernels: the dense FP32/FP64 layouts, schedule validation and the host
// argmin over trajectories.
#ifndef ONESOLVER_SA_COMMON_CUH_
#define ONESOLVER_SA_COMMON_CUH_

#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace os {
namespace sa {

constexpr int MAX_DENSE_N = 2048;  // 64 field slots per lane

// Dense instance staged for the sweep kernels. Sites are padded to a
// multiple of 128 (nslots = ld / 32 slots, a multiple of 4); padding sites
// have zero couplings and never flip. The FP32 coupling rows are stored in
// slot order: row p = s*32 + l holds the couplings of site
// ((s >> 2) << 7) + (l << 2) + (s & 3) (the site lane l owns in slot s),
// columns in site order.
struct DenseHost {
  int n = 0, nslots = 0, ld = 0;
  std::vector<float> c32;    // ld*ld couplings, zero diagonal, rows in slot order
  std::vector<float> d32;    // ld diagonal (linear) terms
  std::vector<double> c64;   // ld*ld FP64 couplings, zero diagonal
  std::vector<double> d64;   // ld
  std::vector<double> f;     // n*n flattened matrix as given (re-score)
};

inline int slots_for(int n) { return (n + 127) / 128 * 4; }

// Power-of-two slot count (>= 4) of the kernel instance that serves nslots.
inline int slot_class(int nslots) {
  int s = 4;
  while (s < nslots) s <<= 1;
  return s;
}

inline int slot_site_host(int p) {
  const int s = p >> 5, l = p & 31;
  return ((s >> 2) << 7) + (l << 2) + (s & 3);
}

inline void stage_dense(const os_qubo_dense *q, DenseHost &h) {
  const int n = q->n;
  h.n = n;
  h.nslots = slots_for(n);
  h.ld = h.nslots * 32;
  const size_t ld = h.ld;
  h.c32.assign(ld * ld, 0.f);
  h.c64.assign(ld * ld, 0.0);
  h.d32.assign(ld, 0.f);
  h.d64.assign(ld, 0.0);
  h.f.assign(q->f, q->f + (size_t)n * n);
  for (int i = 0; i < n; ++i) {
    const double di = q->f[(size_t)i * n + i];
    OS_REQUIRE(std::isfinite(di), "coefficient (%d,%d) is not finite", i, i);
    h.d64[i] = di;
    h.d32[i] = (float)di;
    for (int j = i + 1; j < n; ++j) {
      const double v = q->f[(size_t)i * n + j];
      OS_REQUIRE(std::isfinite(v), "coefficient (%d,%d) is not finite", i, j);
      h.c64[i * ld + j] = h.c64[j * ld + i] = v;
    }
  }
  for (size_t p = 0; p < ld; ++p) {
    const int site = slot_site_host((int)p);
    if (site >= n) continue;
    for (int j = 0; j < n; ++j) h.c32[p * ld + j] = (float)h.c64[(size_t)site * ld + j];
  }
}

inline void check_schedule(const os_sa_params *p) {
  OS_REQUIRE(p != nullptr, "null parameters");
  OS_REQUIRE(p->beta != nullptr && p->num_iter > 0, "empty beta schedule");
  OS_REQUIRE(p->sweeps_per_beta > 0, "sweeps_per_beta must be positive");
  OS_REQUIRE(p->num_tries > 0, "num_tries must be positive");
  OS_REQUIRE(p->acceptance == OS_ACCEPT_REFERENCE || p->acceptance == OS_ACCEPT_PHYSICAL,
             "unknown acceptance rule %d", p->acceptance);
  OS_REQUIRE(p->site_order == OS_SITES_RANDOM || p->site_order == OS_SITES_SEQUENTIAL,
             "unknown site order %d", p->site_order);
  OS_REQUIRE(p->resync_every >= -1, "resync_every must be >= -1");
  for (int i = 0; i < p->num_iter; ++i)
    OS_REQUIRE(!std::isnan(p->beta[i]), "beta[%d] is NaN", i);
}

// First minimum over trajectories (annealing.hpp:134-139).
inline int argmin_first(const std::vector<double> &e) {
  int best = 0;
  for (int i = 1; i < (int)e.size(); ++i)
    if (e[i] < e[best]) best = i;
  return best;
}

}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_COMMON_CUH_
