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

// Dense instances are staged for the sweep kernels on the device
// (stage_dense_device). Sites are padded to a multiple of 128 (nslots =
// ld / 32 slots, a multiple of 4); padding sites have zero couplings and
// never flip. The FP32 coupling rows are stored in slot order: row
// p = s*32 + l holds the couplings of site ((s >> 2) << 7) + (l << 2) +
// (s & 3) (the site lane l owns in slot s), columns in site order; the FP64
// rows (resync) are in site order.
inline int slots_for(int n) { return (n + 127) / 128 * 4; }

// Power-of-two slot count (>= 4) of the kernel instance that serves nslots.
inline int slot_class(int nslots) {
  int s = 4;
  while (s < nslots) s <<= 1;
  return s;
}

// Device staging of one dense instance from its matrix as given (d_f, n x n,
// already in HBM): slot-ordered FP32 rows, site-ordered FP64 rows, both
// diagonals; *bad accumulates the count of non-finite coefficients on or
// above the diagonal (sa_dense.cu).
void stage_dense_device(const double *d_f, int n, int ld, float *c32, double *c64, float *d32, double *d64,
                        int *bad, cudaStream_t s);

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
