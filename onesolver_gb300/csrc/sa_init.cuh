// sa_init.cuh -- tensor-core initialisation of the dense annealing plans
// (sa_init.cu): initial spins and the FP32 local fields H = X C of all
// trajectories.
#ifndef ONESOLVER_SA_INIT_CUH_
#define ONESOLVER_SA_INIT_CUH_

#include <cstdint>

#include <cuda_runtime.h>

struct os_sa_plan;

namespace os {
namespace sa {

struct InitArgs {
  int n, nslots, ld;
  int traj_offset;
  uint32_t seed_lo, seed_hi, instance;
  const float *init_prob;  // optional warm start (n)
  const double *d64;       // diagonal (ld)
  float *h;                // fields [T][nslots/2][32] FP32 pairs
  unsigned long long *x, *xbest;
  float *e, *ebest;
  const uint8_t *init_bits; // optional initial spins [T][n] (replay mode)
};

// Split the plan's FP64 couplings into the three BF16 terms of the product
// and size its spin matrix (plan creation).
void dense_init_prepare(os_sa_plan *p, cudaStream_t s);

// Initial spins, fields and tracked energies of all trajectories; returns
// the number of kernel launches.
int dense_init_tc(os_sa_plan *p, const InitArgs &a, cudaStream_t s);

}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_INIT_CUH_
