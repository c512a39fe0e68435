// sa_plan.cuh -- the device-resident annealing plan behind os_sa_plan.
#ifndef ONESOLVER_SA_PLAN_CUH_
#define ONESOLVER_SA_PLAN_CUH_

#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace os {
namespace sa {
struct BatchState;
}  // namespace sa
}  // namespace os

struct os_sa_plan {
  os_ctx *ctx = nullptr;
  int kind = 0;                 // 0 dense, 1 sparse, 2 batched dense
  os::sa::BatchState *batch = nullptr;
  int n = 0, T = 0;
  int spb = 1, num_iter = 0, steps = 0, chunk = 0;
  unsigned long long seed = 0;
  int acceptance = 0;
  bool sequential = true;
  unsigned long long attempts_per_step = 1;
  int launches = 0;
  int warps = 4;
  bool tiled = false;
  bool drift_off = false;                   // resync_every == -1: no FP64 resync at all
  os::DevBuf<int> status;                   // bounded-wait failures
  // CUDA events around every sweep launch of the last execute (kernel time)
  std::vector<cudaEvent_t> sweep_ev;
  int sweep_ev_used = 0;
  ~os_sa_plan() {
    for (auto e : sweep_ev) cudaEventDestroy(e);
  }
  // Events for sweep launch i (start = 2i, end = 2i+1).
  cudaEvent_t event(int k) {
    while ((int)sweep_ev.size() <= k) {
      cudaEvent_t e;
      OS_CUDA(cudaEventCreate(&e));
      sweep_ev.push_back(e);
    }
    return sweep_ev[k];
  }

  // schedule and results
  os::DevBuf<double> beta;
  os::DevBuf<float> init_prob;
  os::DevBuf<unsigned long long> drift;     // FP64 bits of the max drift
  os::DevBuf<unsigned long long> accepted;  // per trajectory
  os::DevBuf<uint8_t> states;               // best states, T x n bytes
  os::DevBuf<double> e64;                   // re-scored best energies
  os::DevBuf<double> f;                     // n x n flattened matrix (re-score)

  // dense
  int nslots = 0, ld = 0, slot_cls = 1;
  os::DevBuf<float> c32, d32, h, e, ebest;
  os::DevBuf<double> c64, d64;
  os::DevBuf<unsigned long long> x, xbest;
  os::DevBuf<__nv_bfloat16> bsplit, xmat;   // tensor-core initialisation operands
  alignas(64) unsigned char init_tmap[2][128];  // TMA tensor maps of xmat and bsplit (CUtensorMap)

  // sparse
  int ncolors = 0, nnz = 0, traj_per_cta = 0, deg_max = 1;
  cudaEvent_t ready = nullptr;  // dense plans: buffers allocated and filled (creation stream)
  os::DevBuf<int> row_ptr, col, color_sites, color_ptr;
  os::DevBuf<int2> ell;                     // padded neighbour table (site, coupling bits)
  os::DevBuf<float> val32, diag32;
  os::DevBuf<double> val64, diag64;
  os::DevBuf<float> sh;                     // fields [T][n]
  os::DevBuf<uint8_t> sx, sxbest;           // spins [T][n]
  os::DevBuf<double> se, sebest;            // energies [T]
  std::vector<int> host_row_ptr, host_col;
  std::vector<double> host_val, host_diag;
  std::vector<int> host_color_sites;        // sweep order: the sites colour by colour

  // Replay (verification) mode, os_sa_plan_set_replay: caller-given initial
  // spins and per-attempt thresholds (and sites, random order) take the
  // place of the Philox draws in the same kernels.
  bool replay = false;
  os::DevBuf<uint8_t> rp_init;
  os::DevBuf<float> rp_thr;
  os::DevBuf<int> rp_site;
};

void os_sa_plan_common(os_sa_plan *p, os_ctx *ctx, const os_sa_params *prm, int n);

namespace os {
namespace sa {
void execute_dense(os_sa_plan *p);
void execute_sparse(os_sa_plan *p);
void execute_batched(os_sa_plan *p);
void release_batch(os_sa_plan *p);
// Batched plans: variables of each instance, and a change of replay mode
// (drops the captured execute graph so the next execute captures the
// kernels of the new mode).
std::vector<int> batch_sizes(const os_sa_plan *p);
void batch_replay_changed(os_sa_plan *p);
}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_PLAN_CUH_
