// sa_replay.cu -- replay (verification) mode of the annealing plans.
//
// The spec check of the annealing path is a deterministic replay: one
// precomputed array of randoms fed both to the GPU kernels and to a CPU
// transcription of the reference's Metropolis loop
// (include/simulated_annealing/annealing.hpp:87-125), which must then agree
// bit for bit. The reference draws from oneMKL's philox4x32x10, whose stream
// cannot be reproduced, so the randoms come from the caller.
//
// Replay runs the production path of a plan (dense, sparse or batched):
// its execute sequence, its initialisation kernels, its sweep kernels in
// their REPLAY instantiation (sa_kernels.cuh, sa_sparse.cu) and its FP64
// resyncs, with two substitutions only: the initial spins are the caller's,
// and the attempt at site k in step `step` of trajectory t accepts when
// dE < threshold[t][step][k] (random sites: the site and threshold of
// [t][step]). The threshold is the form both acceptance rules take in the
// kernels: exp((E - E') / beta) > u is dE < -beta ln u and
// exp(-beta dE) > u is dE < -ln(u) / beta.
//
// This file holds the dense REPLAY instantiations (their own translation
// unit, compiled beside the production kernels; the batched ones are in
// sa_replay_batch.cu) and the entry points os_sa_plan_set_replay,
// os_sa_plan_trajectories and os_sa_plan_sweep_order.
#include <cstring>
#include <vector>

#include "common.cuh"
#include "sa_common.cuh"
#include "sa_kernels.cuh"
#include "sa_plan.cuh"
#include "sa_replay.cuh"

namespace os {
namespace sa {

namespace {

template <int SLOTS> void replay_tile(const DenseArgs &a, int warps, cudaStream_t s) {
  const int grid = (a.traj_count + warps - 1) / warps;
  const size_t smem = (size_t)2 * TILE_ROWS * a.ld * sizeof(float);
  OS_CUDA(cudaFuncSetAttribute(sa_dense_tile_kernel<SLOTS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  sa_dense_tile_kernel<SLOTS, true><<<grid, warps * 32, smem, s>>>(a);
}
template <int SLOTS> void replay_seq(const DenseArgs &a, int warps, cudaStream_t s) {
  const int grid = (a.traj_count + warps - 1) / warps;
  sa_dense_seq_kernel<SLOTS, true><<<grid, warps * 32, 0, s>>>(a);
}
template <int SLOTS> void replay_rand(const DenseArgs &a, int warps, cudaStream_t s) {
  const int grid = (a.traj_count + warps - 1) / warps;
  sa_dense_rand_kernel<SLOTS, true><<<grid, warps * 32, 0, s>>>(a);
}

#define OS_REPLAY_DISPATCH(cls, fn, ...)                                \
  switch (cls) {                                                        \
    case 4: fn<4>(__VA_ARGS__); break;                                  \
    case 8: fn<8>(__VA_ARGS__); break;                                  \
    case 16: fn<16>(__VA_ARGS__); break;                                \
    case 32: fn<32>(__VA_ARGS__); break;                                \
    case 64: fn<64>(__VA_ARGS__); break;                                \
    default: throw_error(OS_INVALID_ARG, "unsupported slot count %d", cls); \
  }

// Site of one lane-mask layout (dense and batched plans) as a byte.
void unpack_masks(const unsigned long long *xm, int n, char *out) {
  for (int k = 0; k < n; ++k) out[k] = (char)((xm[site_lane(k)] >> site_slot(k)) & 1ull);
}

}  // namespace

void dense_sweeps_replay(const DenseArgs &a, int slot_cls, int warps, bool sequential, cudaStream_t s) {
  if (sequential && a.ld <= TILE_MAX_LD) {
    OS_REPLAY_DISPATCH(slot_cls, replay_tile, a, warps, s);
  } else if (sequential) {
    OS_REPLAY_DISPATCH(slot_cls, replay_seq, a, warps, s);
  } else {
    OS_REPLAY_DISPATCH(slot_cls, replay_rand, a, warps, s);
  }
  OS_CUDA(cudaGetLastError());
}


}  // namespace sa
}  // namespace os

using namespace os;
using namespace os::sa;

namespace {

// Variables of each instance of a plan (one entry unless batched).
std::vector<int> plan_sizes(const os_sa_plan *p) {
  if (p->kind == 2) return batch_sizes(p);
  return std::vector<int>(1, p->n);
}

}  // namespace

extern "C" {

os_status os_sa_plan_set_replay(os_sa_plan *p, const os_sa_replay *rp) {
  return guard([&] {
    OS_REQUIRE(p != nullptr, "null plan");
    activate(p->ctx);
    OS_CUDA(cudaStreamSynchronize(p->ctx->stream));
    if (!rp) {
      p->replay = false;
      if (p->kind == 2) batch_replay_changed(p);
      return;
    }
    OS_REQUIRE(rp->init && rp->threshold, "replay needs the initial spins and the thresholds");
    const std::vector<int> sizes = plan_sizes(p);
    size_t vars = 0;  // sum over instances of T * n_k
    for (int nk : sizes) vars += (size_t)p->T * nk;
    const size_t steps = (size_t)p->steps;
    size_t nthr;
    if (p->sequential) {
      nthr = vars * steps;
    } else {
      OS_REQUIRE(rp->site, "random-site replay needs the site of every attempt");
      nthr = (size_t)p->T * steps;
      const int n = p->n;
      for (size_t i = 0; i < nthr; ++i)
        OS_REQUIRE(rp->site[i] >= 0 && rp->site[i] < n, "site[%zu] = %d outside [0, %d)", i, rp->site[i], n);
    }
    p->rp_init.alloc(vars);
    OS_CUDA(cudaMemcpy(p->rp_init.get(), rp->init, vars, cudaMemcpyHostToDevice));
    p->rp_thr.alloc(nthr);
    OS_CUDA(cudaMemcpy(p->rp_thr.get(), rp->threshold, sizeof(float) * nthr, cudaMemcpyHostToDevice));
    if (!p->sequential) {
      p->rp_site.alloc(nthr);
      OS_CUDA(cudaMemcpy(p->rp_site.get(), rp->site, sizeof(int) * nthr, cudaMemcpyHostToDevice));
    }
    p->replay = true;
    if (p->kind == 2) batch_replay_changed(p);
  });
}

os_status os_sa_plan_trajectories(os_sa_plan *p, char *final_states, char *best_states, double *energies,
                                  double *best_energies, uint64_t *accepted) {
  return guard([&] {
    OS_REQUIRE(p != nullptr, "null plan");
    activate(p->ctx);
    OS_CUDA(cudaStreamSynchronize(p->ctx->stream));
    if (p->status.count) {
      int st = 0;
      OS_CUDA(cudaMemcpy(&st, p->status.get(), sizeof st, cudaMemcpyDeviceToHost));
      if (st) throw_error(OS_TIMEOUT, "a sweep kernel's bounded wait for a coupling tile ran out");
    }
    const std::vector<int> sizes = plan_sizes(p);
    const size_t G = (size_t)p->T * sizes.size();  // trajectories of all instances
    if (accepted)
      OS_CUDA(cudaMemcpy(accepted, p->accepted.get(), sizeof(uint64_t) * G, cudaMemcpyDeviceToHost));
    if (p->kind == 1) {
      const size_t n = (size_t)p->n;
      if (final_states) OS_CUDA(cudaMemcpy(final_states, p->sx.get(), G * n, cudaMemcpyDeviceToHost));
      if (best_states) OS_CUDA(cudaMemcpy(best_states, p->sxbest.get(), G * n, cudaMemcpyDeviceToHost));
      if (energies) OS_CUDA(cudaMemcpy(energies, p->se.get(), sizeof(double) * G, cudaMemcpyDeviceToHost));
      if (best_energies)
        OS_CUDA(cudaMemcpy(best_energies, p->sebest.get(), sizeof(double) * G, cudaMemcpyDeviceToHost));
      return;
    }
    std::vector<unsigned long long> x(G * 32), xb(G * 32);
    std::vector<float> e(G), eb(G);
    OS_CUDA(cudaMemcpy(x.data(), p->x.get(), sizeof(unsigned long long) * x.size(), cudaMemcpyDeviceToHost));
    OS_CUDA(cudaMemcpy(xb.data(), p->xbest.get(), sizeof(unsigned long long) * xb.size(), cudaMemcpyDeviceToHost));
    OS_CUDA(cudaMemcpy(e.data(), p->e.get(), sizeof(float) * G, cudaMemcpyDeviceToHost));
    OS_CUDA(cudaMemcpy(eb.data(), p->ebest.get(), sizeof(float) * G, cudaMemcpyDeviceToHost));
    size_t g = 0, off = 0;
    for (int nk : sizes)
      for (int t = 0; t < p->T; ++t, ++g, off += nk) {
        if (final_states) unpack_masks(&x[g * 32], nk, final_states + off);
        if (best_states) unpack_masks(&xb[g * 32], nk, best_states + off);
        if (energies) energies[g] = e[g];
        if (best_energies) best_energies[g] = eb[g];
      }
  });
}

os_status os_sa_plan_sweep_order(const os_sa_plan *p, int32_t *order) {
  return guard([&] {
    OS_REQUIRE(p && order, "null argument");
    OS_REQUIRE(p->sequential, "a random-site plan has no fixed sweep order");
    if (p->kind == 1) {
      std::memcpy(order, p->host_color_sites.data(), sizeof(int32_t) * p->host_color_sites.size());
      return;
    }
    size_t off = 0;
    for (int nk : plan_sizes(p)) {
      const int nslots = slots_for(nk);
      for (int s = 0; s < nslots; ++s)
        for (int l = 0; l < 32; ++l) {
          const int k = slot_site(s, l);
          if (k < nk) order[off++] = k;
        }
    }
  });
}

}  // extern "C"
