// sa_dense.cu -- dense simulated annealing: the device-resident plan, the
// os_sa_run entry point and os_sa_verify (the reference's one-thread-per-
// trajectory loop with caller-given randoms).
//
// Replaces sa::anneal (include/simulated_annealing/annealing.hpp:55-140).
// One anneal is: draw the initial spins and compute the FP64 fields; run the
// schedule in chunks of resync_every steps, with an FP64 field resync (and
// drift measurement) between chunks; re-score every trajectory's best state
// with the reference's FP64 energy function; take the first minimum on the
// host (annealing.hpp:134-139).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "rescore.cuh"
#include "sa_common.cuh"
#include "sa_kernels.cuh"
#include "sa_init.cuh"
#include "sa_plan.cuh"
#include "sa_replay.cuh"

namespace os {
namespace sa {

// Deterministic verification: one thread per trajectory replays the
// reference's kernel body (annealing.hpp:87-125) with caller-given randoms.
// Fields are FP64 and the energy is the reference's initial FP64 energy plus
// the FP64 deltas, which equals the reference's per-attempt recomputation
// exactly whenever the coefficients are integers.
__global__ void sa_verify_kernel(const double *__restrict__ f, int n, const double *__restrict__ beta,
                                 int num_iter, int spb, int T, int acceptance,
                                 const uint8_t *__restrict__ init, const int *__restrict__ site,
                                 const double *__restrict__ u, double *__restrict__ hbuf,
                                 uint8_t *__restrict__ cur, uint8_t *__restrict__ best,
                                 double *__restrict__ ebest, double *__restrict__ efinal,
                                 long long *__restrict__ acc_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const long long S = (long long)num_iter * spb;
  uint8_t *x = cur + (size_t)t * n;
  uint8_t *bx = best + (size_t)t * n;
  double *h = hbuf + (size_t)t * n;
  for (int i = 0; i < n; ++i) x[i] = bx[i] = init[(size_t)t * n + i] ? 1 : 0;
  // Fields from the symmetric couplings (f holds the upper triangle).
  for (int j = 0; j < n; ++j) {
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
      if (i == j || !x[i]) continue;
      acc += i < j ? f[(size_t)i * n + j] : f[(size_t)j * n + i];
    }
    h[j] = acc;
  }
  double E = rescore_energy(f, n, x);
  double Eb = E;
  long long accepted = 0;
  for (int it = 0; it < num_iter; ++it) {
    const double b = beta[it];
    for (int sw = 0; sw < spb; ++sw) {
      const long long a = (long long)it * spb + sw;
      const int k = site[(size_t)t * S + a];
      const double uu = u[(size_t)t * S + a];
      const double loc = f[(size_t)k * n + k] + h[k];
      const double dE = x[k] ? -loc : loc;
      const double Enew = E + dE;
      bool accept;
      if (Enew < E)
        accept = true;
      else if (acceptance == OS_ACCEPT_REFERENCE)
        accept = exp((E - Enew) / b) > uu;
      else
        accept = exp(-b * (Enew - E)) > uu;
      if (accept) {
        x[k] ^= 1;
        const double sgn = x[k] ? 1.0 : -1.0;
        for (int j = 0; j < n; ++j) {
          if (j == k) continue;
          h[j] += sgn * (j < k ? f[(size_t)j * n + k] : f[(size_t)k * n + j]);
        }
        E = Enew;
        ++accepted;
      }
      if (E < Eb) {
        Eb = E;
        for (int i = 0; i < n; ++i) bx[i] = x[i];
      }
    }
  }
  ebest[t] = Eb;
  efinal[t] = E;
  acc_out[t] = accepted;
}

template <int SLOTS> void launch_seq(const DenseArgs &a, int warps, cudaStream_t s) {
  const int grid = (a.traj_count + warps - 1) / warps;
  sa_dense_seq_kernel<SLOTS><<<grid, warps * 32, 0, s>>>(a);
}
template <int SLOTS> void launch_tile(const DenseArgs &a, int warps, cudaStream_t s) {
  // ceil(T / W) CTAs; each takes T / grid trajectories, rounded (<= W).
  const int grid = (a.traj_count + warps - 1) / warps;
  const size_t smem = (size_t)2 * TILE_ROWS * a.ld * sizeof(float);
  OS_CUDA(cudaFuncSetAttribute(sa_dense_tile_kernel<SLOTS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  sa_dense_tile_kernel<SLOTS><<<grid, warps * 32, smem, s>>>(a);
}
template <int SLOTS> void launch_rand(const DenseArgs &a, int warps, cudaStream_t s) {
  const int grid = (a.traj_count + warps - 1) / warps;
  sa_dense_rand_kernel<SLOTS><<<grid, warps * 32, 0, s>>>(a);
}
template <int SLOTS> void launch_resync(const ResyncArgs &a, int warps, cudaStream_t s) {
  const int grid = (a.traj_count + warps - 1) / warps;
  sa_dense_resync_kernel<SLOTS><<<grid, warps * 32, 0, s>>>(a);
}

#define OS_SLOT_DISPATCH(cls, fn, ...)                                  \
  switch (cls) {                                                        \
    case 4: fn<4>(__VA_ARGS__); break;                                  \
    case 8: fn<8>(__VA_ARGS__); break;                                  \
    case 16: fn<16>(__VA_ARGS__); break;                                \
    case 32: fn<32>(__VA_ARGS__); break;                                \
    case 64: fn<64>(__VA_ARGS__); break;                                \
    default: throw_error(OS_INVALID_ARG, "unsupported slot count %d", cls); \
  }

void dense_sweeps(const DenseArgs &a, int slot_cls, int warps, bool sequential, cudaStream_t s) {
  if (sequential && a.ld <= TILE_MAX_LD) {
    OS_SLOT_DISPATCH(slot_cls, launch_tile, a, warps, s);
  } else if (sequential) {
    OS_SLOT_DISPATCH(slot_cls, launch_seq, a, warps, s);
  } else {
    OS_SLOT_DISPATCH(slot_cls, launch_rand, a, warps, s);
  }
  OS_CUDA(cudaGetLastError());
}

void dense_resync(const ResyncArgs &a, int slot_cls, int warps, cudaStream_t s) {
  warps = warps > 4 ? 4 : warps;
  OS_SLOT_DISPATCH(slot_cls, launch_resync, a, warps, s);
  OS_CUDA(cudaGetLastError());
}

// Warps (trajectories) per CTA: spread small trajectory counts over all SMs;
// larger CTAs share each staged coupling tile among more trajectories.
int dense_warps(int traj, int sm_count, bool tiled) {
  if (tiled) {
    int w = (traj + sm_count - 1) / sm_count;
    return w < 1 ? 1 : (w > 8 ? 8 : w);
  }
  if (traj <= sm_count * 4) return 1;
  if (traj <= sm_count * 16) return 2;
  return 4;
}

// Device staging of a dense instance from the matrix as given (already in
// HBM for the re-score).
// c32 row p (slot order) holds the couplings of site slot_site(p) with every
// site; c64 row i (site order) those of site i; couplings are the upper
// triangle of f mirrored, the diagonal is zero and padding sites are zero.
// A warp per row; *bad counts non-finite coefficients on or above the
// diagonal.
__global__ void __launch_bounds__(256) stage_dense_kernel(const double *__restrict__ f, int n, int ld,
                                                          float *__restrict__ c32, double *__restrict__ c64,
                                                          float *__restrict__ d32, double *__restrict__ d64,
                                                          int *__restrict__ bad) {
  const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= ld) return;
  const int site = slot_site(row >> 5, row & 31);  // c32 row `row`
  int nonfinite = 0;
  for (int j = lane; j < ld; j += 32) {
    double a = 0.0, b = 0.0;
    if (row < n && j < n && j != row) {
      a = row < j ? f[(size_t)row * n + j] : f[(size_t)j * n + row];
      if (row < j && !isfinite(a)) ++nonfinite;
    }
    if (site < n && j < n && j != site) b = site < j ? f[(size_t)site * n + j] : f[(size_t)j * n + site];
    c64[(size_t)row * ld + j] = a;
    c32[(size_t)row * ld + j] = (float)b;
  }
  if (lane == 0) {
    const double d = row < n ? f[(size_t)row * n + row] : 0.0;
    if (!isfinite(d)) ++nonfinite;
    d64[row] = d;
    d32[row] = (float)d;
  }
  if (nonfinite) atomicAdd(bad, nonfinite);
}

void stage_dense_device(const double *d_f, int n, int ld, float *c32, double *c64, float *d32, double *d64,
                        int *bad, cudaStream_t s) {
  stage_dense_kernel<<<(unsigned)((ld + 7) / 8), 256, 0, s>>>(d_f, n, ld, c32, c64, d32, d64, bad);
  OS_CUDA(cudaGetLastError());
}

void plan_create_dense(os_sa_plan *p, const os_qubo_dense *q) {
  OS_REQUIRE(q && q->f, "null QUBO");
  OS_REQUIRE(q->n >= 1 && q->n <= MAX_DENSE_N, "dense annealing supports 1..%d variables (got %d)",
             MAX_DENSE_N, q->n);
  struct {
    int n, nslots, ld;
  } hst;
  hst.n = q->n;
  hst.nslots = slots_for(q->n);
  hst.ld = hst.nslots * 32;
  p->n = hst.n;
  p->nslots = hst.nslots;
  p->ld = hst.ld;
  p->slot_cls = slot_class(hst.nslots);
  const size_t T = p->T;
  const size_t ld = hst.ld;
  // The plan's device buffers come stream-ordered from the context's pool
  // (freed in order at destruction, the blocks kept for the next plan).
  cudaStream_t s = p->ctx->stream;
  cudaMemPool_t mp = p->ctx->pool;
  p->c32.alloc_on(ld * ld, mp, s);
  p->d32.alloc_on(ld, mp, s);
  p->c64.alloc_on(ld * ld, mp, s);
  p->d64.alloc_on(ld, mp, s);
  p->f.alloc_on((size_t)hst.n * hst.n, mp, s);
  OS_CUDA(cudaMemcpyAsync(p->f.get(), q->f, sizeof(double) * hst.n * hst.n, cudaMemcpyHostToDevice, s));
  DevBuf<int> bad;
  bad.alloc_on(1, mp, s);
  OS_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(int), s));
  stage_dense_kernel<<<(unsigned)((ld + 7) / 8), 256, 0, s>>>(p->f.get(), hst.n, hst.ld, p->c32.get(), p->c64.get(),
                                                             p->d32.get(), p->d64.get(), bad.get());
  OS_CUDA(cudaGetLastError());
  int nbad = 0;
  OS_CUDA(cudaMemcpyAsync(&nbad, bad.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  OS_CUDA(cudaStreamSynchronize(s));
  OS_REQUIRE(nbad == 0, "the QUBO has %d non-finite coefficients", nbad);
  p->h.alloc_on(T * hst.nslots * 32, mp, s);
  dense_init_prepare(p, s);
  p->x.alloc_on(T * 32, mp, s);
  p->xbest.alloc_on(T * 32, mp, s);
  p->e.alloc_on(T, mp, s);
  p->ebest.alloc_on(T, mp, s);
  p->accepted.alloc_on(T, mp, s);
  p->states.alloc_on(T * (size_t)hst.n, mp, s);
  p->e64.alloc_on(T, mp, s);
  p->tiled = p->sequential && hst.ld <= TILE_MAX_LD;
  p->warps = dense_warps((int)T, p->ctx->sm_count, p->tiled);
  p->status.alloc_on(1, mp, s);
  OS_CUDA(cudaMemsetAsync(p->status.get(), 0, sizeof(int), s));
  if (!p->ready) OS_CUDA(cudaEventCreateWithFlags(&p->ready, cudaEventDisableTiming));
  OS_CUDA(cudaEventRecord(p->ready, s));  // an execution on another stream waits for it
}

ResyncArgs dense_resync_args(os_sa_plan *p, int init) {
  ResyncArgs r{};
  r.c64 = p->c64.get();
  r.d64 = p->d64.get();
  r.n = p->n;
  r.nslots = p->nslots;
  r.ld = p->ld;
  r.init = init;
  r.init_prob = p->init_prob.count ? p->init_prob.get() : nullptr;
  r.traj_count = p->T;
  r.traj_offset = 0;
  r.seed_lo = (uint32_t)p->seed;
  r.seed_hi = (uint32_t)(p->seed >> 32);
  r.instance = 0;
  r.h = p->h.get();
  r.x = p->x.get();
  r.xbest = p->xbest.get();
  r.e = p->e.get();
  r.ebest = p->ebest.get();
  r.drift_bits = p->drift.get();
  return r;
}

InitArgs dense_init_args(os_sa_plan *p) {
  InitArgs a{};
  a.n = p->n;
  a.nslots = p->nslots;
  a.ld = p->ld;
  a.traj_offset = 0;
  a.seed_lo = (uint32_t)p->seed;
  a.seed_hi = (uint32_t)(p->seed >> 32);
  a.instance = 0;
  a.init_prob = p->init_prob.count ? p->init_prob.get() : nullptr;
  a.d64 = p->d64.get();
  a.h = p->h.get();
  a.x = p->x.get();
  a.xbest = p->xbest.get();
  a.e = p->e.get();
  a.ebest = p->ebest.get();
  a.init_bits = p->replay ? p->rp_init.get() : nullptr;
  return a;
}

DenseArgs dense_args(os_sa_plan *p) {
  DenseArgs a{};
  a.c = p->c32.get();
  a.diag = p->d32.get();
  a.n = p->n;
  a.nslots = p->nslots;
  a.ld = p->ld;
  a.spb = p->spb;
  a.beta = p->beta.get();
  a.acceptance = p->acceptance;
  a.traj_count = p->T;
  a.traj_offset = 0;
  a.seed_lo = (uint32_t)p->seed;
  a.seed_hi = (uint32_t)(p->seed >> 32);
  a.instance = 0;
  a.h = p->h.get();
  a.x = p->x.get();
  a.xbest = p->xbest.get();
  a.e = p->e.get();
  a.ebest = p->ebest.get();
  a.accepted = p->accepted.get();
  a.status = p->status.get();
  a.thr = p->replay ? p->rp_thr.get() : nullptr;
  a.rsite = p->replay && !p->sequential ? p->rp_site.get() : nullptr;
  a.nsteps = p->steps;
  return a;
}

// Trajectories per CTA of the staged-tile sweep: every CTA streams the whole
// coupling matrix from L2 once per sweep, so more trajectories per CTA mean
// less tile traffic but fewer SMs and more warps per scheduler. Time a few
// sweeps of each candidate on the plan's own instance and keep the fastest
// (execute re-initialises every trajectory afterwards).
constexpr int DENSE_PROBE_STEPS = 8;
int autotune_dense_warps(os_sa_plan *p) {
  const int w0 = dense_warps(p->T, p->ctx->sm_count, true);
  if (!p->tiled || p->T <= w0) return w0;
  const auto key = std::make_tuple(p->ld, p->T, p->acceptance);
  auto hit = p->ctx->dense_warps.find(key);
  if (hit != p->ctx->dense_warps.end()) return hit->second;
  cudaStream_t s = p->ctx->stream;
  OS_CUDA(cudaMemsetAsync(p->status.get(), 0, sizeof(int), s));
  dense_init_tc(p, dense_init_args(p), s);
  DenseArgs a = dense_args(p);
  a.step_begin = 0;
  a.step_end = std::min(DENSE_PROBE_STEPS, p->steps);
  cudaEvent_t e0, e1;
  OS_CUDA(cudaEventCreate(&e0));
  OS_CUDA(cudaEventCreate(&e1));
  int best_w = w0;
  float best_ms = -1.f;
  for (int W = w0; W <= 16 && W <= 4 * w0; W *= 2) {
    OS_CUDA(cudaEventRecord(e0, s));
    dense_sweeps(a, p->slot_cls, W, true, s);
    OS_CUDA(cudaEventRecord(e1, s));
    OS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    OS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (best_ms < 0.f || ms < best_ms) {
      best_w = W;
      best_ms = ms;
    }
    if (W * 2 > p->T) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  p->ctx->dense_warps[key] = best_w;
  return best_w;
}

void execute_dense(os_sa_plan *p) {
  cudaStream_t s = p->ctx->stream;
  p->launches = 0;
  OS_CUDA(cudaMemsetAsync(p->accepted.get(), 0, sizeof(unsigned long long) * p->T, s));
  OS_CUDA(cudaMemsetAsync(p->drift.get(), 0, sizeof(unsigned long long), s));
  ResyncArgs r = dense_resync_args(p, 0);
  p->launches += dense_init_tc(p, dense_init_args(p), s);

  DenseArgs a = dense_args(p);
  OS_CUDA(cudaMemsetAsync(p->status.get(), 0, sizeof(int), s));
  const int chunk = p->chunk;
  p->sweep_ev_used = 0;
  for (int s0 = 0; s0 < p->steps; s0 += chunk) {
    a.step_begin = s0;
    a.step_end = std::min(p->steps, s0 + chunk);
    OS_CUDA(cudaEventRecord(p->event(2 * p->sweep_ev_used), s));
    if (p->replay)
      dense_sweeps_replay(a, p->slot_cls, p->warps, p->sequential, s);
    else
      dense_sweeps(a, p->slot_cls, p->warps, p->sequential, s);
    OS_CUDA(cudaEventRecord(p->event(2 * p->sweep_ev_used + 1), s));
    ++p->sweep_ev_used;
    ++p->launches;
    if (!p->drift_off) {
      dense_resync(r, p->slot_cls, p->warps, s);
      ++p->launches;
    }
  }
  const size_t total = (size_t)p->T * p->n;
  unpack_states_kernel<<<(unsigned)ceil_div_u64(total, 256), 256, 0, s>>>(p->xbest.get(), p->n, p->T,
                                                                        p->states.get());
  OS_CUDA(cudaGetLastError());
  launch_rescore_warp(p->f.get(), p->n, p->states.get(), p->T, p->e64.get(), s);
  p->launches += 2;
}

}  // namespace sa
}  // namespace os

using namespace os;
using namespace os::sa;

// Common plan set-up: schedule, seeds, chunking.
void os_sa_plan_common(os_sa_plan *p, os_ctx *ctx, const os_sa_params *prm, int n) {
  p->ctx = ctx;
  p->T = (int)prm->num_tries;
  p->spb = prm->sweeps_per_beta;
  p->num_iter = prm->num_iter;
  const long long steps = (long long)prm->num_iter * prm->sweeps_per_beta;
  OS_REQUIRE(steps < (1ll << 31), "too many steps (%lld)", steps);
  p->steps = (int)steps;
  p->chunk = prm->resync_every > 0 ? prm->resync_every : p->steps;
  p->drift_off = prm->resync_every < 0;
  p->seed = prm->seed;
  p->acceptance = prm->acceptance;
  p->sequential = prm->site_order == OS_SITES_SEQUENTIAL;
  p->attempts_per_step = p->sequential ? (unsigned long long)n : 1ull;
  p->beta.alloc(prm->num_iter);
  OS_CUDA(cudaMemcpy(p->beta.get(), prm->beta, sizeof(double) * prm->num_iter, cudaMemcpyHostToDevice));
  if (prm->init_prob) {
    for (int i = 0; i < n; ++i)
      OS_REQUIRE(prm->init_prob[i] >= 0.f && prm->init_prob[i] <= 1.f, "init_prob[%d] outside [0,1]", i);
    p->init_prob.alloc(n);
    OS_CUDA(cudaMemcpy(p->init_prob.get(), prm->init_prob, sizeof(float) * n, cudaMemcpyHostToDevice));
  }
  p->drift.alloc(1);
}

os_status os_sa_plan_result(os_sa_plan *p, os_sa_result *res) {
  return guard([&] {
    OS_REQUIRE(p && res, "null argument");
    OS_REQUIRE(p->kind != 2, "batched plans return one result per instance (os_sa_plan_result_batched)");
    activate(p->ctx);
    cudaStream_t s = p->ctx->stream;
    OS_CUDA(cudaStreamSynchronize(s));
    const int T = p->T, n = p->n;
    if (p->status.count) {
      int st = 0;
      OS_CUDA(cudaMemcpy(&st, p->status.get(), sizeof st, cudaMemcpyDeviceToHost));
      if (st) throw_error(OS_TIMEOUT, "a sweep kernel's bounded wait for a coupling tile ran out");
    }
    std::vector<double> e(T);
    OS_CUDA(cudaMemcpy(e.data(), p->e64.get(), sizeof(double) * T, cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> acc(T);
    OS_CUDA(cudaMemcpy(acc.data(), p->accepted.get(), sizeof(unsigned long long) * T, cudaMemcpyDeviceToHost));
    unsigned long long drift_bits = 0;
    OS_CUDA(cudaMemcpy(&drift_bits, p->drift.get(), sizeof drift_bits, cudaMemcpyDeviceToHost));
    const int best = argmin_first(e);
    if (res->state)
      OS_CUDA(cudaMemcpy(res->state, p->states.get() + (size_t)best * n, n, cudaMemcpyDeviceToHost));
    if (res->traj_states)
      OS_CUDA(cudaMemcpy(res->traj_states, p->states.get(), (size_t)T * n, cudaMemcpyDeviceToHost));
    if (res->traj_energies) std::memcpy(res->traj_energies, e.data(), sizeof(double) * T);
    res->energy = e[best];
    double drift;
    std::memcpy(&drift, &drift_bits, sizeof drift);
    res->max_field_drift = p->drift_off ? -1.0 : drift;
    res->attempts = (unsigned long long)p->steps * p->attempts_per_step * (unsigned long long)T;
    unsigned long long total = 0;
    for (auto v : acc) total += v;
    res->accepted = total;
  });
}

extern "C" {

os_status os_sa_plan_create_dense(os_ctx *ctx, const os_qubo_dense *qubo, const os_sa_params *params,
                                  os_sa_plan **out) {
  return guard([&] {
    OS_REQUIRE(out != nullptr, "null output");
    check_schedule(params);
    OS_REQUIRE(qubo != nullptr, "null QUBO");
    activate(ctx);
    auto *p = new os_sa_plan();
    try {
      p->kind = 0;
      os_sa_plan_common(p, ctx, params, qubo->n);
      plan_create_dense(p, qubo);
      p->warps = autotune_dense_warps(p);
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

os_status os_sa_plan_execute(os_sa_plan *p) {
  return guard([&] {
    OS_REQUIRE(p != nullptr, "null plan");
    activate(p->ctx);
    if (p->ready) OS_CUDA(cudaStreamWaitEvent(p->ctx->stream, p->ready, 0));
    if (p->kind == 0)
      execute_dense(p);
    else if (p->kind == 1)
      execute_sparse(p);
    else
      execute_batched(p);
  });
}

int32_t os_sa_plan_launches(const os_sa_plan *p) { return p ? p->launches : 0; }

os_status os_sa_plan_kernel_ms(os_sa_plan *p, float *ms) {
  return guard([&] {
    OS_REQUIRE(p && ms, "null argument");
    activate(p->ctx);
    float total = 0.f;
    for (int i = 0; i < p->sweep_ev_used; ++i) {
      float t = 0.f;
      OS_CUDA(cudaEventSynchronize(p->sweep_ev[2 * i + 1]));
      OS_CUDA(cudaEventElapsedTime(&t, p->sweep_ev[2 * i], p->sweep_ev[2 * i + 1]));
      total += t;
    }
    *ms = total;
  });
}

void os_sa_plan_destroy(os_sa_plan *p) {
  if (!p) return;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  release_batch(p);
  if (p->ready) cudaEventDestroy(p->ready);
  delete p;
}

os_status os_sa_run(os_ctx *ctx, const os_qubo_dense *qubo, const os_sa_params *params,
                    os_sa_result *result) {
  os_sa_plan *plan = nullptr;
  os_status st = os_sa_plan_create_dense(ctx, qubo, params, &plan);
  if (st != OS_OK) return st;
  st = os_sa_plan_execute(plan);
  if (st == OS_OK) st = os_sa_plan_result(plan, result);
  os_sa_plan_destroy(plan);
  return st;
}

os_status os_sa_verify(os_ctx *ctx, const os_qubo_dense *qubo, const double *beta, int32_t num_iter,
                       int32_t sweeps_per_beta, uint32_t num_tries, int32_t acceptance,
                       const char *init, const int32_t *site, const double *u, char *best_states,
                       double *best_energies, char *final_states, double *final_energies,
                       int64_t *accept_count) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(qubo && qubo->f && qubo->n >= 1, "bad QUBO");
    OS_REQUIRE(beta && num_iter > 0 && sweeps_per_beta > 0 && num_tries > 0, "bad schedule");
    OS_REQUIRE(init && site && u, "null random arrays");
    OS_REQUIRE(acceptance == OS_ACCEPT_REFERENCE || acceptance == OS_ACCEPT_PHYSICAL,
               "unknown acceptance rule %d", acceptance);
    const int n = qubo->n, T = (int)num_tries;
    const size_t S = (size_t)num_iter * sweeps_per_beta;
    for (size_t i = 0; i < S * T; ++i)
      OS_REQUIRE(site[i] >= 0 && site[i] < n, "site[%zu] = %d outside [0, n)", i, site[i]);
    cudaStream_t s = ctx->stream;
    DevBuf<double> d_f, d_beta, d_u, d_h, d_eb, d_ef;
    DevBuf<int> d_site;
    DevBuf<uint8_t> d_init, d_cur, d_best;
    DevBuf<long long> d_acc;
    d_f.alloc((size_t)n * n);
    d_beta.alloc(num_iter);
    d_u.alloc(S * T);
    d_site.alloc(S * T);
    d_h.alloc((size_t)T * n);
    d_init.alloc((size_t)T * n);
    d_cur.alloc((size_t)T * n);
    d_best.alloc((size_t)T * n);
    d_eb.alloc(T);
    d_ef.alloc(T);
    d_acc.alloc(T);
    OS_CUDA(cudaMemcpyAsync(d_f.get(), qubo->f, sizeof(double) * n * n, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemcpyAsync(d_beta.get(), beta, sizeof(double) * num_iter, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemcpyAsync(d_u.get(), u, sizeof(double) * S * T, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemcpyAsync(d_site.get(), site, sizeof(int) * S * T, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemcpyAsync(d_init.get(), init, (size_t)T * n, cudaMemcpyHostToDevice, s));
    sa_verify_kernel<<<(T + 63) / 64, 64, 0, s>>>(d_f.get(), n, d_beta.get(), num_iter, sweeps_per_beta, T,
                                                  acceptance, d_init.get(), d_site.get(), d_u.get(), d_h.get(),
                                                  d_cur.get(), d_best.get(), d_eb.get(), d_ef.get(), d_acc.get());
    OS_CUDA(cudaGetLastError());
    if (best_states)
      OS_CUDA(cudaMemcpyAsync(best_states, d_best.get(), (size_t)T * n, cudaMemcpyDeviceToHost, s));
    if (final_states)
      OS_CUDA(cudaMemcpyAsync(final_states, d_cur.get(), (size_t)T * n, cudaMemcpyDeviceToHost, s));
    if (best_energies)
      OS_CUDA(cudaMemcpyAsync(best_energies, d_eb.get(), sizeof(double) * T, cudaMemcpyDeviceToHost, s));
    if (final_energies)
      OS_CUDA(cudaMemcpyAsync(final_energies, d_ef.get(), sizeof(double) * T, cudaMemcpyDeviceToHost, s));
    if (accept_count)
      OS_CUDA(cudaMemcpyAsync(accept_count, d_acc.get(), sizeof(long long) * T, cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
  });
}

}  // extern "C"
