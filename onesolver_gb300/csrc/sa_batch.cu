// sa_batch.cu -- many dense instances of uneven size annealed together.
//
// The reference anneals one instance per sa::anneal call
// (include/simulated_annealing/annealing.hpp:55-140). Here a batch of dense
// instances shares one schedule and runs as:
//
//   init resync -> [sweep chunk -> FP64 resync] x chunks -> unpack + re-score
//
// where every sweep chunk is ONE persistent launch (sa_batch_tile_kernel):
// each CTA takes (instance, block of W trajectories) items from a global
// counter, largest instances first, and runs the tiled sequential sweeps of
// sa_dense_tile_kernel on them. The whole sequence is captured once as a CUDA
// graph and replayed on every execute. W (trajectories per CTA, i.e. how many
// trajectories share each staged coupling tile) is picked by timing short
// probe launches of the candidates on the batch itself.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "rescore.cuh"
#include "sa_common.cuh"
#include "sa_kernels.cuh"
#include "sa_plan.cuh"
#include "sa_replay.cuh"

namespace os {
namespace sa {

constexpr int BATCH_MAX_LD = 1792;     // two 16-row FP32 tiles in shared memory
constexpr int BATCH_PROBE_STEPS = 4;

template <int SLOTS> void launch_batch_resync(const BatchResyncArgs &b, cudaStream_t s) {
  const int warps = 4;
  const unsigned grid = (unsigned)ceil_div_u64((unsigned long long)b.total, warps);
  sa_batch_resync_kernel<SLOTS><<<grid, warps * 32, 0, s>>>(b);
}

#define OS_BATCH_DISPATCH(cls, fn, ...)                                  \
  switch (cls) {                                                         \
    case 4: fn<4>(__VA_ARGS__); break;                                   \
    case 8: fn<8>(__VA_ARGS__); break;                                   \
    case 16: fn<16>(__VA_ARGS__); break;                                 \
    case 32: fn<32>(__VA_ARGS__); break;                                 \
    case 64: fn<64>(__VA_ARGS__); break;                                 \
    default: throw_error(OS_INVALID_ARG, "unsupported slot count %d", cls); \
  }

struct BatchState {
  int num = 0;
  std::vector<int> n, nslots, ld;
  std::vector<long long> traj_base, h_off, state_off_inst;
  DevBuf<BatchInstance> inst;
  DevBuf<int> traj_inst;
  DevBuf<long long> state_off;
  DevBuf<int2> items;
  DevBuf<unsigned int> work;
  int num_items = 0;
  long long total_traj = 0;
  size_t smem = 0;
  int grid = 0;
  cudaGraphExec_t graph = nullptr;
  ~BatchState() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

// Items (instance, first trajectory) for W trajectories per CTA, most
// expensive first (work ~ ld^2 per trajectory sweep).
void build_items(os_sa_plan *p, BatchState &B, int W) {
  std::vector<std::pair<long long, int2>> v;
  for (int k = 0; k < B.num; ++k)
    for (int t0 = 0; t0 < p->T; t0 += W) {
      const int cnt = std::min(W, p->T - t0);
      v.push_back({(long long)B.ld[k] * B.ld[k] * cnt, make_int2(k, t0)});
    }
  std::stable_sort(v.begin(), v.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
  std::vector<int2> items(v.size());
  for (size_t i = 0; i < v.size(); ++i) items[i] = v[i].second;
  B.items.alloc(items.size());
  OS_CUDA(cudaMemcpy(B.items.get(), items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice));
  B.num_items = (int)items.size();
}

BatchArgs batch_args(os_sa_plan *p, BatchState &B, int W, int s0, int s1) {
  BatchArgs a{};
  a.inst = B.inst.get();
  a.items = B.items.get();
  a.num_items = B.num_items;
  a.work = B.work.get();
  a.W = W;
  a.beta = p->beta.get();
  a.spb = p->spb;
  a.step_begin = s0;
  a.step_end = s1;
  a.acceptance = p->acceptance;
  a.seed_lo = (uint32_t)p->seed;
  a.seed_hi = (uint32_t)(p->seed >> 32);
  a.h = p->h.get();
  a.x = p->x.get();
  a.xbest = p->xbest.get();
  a.e = p->e.get();
  a.ebest = p->ebest.get();
  a.accepted = p->accepted.get();
  a.status = p->status.get();
  a.thr = p->replay ? p->rp_thr.get() : nullptr;
  a.state_off = B.state_off.get();
  a.nsteps = p->steps;
  return a;
}

BatchResyncArgs resync_args(os_sa_plan *p, BatchState &B, int init) {
  BatchResyncArgs r{};
  r.inst = B.inst.get();
  r.traj_inst = B.traj_inst.get();
  r.total = B.total_traj;
  r.init = init;
  r.seed_lo = (uint32_t)p->seed;
  r.seed_hi = (uint32_t)(p->seed >> 32);
  r.h = p->h.get();
  r.x = p->x.get();
  r.xbest = p->xbest.get();
  r.e = p->e.get();
  r.ebest = p->ebest.get();
  r.drift_bits = p->drift.get();
  r.init_bits = p->replay ? p->rp_init.get() : nullptr;
  r.state_off = B.state_off.get();
  return r;
}

int batch_grid(os_sa_plan *p, BatchState &B, int W) {
  int occ = 0;
  batch_tile_occupancy(p->slot_cls, W, B.smem, &occ);
  if (occ < 1) occ = 1;
  return std::max(1, std::min(B.num_items, p->ctx->sm_count * occ));
}

// Time short probe launches for each candidate W and keep the fastest.
int autotune_warps(os_sa_plan *p, BatchState &B) {
  cudaStream_t s = p->ctx->stream;
  int max_threads = 0;
  batch_tile_max_threads(p->slot_cls, &max_threads);
  BatchResyncArgs r = resync_args(p, B, 1);
  OS_BATCH_DISPATCH(p->slot_cls, launch_batch_resync, r, s);
  OS_CUDA(cudaGetLastError());
  cudaEvent_t e0, e1;
  OS_CUDA(cudaEventCreate(&e0));
  OS_CUDA(cudaEventCreate(&e1));
  int best_w = 0;
  float best_ms = 0.f;
  const int probe = std::min(BATCH_PROBE_STEPS, p->steps);
  for (int W : {4, 8, 16}) {
    if (W * 32 > max_threads) continue;
    build_items(p, B, W);
    const int grid = batch_grid(p, B, W);
    OS_CUDA(cudaMemsetAsync(B.work.get(), 0, sizeof(unsigned), s));
    BatchArgs a = batch_args(p, B, W, 0, probe);
    OS_CUDA(cudaEventRecord(e0, s));
    batch_tile_launch(a, p->slot_cls, grid, B.smem, s);
    OS_CUDA(cudaGetLastError());
    OS_CUDA(cudaEventRecord(e1, s));
    OS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    OS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (best_w == 0 || ms < best_ms) {
      best_w = W;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  OS_REQUIRE(best_w > 0, "no trajectories-per-CTA candidate fits this batch");
  return best_w;
}

void plan_create_batched(os_sa_plan *p, int num, const os_qubo_dense *qs) {
  OS_REQUIRE(num >= 1 && qs, "empty batch");
  OS_REQUIRE(p->sequential, "batched annealing sweeps all sites per step (site_order must be SEQUENTIAL)");
  OS_REQUIRE(!p->init_prob.count, "batched annealing starts from random spins (init_prob must be NULL)");
  auto *B = new BatchState();
  p->batch = B;
  B->num = num;
  const int T = p->T;
  // Pack the instances into shared buffers; every matrix starts on a
  // 128-byte boundary (a multiple of 32 floats / 16 doubles). Only the
  // matrices as given go up; the padded FP32/FP64 arrays are staged on the
  // device, one kernel per instance.
  std::vector<size_t> oc(num), od(num), of(num);
  size_t nc = 0, nd = 0, nf = 0;
  int max_slots = 1;
  long long h_total = 0, traj = 0, st_total = 0;
  for (int k = 0; k < num; ++k) {
    OS_REQUIRE(qs[k].f && qs[k].n >= 1, "instance %d is empty", k);
    const int n = qs[k].n, nslots = slots_for(n), ld = nslots * 32;
    OS_REQUIRE(ld <= BATCH_MAX_LD, "instance %d has %d variables (batched limit %d)", k, n, BATCH_MAX_LD);
    B->n.push_back(n);
    B->nslots.push_back(nslots);
    B->ld.push_back(ld);
    max_slots = std::max(max_slots, nslots);
    oc[k] = nc;
    nc += (size_t)ld * ld;
    od[k] = nd;
    nd += ld;
    of[k] = nf;
    nf += ((size_t)n * n + 15) / 16 * 16;
    B->traj_base.push_back(traj);
    B->h_off.push_back(h_total);
    B->state_off_inst.push_back(st_total);
    traj += T;
    h_total += (long long)T * nslots * 32;
    st_total += (long long)T * n;
  }
  p->c32.alloc(nc);
  p->d32.alloc(nd);
  p->c64.alloc(nc);
  p->d64.alloc(nd);
  p->f.alloc(nf);
  {
    cudaStream_t s = p->ctx->stream;
    DevBuf<int> bad;
    bad.alloc(1);
    OS_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(int), s));
    for (int k = 0; k < num; ++k) {
      const int n = B->n[k];
      OS_CUDA(cudaMemcpyAsync(p->f.get() + of[k], qs[k].f, sizeof(double) * n * n, cudaMemcpyHostToDevice, s));
      stage_dense_device(p->f.get() + of[k], n, B->ld[k], p->c32.get() + oc[k], p->c64.get() + oc[k],
                         p->d32.get() + od[k], p->d64.get() + od[k], bad.get(), s);
    }
    int nbad = 0;
    OS_CUDA(cudaMemcpyAsync(&nbad, bad.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
    OS_REQUIRE(nbad == 0, "the batch has %d non-finite coefficients", nbad);
  }
  B->total_traj = traj;
  p->slot_cls = slot_class(max_slots);
  std::vector<BatchInstance> inst(num);
  std::vector<int> tinst(traj);
  std::vector<long long> soff(traj);
  for (int k = 0; k < num; ++k) {
    BatchInstance &in = inst[k];
    in.c = p->c32.get() + oc[k];
    in.diag = p->d32.get() + od[k];
    in.c64 = p->c64.get() + oc[k];
    in.d64 = p->d64.get() + od[k];
    in.f = p->f.get() + of[k];
    in.n = B->n[k];
    in.nslots = B->nslots[k];
    in.ld = B->ld[k];
    in.T = T;
    in.h_off = B->h_off[k];
    in.traj_base = B->traj_base[k];
    for (int t = 0; t < T; ++t) {
      tinst[B->traj_base[k] + t] = k;
      soff[B->traj_base[k] + t] = B->state_off_inst[k] + (long long)t * B->n[k];
    }
  }
  B->inst.alloc(num);
  OS_CUDA(cudaMemcpy(B->inst.get(), inst.data(), sizeof(BatchInstance) * num, cudaMemcpyHostToDevice));
  B->traj_inst.alloc(traj);
  OS_CUDA(cudaMemcpy(B->traj_inst.get(), tinst.data(), sizeof(int) * traj, cudaMemcpyHostToDevice));
  B->state_off.alloc(traj);
  OS_CUDA(cudaMemcpy(B->state_off.get(), soff.data(), sizeof(long long) * traj, cudaMemcpyHostToDevice));
  p->h.alloc(h_total);
  p->x.alloc(traj * 32);
  p->xbest.alloc(traj * 32);
  p->e.alloc(traj);
  p->ebest.alloc(traj);
  p->accepted.alloc(traj);
  p->states.alloc(st_total);
  p->e64.alloc(traj);
  p->status.alloc(1);
  B->work.alloc(1);
  B->smem = 0;
  for (int ldk : B->ld) B->smem = std::max(B->smem, tile_smem_bytes(ldk));
  batch_tile_set_smem(p->slot_cls, B->smem);
  OS_CUDA(cudaMemset(p->status.get(), 0, sizeof(int)));
  p->warps = autotune_warps(p, *B);
  build_items(p, *B, p->warps);
  B->grid = batch_grid(p, *B, p->warps);
  unsigned long long att = 0;
  for (int k = 0; k < num; ++k) att += (unsigned long long)B->n[k];
  p->attempts_per_step = att;  // per trajectory index, summed over instances
}

// The execute sequence (captured into a graph on the first call).
void enqueue_batched(os_sa_plan *p, BatchState &B, cudaStream_t s) {
  OS_CUDA(cudaMemsetAsync(p->accepted.get(), 0, sizeof(unsigned long long) * B.total_traj, s));
  OS_CUDA(cudaMemsetAsync(p->drift.get(), 0, sizeof(unsigned long long), s));
  OS_CUDA(cudaMemsetAsync(p->status.get(), 0, sizeof(int), s));
  BatchResyncArgs r = resync_args(p, B, 1);
  OS_BATCH_DISPATCH(p->slot_cls, launch_batch_resync, r, s);
  OS_CUDA(cudaGetLastError());
  r.init = 0;
  int chunk = 0;
  for (int s0 = 0; s0 < p->steps; s0 += p->chunk, ++chunk) {
    const int s1 = std::min(p->steps, s0 + p->chunk);
    OS_CUDA(cudaMemsetAsync(B.work.get(), 0, sizeof(unsigned), s));
    BatchArgs a = batch_args(p, B, p->warps, s0, s1);
    // External records: inside the captured graph they become event-record
    // nodes that the host can wait on after a replay.
    OS_CUDA(cudaEventRecordWithFlags(p->event(2 * chunk), s, cudaEventRecordExternal));
    if (p->replay)
      batch_tile_replay(a, p->slot_cls, B.grid, B.smem, s);
    else
      batch_tile_launch(a, p->slot_cls, B.grid, B.smem, s);
    OS_CUDA(cudaGetLastError());
    OS_CUDA(cudaEventRecordWithFlags(p->event(2 * chunk + 1), s, cudaEventRecordExternal));
    OS_BATCH_DISPATCH(p->slot_cls, launch_batch_resync, r, s);
    OS_CUDA(cudaGetLastError());
  }
  sa_batch_rescore_kernel<<<(unsigned)B.total_traj, RESCORE_WARPS * 32, 0, s>>>(B.inst.get(), B.traj_inst.get(), B.state_off.get(), B.total_traj,
                                              p->xbest.get(), p->states.get(), p->e64.get());
  OS_CUDA(cudaGetLastError());
}

void execute_batched(os_sa_plan *p) {
  BatchState &B = *p->batch;
  cudaStream_t s = p->ctx->stream;
  const int chunks = (int)ceil_div_u64((unsigned long long)p->steps, (unsigned long long)p->chunk);
  p->sweep_ev_used = chunks;
  p->launches = 2 + 2 * chunks;
  if (!B.graph) {
    for (int i = 0; i < 2 * chunks; ++i) p->event(i);  // events exist before capture
    cudaGraph_t g;
    OS_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue_batched(p, B, s);
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      throw;
    }
    OS_CUDA(cudaStreamEndCapture(s, &g));
    cudaError_t err = cudaGraphInstantiate(&B.graph, g, 0);
    cudaGraphDestroy(g);
    OS_CUDA(err);
  }
  OS_CUDA(cudaGraphLaunch(B.graph, s));
}

void release_batch(os_sa_plan *p) {
  delete p->batch;
  p->batch = nullptr;
}

std::vector<int> batch_sizes(const os_sa_plan *p) { return p->batch->n; }

void batch_replay_changed(os_sa_plan *p) {
  BatchState &B = *p->batch;
  if (B.graph) {
    OS_CUDA(cudaGraphExecDestroy(B.graph));
    B.graph = nullptr;
  }
  if (p->replay) batch_replay_smem(p->slot_cls, B.smem);
}

}  // namespace sa
}  // namespace os

using namespace os;
using namespace os::sa;

extern "C" {

os_status os_sa_plan_create_batched(os_ctx *ctx, int32_t num_instances, const os_qubo_dense *instances,
                                    const os_sa_params *params, os_sa_plan **out) {
  return guard([&] {
    OS_REQUIRE(out != nullptr, "null output");
    check_schedule(params);
    OS_REQUIRE(params->resync_every >= 0, "resync_every = -1 (no resync) is for dense plans only");
    OS_REQUIRE(num_instances >= 1 && instances, "empty batch");
    activate(ctx);
    auto *p = new os_sa_plan();
    try {
      p->kind = 2;
      int nmax = 1;
      for (int k = 0; k < num_instances; ++k) nmax = std::max(nmax, instances[k].n);
      os_sa_plan_common(p, ctx, params, nmax);
      plan_create_batched(p, num_instances, instances);
    } catch (...) {
      release_batch(p);
      delete p;
      throw;
    }
    *out = p;
  });
}

int32_t os_sa_plan_tuned_warps(const os_sa_plan *p) { return p ? p->warps : 0; }

os_status os_sa_plan_result_batched(os_sa_plan *p, os_sa_result *results) {
  return guard([&] {
    OS_REQUIRE(p && results && p->kind == 2 && p->batch, "not a batched plan");
    activate(p->ctx);
    OS_CUDA(cudaStreamSynchronize(p->ctx->stream));
    BatchState &B = *p->batch;
    int st = 0;
    OS_CUDA(cudaMemcpy(&st, p->status.get(), sizeof st, cudaMemcpyDeviceToHost));
    if (st) throw_error(OS_TIMEOUT, "a sweep kernel's bounded wait for a coupling tile ran out");
    std::vector<double> e(B.total_traj);
    OS_CUDA(cudaMemcpy(e.data(), p->e64.get(), sizeof(double) * e.size(), cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> acc(B.total_traj);
    OS_CUDA(cudaMemcpy(acc.data(), p->accepted.get(), sizeof(unsigned long long) * acc.size(),
                       cudaMemcpyDeviceToHost));
    unsigned long long drift_bits = 0;
    OS_CUDA(cudaMemcpy(&drift_bits, p->drift.get(), sizeof drift_bits, cudaMemcpyDeviceToHost));
    double drift;
    std::memcpy(&drift, &drift_bits, sizeof drift);
    const int T = p->T;
    for (int k = 0; k < B.num; ++k) {
      std::vector<double> ek(e.begin() + B.traj_base[k], e.begin() + B.traj_base[k] + T);
      const int best = argmin_first(ek);
      os_sa_result &r = results[k];
      const int n = B.n[k];
      const long long so = B.state_off_inst[k];
      if (r.state)
        OS_CUDA(cudaMemcpy(r.state, p->states.get() + so + (long long)best * n, n, cudaMemcpyDeviceToHost));
      if (r.traj_states)
        OS_CUDA(cudaMemcpy(r.traj_states, p->states.get() + so, (size_t)T * n, cudaMemcpyDeviceToHost));
      if (r.traj_energies) std::memcpy(r.traj_energies, ek.data(), sizeof(double) * T);
      r.energy = ek[best];
      r.max_field_drift = drift;
      r.attempts = (unsigned long long)p->steps * n * T;
      unsigned long long a = 0;
      for (int t = 0; t < T; ++t) a += acc[B.traj_base[k] + t];
      r.accepted = a;
    }
  });
}

os_status os_sa_run_batched(os_ctx *ctx, int32_t num_instances, const os_qubo_dense *instances,
                            const os_sa_params *params, os_sa_result *results) {
  os_sa_plan *plan = nullptr;
  os_status st = os_sa_plan_create_batched(ctx, num_instances, instances, params, &plan);
  if (st != OS_OK) return st;
  st = os_sa_plan_execute(plan);
  if (st == OS_OK) st = os_sa_plan_result_batched(plan, results);
  os_sa_plan_destroy(plan);
  return st;
}

}  // extern "C"
