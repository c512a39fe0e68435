// exhaustive.cu -- exhaustive QUBO search on sm_103a.
//
// Replaces exhaustive::solve (include/exhaustive/exhaustive.hpp:29-167). The
// reference evaluates every state with an O(n^2) FP64 loop (:110-134) over
// one contiguous state range per compute unit and keeps the first strict
// minimum; the host then takes std::min_element (:158-159), which returns the
// smallest state integer among exact minima.
//
// Here the 2^n states are enumerated in Gray-code order so that consecutive
// states differ in one bit and the energy changes by one precomputed delta:
//
//   * the low G bits ("inner" bits, G = 9 or 10, 10 by default) are walked by
//     fully unrolled code.
//     For step t of the inner Gray sequence the flipped bit k = ctz(t) and
//     its direction are compile-time constants, so the energy update is
//       E += K[t] +/- c[k]
//     where K[t] (the coupling of bit k to the other inner bits at that step,
//     plus its diagonal term) sits in the kernel-parameter constant bank and
//     c[k] (the coupling of bit k to the current outer bits) in a register:
//     one three-input integer add and one integer min per state;
//   * every block walks the same forward sequence, which ends with only the
//     top inner bit set; one more add clears that bit (back to the block's
//     first state, not counted twice) so all blocks start from inner state 0
//     and one copy of the unrolled code serves them all;
//   * between blocks one outer bit flips; its energy delta is a row sum over
//     the set bits and the G inner couplings c[] are updated (O(n) work per
//     2^G states);
//   * states are split into work items (fixed top bits) that warps take
//     from a global counter, so the persistent grid stays balanced.
//
// Integer coefficients are enumerated exactly in int32 (or int64): the
// reference's FP64 sums of integers below 2^53 are exact, so the energies and
// the tie set are identical. Non-integer coefficients are quantised to int64
// fixed point; all states within a rigorous error window of the quantised
// minimum are collected and re-scored in FP64 with the reference's own
// summation order, which decides the minimum and its ties exactly.
//
// The degenerate set: each thread keeps its best energy and up to LCAP
// states reaching it; a CTA reduces (warp shuffles, then shared memory) to
// its minimum and the states reaching it; a one-CTA gather kernel reduces the
// CTA records. If any list overflowed, a second pass re-enumerates and
// collects every state at the known minimum.
#include <algorithm>
#include <climits>
#include <cmath>
#include <type_traits>
#include <utility>
#include <vector>

#include "common.cuh"
#include "exhaustive_kernels.cuh"
#include "rescore.cuh"

namespace os {
namespace exh {

// Few free bits: one thread per state, energies from scratch.
template <class T, bool COLLECT>
__global__ void __launch_bounds__(THREADS) small_kernel(const __grid_constant__ GrayParams<T> P) {
  ThreadBest<T> tb;
  tb.best = tmax<T>();
  tb.cnt = 0;
  tb.minstate = ~0ull;
  CollectState cs{0ull, ~0ull, false};
  const unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < P.nstates) {
    const unsigned long long x = P.prefix_state | idx;
    const T E = energy_from_scratch(P.q, P.n, x);
    if (COLLECT) {
      collect_state(cs, P, x, E, (T)(P.summary->gmin + P.window));
    } else {
      tb.best = E;
      tb.cnt = 1;
      tb.list[0] = x;
      tb.minstate = x;
    }
  }
  if (COLLECT) {
    if (cs.count) {
      atomicAdd(P.out_count, cs.count);
      atomicMin(P.out_minstate, cs.minstate);
    }
  } else {
    cta_reduce(P, tb);
  }
}

// One CTA: reduce the CTA records to the global minimum, the count and the
// smallest minimising state, and compact the kept states.
template <class T>
__global__ void __launch_bounds__(1024) gather_kernel(const CtaRecord<T> *__restrict__ rec, int ncta,
                                                      const unsigned long long *__restrict__ cta_states,
                                                      Summary *sum, unsigned long long *out_states,
                                                      unsigned long long out_cap) {
  __shared__ long long s_min;
  __shared__ unsigned long long s_count, s_pos, s_minstate;
  __shared__ unsigned s_ovf;
  if (threadIdx.x == 0) {
    s_min = LLONG_MAX;
    s_count = 0;
    s_pos = 0;
    s_minstate = ~0ull;
    s_ovf = 0;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < ncta; c += blockDim.x)
    if (rec[c].count > 0) atomicMin(&s_min, (long long)rec[c].min);
  __syncthreads();
  const long long gmin = s_min;
  for (int c = threadIdx.x; c < ncta; c += blockDim.x) {
    const CtaRecord<T> r = rec[c];
    if (r.count == 0 || (long long)r.min != gmin) continue;
    atomicAdd(&s_count, (unsigned long long)r.count);
    if (r.ovf) atomicOr(&s_ovf, 1u);
    atomicMin(&s_minstate, r.minstate);
    const unsigned kept = min(r.count, (unsigned)CTA_CAP);
    unsigned long long p = atomicAdd(&s_pos, (unsigned long long)kept);
    for (unsigned e = 0; e < kept; ++e)
      if (p + e < out_cap) out_states[p + e] = cta_states[(size_t)c * CTA_CAP + e];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    sum->gmin = gmin;
    sum->count = s_count;
    sum->ovf = s_ovf;
    sum->minstate = s_minstate;
    sum->collected = min(s_pos, out_cap);
  }
}

// Fixed-point path: FP64 re-score of the candidates in the reference's order.
__global__ void cand_rescore_kernel(const double *__restrict__ f, int n,
                                    const unsigned long long *__restrict__ cand,
                                    const unsigned long long *__restrict__ ncand_p,
                                    unsigned long long cap, double *__restrict__ e_out) {
  const unsigned long long ncand = min(*ncand_p, cap);
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < ncand;
       i += (unsigned long long)gridDim.x * blockDim.x)
    e_out[i] = rescore_energy_bits(f, n, cand[i]);
}

// Fixed-point path: exact FP64 minimum among candidates and its ties.
__global__ void __launch_bounds__(1024) cand_final_kernel(const unsigned long long *__restrict__ cand,
                                                          const double *__restrict__ e,
                                                          const unsigned long long *__restrict__ ncand_p,
                                                          unsigned long long cap, Summary *sum,
                                                          unsigned long long *out_states,
                                                          unsigned long long out_cap) {
  __shared__ double s_min;
  __shared__ unsigned long long s_count, s_minstate;
  const unsigned long long ncand = min(*ncand_p, cap);
  if (threadIdx.x == 0) {
    double mm = INFINITY;
    for (unsigned long long i = 0; i < ncand; ++i) mm = fmin(mm, e[i]);
    s_min = mm;
    s_count = 0;
    s_minstate = ~0ull;
  }
  __syncthreads();
  for (unsigned long long i = threadIdx.x; i < ncand; i += blockDim.x) {
    if (e[i] == s_min) {
      unsigned long long p = atomicAdd(&s_count, 1ull);
      if (p < out_cap) out_states[p] = cand[i];
      atomicMin(&s_minstate, cand[i]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    sum->energy = s_min;
    sum->count = s_count;
    sum->minstate = s_minstate;
    sum->collected = min(s_count, out_cap);
    sum->ovf = 0;
  }
}

}  // namespace exh
}  // namespace os

using namespace os;
using namespace os::exh;

struct os_exh_plan {
  os_ctx *ctx = nullptr;
  int n = 0, fixed = 0, free_bits = 0;
  int kind = OS_COEF_INT32;
  int G = G_DEFAULT;             // unrolled inner bits
  int variant = OS_EXH_VARIANT_ADD_MIN;
  bool small = false;
  unsigned long long prefix_state = 0;
  int ctas = 0;
  unsigned long long out_cap = 1;
  unsigned long long user_cap = 0;
  long long window = 0;
  int launches = 0;
  bool fixed_path_overflow = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // around the enumeration pass
  cudaEvent_t ready = nullptr;                // buffers allocated and filled (creation stream)
  DevBuf<int> q32, kf32;
  DevBuf<long long> q64, kf64;
  DevBuf<unsigned char> rec;
  DevBuf<unsigned long long> cta_states, out_states, counters, cand;
  DevBuf<Summary> summary;
  DevBuf<double> d_f, cand_e;
  GrayParams<int> p32{};
  GrayParams<long long> p64{};
};

namespace {

// counters layout: [0] work, [1] out_count, [2] out_pos, [3] out_minstate,
//                  [4] cand_count, [5] cand_pos, [6] cand_minstate,
//                  [7] pruning bound (best energy published so far)
enum { C_WORK = 0, C_OUT_COUNT, C_OUT_POS, C_OUT_MIN, C_CAND_COUNT, C_CAND_POS, C_CAND_MIN, C_GBEST, C_N };

// The instruction variant a search runs (os_exh_params.variant): the
// caller's, else the packed variant where it is exact (int32 coefficients
// whose magnitudes sum to at most PACK_MAX_ABS, and at least one loop bit to
// split an item's blocks into pairs), else the fused pair. int64 and
// fixed-point searches run MODE 0 whatever the variant.
int choose_variant(int requested, int kind, double abs_sum, bool small, int free_bits, int G) {
  const bool packable = kind == OS_COEF_INT32 && !small && abs_sum <= PACK_MAX_ABS &&
                        std::min(LOOP_BITS, free_bits - G) >= 1;
  if (requested == OS_EXH_VARIANT_PACKED)
    OS_REQUIRE(packable, "variant 3 (packed) needs int32 coefficients whose magnitudes sum to at most %g "
               "and more than %d free bits", PACK_MAX_ABS, G);
  if (requested) return requested;
  return packable ? OS_EXH_VARIANT_PACKED : OS_EXH_VARIANT_DEFAULT;
}

// v in both 16-bit halves of a word: v * 65537 mod 2^32, the packed form of
// the pair (v, v) (the packed variant's constants).
inline int pack2(long long v) { return (int)((uint32_t)v * 65537u); }

// Inner step constants for width G: kf[t] = +/- (Q_kk + sum of Q_kj over
// the other inner bits set before step t), k = ctz(t).
template <class T> void inner_constants(const T *q, int n, int G, T *kf) {
  for (int t = 0; t < INNER_MAX; ++t) kf[t] = 0;
  for (int t = 1; t < (1 << G); ++t) {
    const int k = ctz_c(t);
    const int prev = gray_c(t - 1);
    const bool up = (gray_c(t) >> k) & 1;
    T base = q[(size_t)k * n + k];
    for (int j = 0; j < G; ++j)
      if (j != k && ((prev >> j) & 1)) base += q[(size_t)k * n + j];
    kf[t] = up ? base : -base;
  }
}

// Step constants of the packed variant: kf[t] in both halves.
template <class T> void packed_constants(const T *kf, GrayParams<T> &P) {
  for (int t = 0; t < INNER_MAX; ++t) P.kp[t] = pack2(kf[t]);
}

template <class T>
void fill_params(os_exh_plan *p, GrayParams<T> &P, const std::vector<T> &q,
                 DevBuf<T> &dq, DevBuf<T> &dkf) {
  const int n = p->n;
  std::vector<T> kf(INNER_MAX, 0);
  if (!p->small) inner_constants(q.data(), n, p->G, kf.data());
  cudaStream_t s = p->ctx->stream;
  dq.alloc_on(q.size(), p->ctx->pool, s);
  OS_CUDA(cudaMemcpyAsync(dq.get(), q.data(), sizeof(T) * q.size(), cudaMemcpyHostToDevice, s));
  dkf.alloc_on(INNER_MAX, p->ctx->pool, s);
  OS_CUDA(cudaMemcpyAsync(dkf.get(), kf.data(), sizeof(T) * INNER_MAX, cudaMemcpyHostToDevice, s));
  T acc = 0;
  for (int t = 0; t < INNER_MAX; ++t) {
    P.kf[t] = kf[t];
    acc += kf[t];
    P.ks[t] = acc;
  }
  packed_constants(kf.data(), P);
  P.one = 1;
  P.q = dq.get();
  P.kf_g = dkf.get();
  P.n = n;
  P.prefix_state = p->prefix_state;
  if (p->small) {
    P.loop_bits = 0;
    P.item_bits = 0;
    P.nstates = 1ull << p->free_bits;
  } else {
    const int outer = p->free_bits - p->G;
    P.loop_bits = std::min(LOOP_BITS, outer);
    P.item_bits = outer - P.loop_bits;
    P.nstates = 1ull << p->free_bits;
  }
  P.work = p->counters.get() + C_WORK;
  P.gbest = reinterpret_cast<long long *>(p->counters.get() + C_GBEST);
  P.seed = 0x5EEDu;
  P.var_mask = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
  P.fixed_mask = P.var_mask & ~((1ull << p->free_bits) - 1ull);
  P.cta = reinterpret_cast<CtaRecord<T> *>(p->rec.get());
  P.cta_states = p->cta_states.get();
  P.summary = p->summary.get();
  P.window = 0;
  P.out_count = p->counters.get() + C_OUT_COUNT;
  P.out_pos = p->counters.get() + C_OUT_POS;
  P.out_states = p->out_states.get();
  P.out_cap = p->out_cap;
  P.out_minstate = p->counters.get() + C_OUT_MIN;
}

// Launch gray_kernel for a runtime width G (9 or 10) and variant.
template <class T, bool COLLECT>
void launch_gray(int G, int variant, int grid, cudaStream_t s, const GrayParams<T> &P) {
  if (G == 9)
    launch_gray_width<T, 9>(variant, COLLECT, grid, s, P);
  else if (G == 10)
    launch_gray_width<T, 10>(variant, COLLECT, grid, s, P);
  else
    throw_error(OS_INVALID_ARG, "inner_bits must be 9 or 10");
}

template <class T> int gray_occupancy(int G, int variant) {
  return G == 9 ? gray_occupancy_width<T, 9>(variant) : gray_occupancy_width<T, 10>(variant);
}

template <class T> int grid_for(os_exh_plan *p, const GrayParams<T> &P) {
  if (p->small) return (int)ceil_div_u64(P.nstates, THREADS);
  const int occ = gray_occupancy<T>(p->G, p->variant);
  const unsigned long long items = 1ull << P.item_bits;
  const unsigned long long want = ceil_div_u64(items, THREADS);
  return (int)std::max<unsigned long long>(1, std::min<unsigned long long>(want, (unsigned long long)p->ctx->sm_count * occ));
}

// Reset the collection counters (count, pos, minstate) starting at `first`.
void reset_collect(os_exh_plan *p, int first, cudaStream_t s) {
  OS_CUDA(cudaMemsetAsync(p->counters.get() + first, 0, 2 * sizeof(unsigned long long), s));
  OS_CUDA(cudaMemsetAsync(p->counters.get() + first + 2, 0xff, sizeof(unsigned long long), s));
}

template <class T> void launch_pass(os_exh_plan *p, GrayParams<T> &P, bool collect) {
  cudaStream_t s = p->ctx->stream;
  OS_CUDA(cudaMemsetAsync(p->counters.get() + C_WORK, 0, sizeof(unsigned long long), s));
  if (p->small) {
    if (collect)
      small_kernel<T, true><<<p->ctas, THREADS, 0, s>>>(P);
    else
      small_kernel<T, false><<<p->ctas, THREADS, 0, s>>>(P);
  } else {
    if (collect)
      launch_gray<T, true>(p->G, p->variant, p->ctas, s, P);
    else
      launch_gray<T, false>(p->G, p->variant, p->ctas, s, P);
  }
  OS_CUDA(cudaGetLastError());
  ++p->launches;
}

template <class T> void execute_typed(os_exh_plan *p, GrayParams<T> &P) {
  cudaStream_t s = p->ctx->stream;
  OS_CUDA(cudaStreamWaitEvent(s, p->ready, 0));
  p->launches = 0;
  OS_CUDA(cudaMemsetAsync(p->counters.get() + C_WORK, 0, sizeof(unsigned long long), s));
  OS_CUDA(cudaMemsetAsync(p->counters.get() + C_GBEST, 0x7f, sizeof(unsigned long long), s));
  OS_CUDA(cudaEventRecord(p->ev0, s));
  launch_pass(p, P, false);
  OS_CUDA(cudaEventRecord(p->ev1, s));
  gather_kernel<T><<<1, 1024, 0, s>>>(reinterpret_cast<const CtaRecord<T> *>(p->rec.get()), p->ctas,
                                      p->cta_states.get(), p->summary.get(), p->out_states.get(),
                                      p->out_cap);
  OS_CUDA(cudaGetLastError());
  ++p->launches;
  if (p->kind == OS_COEF_FIXED64) {
    // Collect the window around the quantised minimum into the candidate
    // buffer, re-score in FP64, and take the exact minimum and ties.
    GrayParams<T> C = P;
    C.window = p->window;
    C.out_count = p->counters.get() + C_CAND_COUNT;
    C.out_pos = p->counters.get() + C_CAND_POS;
    C.out_minstate = p->counters.get() + C_CAND_MIN;
    C.out_states = p->cand.get();
    C.out_cap = CAND_CAP;
    reset_collect(p, C_CAND_COUNT, s);
    launch_pass(p, C, true);
    cand_rescore_kernel<<<p->ctx->sm_count * 4, 256, 0, s>>>(
        p->d_f.get(), p->n, p->cand.get(), p->counters.get() + C_CAND_POS, CAND_CAP,
        p->cand_e.get());
    OS_CUDA(cudaGetLastError());
    cand_final_kernel<<<1, 1024, 0, s>>>(p->cand.get(), p->cand_e.get(),
                                         p->counters.get() + C_CAND_POS, CAND_CAP,
                                         p->summary.get(), p->out_states.get(), p->out_cap);
    OS_CUDA(cudaGetLastError());
    p->launches += 2;
  }
}

bool is_integer(double v) { return std::isfinite(v) && v == std::floor(v); }

}  // namespace

extern "C" {

os_status os_exhaustive_plan_create(os_ctx *ctx, const os_qubo_dense *qubo,
                                    const os_exh_params *params, os_exh_plan **out) {
  return guard([&] {
    OS_REQUIRE(qubo && qubo->f && out, "null argument");
    const int n = qubo->n;
    OS_REQUIRE(n >= 1 && n <= MAX_N, "exhaustive search supports 1..%d variables (got %d)", MAX_N, n);
    os_exh_params prm{};
    if (params) prm = *params;
    OS_REQUIRE(prm.fixed_high_bits >= 0 && prm.fixed_high_bits < n,
               "fixed_high_bits must be in [0, n)");
    if (prm.fixed_high_bits > 0)
      OS_REQUIRE(prm.prefix < (1ull << prm.fixed_high_bits), "prefix does not fit in fixed_high_bits");
    else
      OS_REQUIRE(prm.prefix == 0, "prefix given without fixed_high_bits");

    // Upper triangle -> symmetric matrix; classify the coefficients.
    std::vector<double> f((size_t)n * n);
    bool integral = true;
    double abs_sum = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = i; j < n; ++j) {
        const double v = qubo->f[(size_t)i * n + j];
        OS_REQUIRE(std::isfinite(v), "coefficient (%d,%d) is not finite", i, j);
        f[(size_t)i * n + j] = v;
        f[(size_t)j * n + i] = v;
        integral = integral && is_integer(v);
        abs_sum += std::fabs(v);
      }
    int kind = prm.coef_kind;
    if (kind == OS_COEF_AUTO) {
      if (integral && abs_sum < 2147483000.0) kind = OS_COEF_INT32;
      else if (integral && abs_sum < 9.0e15) kind = OS_COEF_INT64;
      else kind = OS_COEF_FIXED64;
    }
    OS_REQUIRE(kind >= OS_COEF_INT32 && kind <= OS_COEF_FIXED64, "unknown coef_kind %d", kind);
    OS_REQUIRE(prm.inner_bits == 0 || prm.inner_bits == 9 || prm.inner_bits == 10,
               "inner_bits must be 0 (default), 9 or 10");
    OS_REQUIRE(prm.variant >= 0 && prm.variant <= OS_EXH_VARIANT_PACKED, "unknown variant %d", prm.variant);
    if (kind == OS_COEF_INT32)
      OS_REQUIRE(integral && abs_sum < 2147483000.0, "coefficients are not int32-exact");
    if (kind == OS_COEF_INT64)
      OS_REQUIRE(integral && abs_sum < 9.0e15, "coefficients are not int64-exact");

    activate(ctx);
    auto *p = new os_exh_plan();
    try {
      p->ctx = ctx;
      p->n = n;
      p->fixed = prm.fixed_high_bits;
      p->free_bits = n - prm.fixed_high_bits;
      p->kind = kind;
      p->small = p->free_bits < SMALL_FREE;
      p->G = prm.inner_bits ? prm.inner_bits : G_DEFAULT;
      p->variant = choose_variant(prm.variant, kind, abs_sum, p->small, p->free_bits, p->G);
      p->prefix_state = prm.fixed_high_bits ? (prm.prefix << p->free_bits) : 0ull;
      p->user_cap = prm.max_minimisers;
      p->out_cap = std::max<unsigned long long>(prm.max_minimisers, 1ull);
      // Plan buffers come stream-ordered from the context's pool, and the
      // uploads are ordered on the same stream (pageable sources are staged
      // before the calls return); `ready` marks their end for an execution
      // on another stream.
      cudaMemPool_t mp = ctx->pool;
      cudaStream_t cs = ctx->stream;
      p->counters.alloc_on(C_N, mp, cs);
      OS_CUDA(cudaEventCreate(&p->ev0));
      OS_CUDA(cudaEventCreate(&p->ev1));
      OS_CUDA(cudaEventCreateWithFlags(&p->ready, cudaEventDisableTiming));
      p->summary.alloc_on(1, mp, cs);
      p->out_states.alloc_on(p->out_cap, mp, cs);

      if (kind == OS_COEF_INT32) {
        std::vector<int> q(f.size());
        for (size_t i = 0; i < f.size(); ++i) q[i] = (int)f[i];
        // Record buffers sized after the grid is known.
        p->rec.alloc_on(sizeof(CtaRecord<int>) * 1, mp, cs);
        fill_params(p, p->p32, q, p->q32, p->kf32);
        p->ctas = grid_for(p, p->p32);
        p->rec.alloc_on(sizeof(CtaRecord<int>) * p->ctas, mp, cs);
        p->cta_states.alloc_on((size_t)p->ctas * CTA_CAP, mp, cs);
        p->p32.cta = reinterpret_cast<CtaRecord<int> *>(p->rec.get());  // records sized for the grid
        p->p32.cta_states = p->cta_states.get();
      } else {
        std::vector<long long> q(f.size());
        if (kind == OS_COEF_INT64) {
          for (size_t i = 0; i < f.size(); ++i) q[i] = (long long)f[i];
        } else {
          // Fixed point: scale by 2^s so that every partial sum stays below
          // 2^60; collect within the rounding-error window (see header).
          const double P = 0.5 * n * (n + 1.0);
          int s = (int)std::floor(std::log2(std::ldexp(1.0, 60) / std::max(abs_sum, 1e-300)));
          s = std::min(s, 60);
          const double S = std::ldexp(1.0, s);
          for (size_t i = 0; i < f.size(); ++i) q[i] = std::llround(f[i] * S);
          const double delta = P * 1.2e-16 * abs_sum;  // bound on the FP64 reference error
          p->window = (long long)std::ceil(P + 2.0 * S * delta) + 2;
          p->d_f.alloc_on(f.size(), mp, cs);
          OS_CUDA(cudaMemcpyAsync(p->d_f.get(), f.data(), sizeof(double) * f.size(), cudaMemcpyHostToDevice, cs));
          p->cand.alloc_on(CAND_CAP, mp, cs);
          p->cand_e.alloc_on(CAND_CAP, mp, cs);
        }
        p->rec.alloc_on(sizeof(CtaRecord<long long>) * 1, mp, cs);
        fill_params(p, p->p64, q, p->q64, p->kf64);
        p->ctas = grid_for(p, p->p64);
        p->rec.alloc_on(sizeof(CtaRecord<long long>) * p->ctas, mp, cs);
        p->cta_states.alloc_on((size_t)p->ctas * CTA_CAP, mp, cs);
        p->p64.cta = reinterpret_cast<CtaRecord<long long> *>(p->rec.get());  // records sized for the grid
        p->p64.cta_states = p->cta_states.get();
      }
      OS_CUDA(cudaEventRecord(p->ready, cs));
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

os_status os_exhaustive_plan_execute(os_exh_plan *p) {
  return guard([&] {
    OS_REQUIRE(p != nullptr, "null plan");
    activate(p->ctx);
    if (p->kind == OS_COEF_INT32)
      execute_typed(p, p->p32);
    else
      execute_typed(p, p->p64);
  });
}

int32_t os_exhaustive_plan_launches(const os_exh_plan *p) { return p ? p->launches : 0; }

int32_t os_exhaustive_plan_variant(const os_exh_plan *p) {
  if (!p || p->small) return 0;
  return p->kind == OS_COEF_INT32 ? p->variant : OS_EXH_VARIANT_ADD_MIN;
}

os_status os_exhaustive_plan_result(os_exh_plan *p, os_exh_result *r) {
  os_status extra = OS_OK;
  os_status st = guard([&] {
    OS_REQUIRE(p && r, "null argument");
    activate(p->ctx);
    cudaStream_t s = p->ctx->stream;
    OS_CUDA(cudaStreamSynchronize(s));
    Summary sum;
    OS_CUDA(cudaMemcpy(&sum, p->summary.get(), sizeof sum, cudaMemcpyDeviceToHost));
    unsigned long long count = sum.count, written = sum.collected, minstate = sum.minstate;
    double energy = (double)sum.gmin;
    int passes = 1;
    if (p->kind == OS_COEF_FIXED64) {
      unsigned long long ccount = 0;
      OS_CUDA(cudaMemcpy(&ccount, p->counters.get() + C_CAND_COUNT, sizeof ccount, cudaMemcpyDeviceToHost));
      if (ccount > CAND_CAP)
        throw_error(OS_OVERFLOW_MINIMISERS,
                    "%llu states lie within the fixed-point error window (limit %llu)",
                    (unsigned long long)ccount, (unsigned long long)CAND_CAP);
      energy = sum.energy;
      passes = 2;
    } else if (sum.ovf) {
      // Second pass: collect every state at the known minimum.
      passes = 2;
      reset_collect(p, C_OUT_COUNT, s);
      if (p->kind == OS_COEF_INT32) {
        GrayParams<int> C = p->p32;
        launch_pass(p, C, true);
      } else {
        GrayParams<long long> C = p->p64;
        launch_pass(p, C, true);
      }
      OS_CUDA(cudaStreamSynchronize(s));
      unsigned long long c3[3];
      OS_CUDA(cudaMemcpy(c3, p->counters.get() + C_OUT_COUNT, sizeof c3, cudaMemcpyDeviceToHost));
      count = c3[0];
      written = std::min<unsigned long long>(c3[1], p->out_cap);
      minstate = c3[2];
    }
    std::vector<unsigned long long> states(written);
    if (written)
      OS_CUDA(cudaMemcpy(states.data(), p->out_states.get(), sizeof(unsigned long long) * written,
                         cudaMemcpyDeviceToHost));
    std::sort(states.begin(), states.end());
    r->energy = energy;
    r->state = minstate;
    r->count = count;
    r->states_enumerated = 1ull << p->free_bits;
    r->coef_kind_used = p->kind;
    r->collect_passes = passes;
    if (r->states) {
      const unsigned long long k = std::min<unsigned long long>(written, p->user_cap);
      for (unsigned long long i = 0; i < k; ++i) r->states[i] = states[i];
    }
    if (p->user_cap > 0 && count > p->user_cap) extra = OS_OVERFLOW_MINIMISERS;
  });
  if (st != OS_OK) return st;
  if (extra != OS_OK)
    return fail(extra, "the degenerate set holds %llu states; only %llu fit the buffer",
                (unsigned long long)r->count, (unsigned long long)(p->user_cap));
  return OS_OK;
}

os_status os_exhaustive_plan_kernel_ms(os_exh_plan *p, float *ms) {
  return guard([&] {
    OS_REQUIRE(p && ms, "null argument");
    activate(p->ctx);
    OS_CUDA(cudaEventSynchronize(p->ev1));
    OS_CUDA(cudaEventElapsedTime(ms, p->ev0, p->ev1));
  });
}

void os_exhaustive_plan_destroy(os_exh_plan *p) {
  if (!p) return;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  if (p->ev0) cudaEventDestroy(p->ev0);
  if (p->ev1) cudaEventDestroy(p->ev1);
  if (p->ready) cudaEventDestroy(p->ready);
  delete p;
}

os_status os_exhaustive_run(os_ctx *ctx, const os_qubo_dense *qubo, const os_exh_params *params,
                            os_exh_result *result) {
  os_exh_plan *plan = nullptr;
  os_status st = os_exhaustive_plan_create(ctx, qubo, params, &plan);
  if (st != OS_OK) return st;
  st = os_exhaustive_plan_execute(plan);
  if (st == OS_OK) st = os_exhaustive_plan_result(plan, result);
  os_exhaustive_plan_destroy(plan);
  return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Exhaustive search without device allocation.
//
// For callers that cannot call cudaMalloc: a serving process that reserves
// the whole device memory for its own pool at start-up, or code on a
// latency-critical path where cudaMalloc / cudaFree would synchronise the
// device and stall every other stream. This entry point keeps every piece of
// device scratch it needs (coefficients, step constants, work counter, CTA
// records, kept minimisers, summary) in one file-scope array of
// OS_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds
// until the process exits, and copies the caller's host inputs and outputs
// in and out of it. It runs the same enumeration kernels as
// os_exhaustive_run.
// ---------------------------------------------------------------------------

#include <mutex>

namespace os {
namespace exh {

constexpr size_t NOALLOC_BYTES = OS_NOALLOC_SCRATCH_BYTES;
constexpr int NOALLOC_MAX_CTAS = 2048;
constexpr unsigned long long NOALLOC_MAX_OUT = OS_NOALLOC_MAX_MINIMISERS;
constexpr int NOALLOC_MAX_DEVICES = 64;

// Section offsets inside the scratch array (256-byte aligned).
constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t NA_COUNTERS = 0;
constexpr size_t NA_SUMMARY = align256(NA_COUNTERS + C_N * sizeof(unsigned long long));
constexpr size_t NA_Q = align256(NA_SUMMARY + sizeof(Summary));
constexpr size_t NA_KF = align256(NA_Q + (size_t)MAX_N * MAX_N * sizeof(long long));
constexpr size_t NA_REC = align256(NA_KF + INNER_MAX * sizeof(long long));
constexpr size_t NA_CTA_STATES = align256(NA_REC + NOALLOC_MAX_CTAS * sizeof(CtaRecord<long long>));
constexpr size_t NA_OUT = align256(NA_CTA_STATES + (size_t)NOALLOC_MAX_CTAS * CTA_CAP * sizeof(unsigned long long));
constexpr size_t NA_END = align256(NA_OUT + NOALLOC_MAX_OUT * sizeof(unsigned long long));
static_assert(NA_END <= NOALLOC_BYTES, "no-allocation scratch layout exceeds its array");

// The scratch itself. In host code `g_noalloc_scratch` is only a stand-in
// for the symbol: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device, looked up once
// per device.
unsigned char *noalloc_scratch(int device) {
  OS_REQUIRE(device >= 0 && device < NOALLOC_MAX_DEVICES, "device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[device]) {
    void *ptr = nullptr;
    OS_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    g_noalloc_ptr[device] = static_cast<unsigned char *>(ptr);
  }
  return g_noalloc_ptr[device];
}

template <class T>
void noalloc_run(const os_qubo_dense *qubo, const os_exh_params &prm, os_exh_result *r, int kind,
                 double abs_sum, cudaStream_t s, int device, unsigned char *base) {
  const int n = qubo->n;
  const int free_bits = n - prm.fixed_high_bits;
  const bool small = free_bits < SMALL_FREE;
  // Host staging on the stack: coefficients and step constants.
  T q[MAX_N * MAX_N];
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j)
      q[(size_t)i * n + j] = q[(size_t)j * n + i] = (T)qubo->f[(size_t)i * n + j];
  // Inner width and instruction variant as os_exhaustive_plan_create
  // chooses them (the caller's values, else the defaults).
  const int G = prm.inner_bits ? prm.inner_bits : G_DEFAULT;
  const int variant = choose_variant(prm.variant, kind, abs_sum, small, free_bits, G);
  GrayParams<T> P{};
  T kf[INNER_MAX];
  if (!small) inner_constants(q, n, G, kf);
  else for (int t = 0; t < INNER_MAX; ++t) kf[t] = 0;
  T acc = 0;
  for (int t = 0; t < INNER_MAX; ++t) {
    P.kf[t] = kf[t];
    acc += kf[t];
    P.ks[t] = acc;
  }
  packed_constants(kf, P);
  P.one = 1;
  unsigned long long *counters = reinterpret_cast<unsigned long long *>(base + NA_COUNTERS);
  Summary *summary = reinterpret_cast<Summary *>(base + NA_SUMMARY);
  T *dq = reinterpret_cast<T *>(base + NA_Q);
  T *dkf = reinterpret_cast<T *>(base + NA_KF);
  P.q = dq;
  P.kf_g = dkf;
  P.n = n;
  P.prefix_state = prm.fixed_high_bits ? (prm.prefix << free_bits) : 0ull;
  P.nstates = 1ull << free_bits;
  if (!small) {
    const int outer = free_bits - G;
    P.loop_bits = std::min(LOOP_BITS, outer);
    P.item_bits = outer - P.loop_bits;
  }
  P.work = counters + C_WORK;
  P.gbest = reinterpret_cast<long long *>(counters + C_GBEST);
  P.seed = 0x5EEDu;
  P.var_mask = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
  P.fixed_mask = P.var_mask & ~((1ull << free_bits) - 1ull);
  P.cta = reinterpret_cast<CtaRecord<T> *>(base + NA_REC);
  P.cta_states = reinterpret_cast<unsigned long long *>(base + NA_CTA_STATES);
  P.summary = summary;
  P.window = 0;
  P.out_count = counters + C_OUT_COUNT;
  P.out_pos = counters + C_OUT_POS;
  P.out_states = reinterpret_cast<unsigned long long *>(base + NA_OUT);
  P.out_minstate = counters + C_OUT_MIN;
  const unsigned long long user_cap = prm.max_minimisers;
  P.out_cap = std::max<unsigned long long>(user_cap, 1ull);

  int ctas;
  if (small) {
    ctas = (int)ceil_div_u64(P.nstates, THREADS);
  } else {
    int occ = 0, sms = 0;
    occ = gray_occupancy<T>(G, variant);
    OS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const unsigned long long want = ceil_div_u64(1ull << P.item_bits, THREADS);
    ctas = (int)std::min<unsigned long long>(want, (unsigned long long)sms * std::max(occ, 1));
    ctas = std::max(1, std::min(ctas, NOALLOC_MAX_CTAS));
  }
  OS_REQUIRE(ctas <= NOALLOC_MAX_CTAS, "too many CTAs for the no-allocation scratch");

  // Every call shares the array: clear what must start at zero.
  OS_CUDA(cudaMemcpyAsync(dq, q, sizeof(T) * n * n, cudaMemcpyHostToDevice, s));
  OS_CUDA(cudaMemcpyAsync(dkf, kf, sizeof(T) * INNER_MAX, cudaMemcpyHostToDevice, s));
  OS_CUDA(cudaMemsetAsync(counters, 0, C_N * sizeof(unsigned long long), s));
  OS_CUDA(cudaMemsetAsync(counters + C_OUT_MIN, 0xff, sizeof(unsigned long long), s));
  OS_CUDA(cudaMemsetAsync(counters + C_GBEST, 0x7f, sizeof(unsigned long long), s));
  if (small) {
    small_kernel<T, false><<<ctas, THREADS, 0, s>>>(P);
  } else {
    launch_gray<T, false>(G, variant, ctas, s, P);
  }
  OS_CUDA(cudaGetLastError());
  gather_kernel<T><<<1, 1024, 0, s>>>(P.cta, ctas, P.cta_states, summary, P.out_states, P.out_cap);
  OS_CUDA(cudaGetLastError());
  Summary sum;
  OS_CUDA(cudaMemcpyAsync(&sum, summary, sizeof sum, cudaMemcpyDeviceToHost, s));
  OS_CUDA(cudaStreamSynchronize(s));
  unsigned long long count = sum.count, written = sum.collected, minstate = sum.minstate;
  int passes = 1;
  if (sum.ovf) {
    passes = 2;
    OS_CUDA(cudaMemsetAsync(counters, 0, C_N * sizeof(unsigned long long), s));
    OS_CUDA(cudaMemsetAsync(counters + C_OUT_MIN, 0xff, sizeof(unsigned long long), s));
    if (small)
      small_kernel<T, true><<<ctas, THREADS, 0, s>>>(P);
    else
      launch_gray<T, true>(G, variant, ctas, s, P);
    OS_CUDA(cudaGetLastError());
    unsigned long long c3[3];
    OS_CUDA(cudaMemcpyAsync(c3, counters + C_OUT_COUNT, sizeof c3, cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
    count = c3[0];
    written = std::min<unsigned long long>(c3[1], P.out_cap);
    minstate = c3[2];
  }
  const unsigned long long k = std::min<unsigned long long>(written, user_cap);
  if (r->states && k) {
    OS_CUDA(cudaMemcpyAsync(r->states, P.out_states, sizeof(unsigned long long) * k,
                            cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
    std::sort(r->states, r->states + k);
  }
  r->energy = (double)sum.gmin;
  r->state = minstate;
  r->count = count;
  r->states_enumerated = 1ull << free_bits;
  r->coef_kind_used = kind;
  r->collect_passes = passes;
}

}  // namespace exh
}  // namespace os

extern "C" os_status os_exhaustive_run_noalloc(const os_qubo_dense *qubo, const os_exh_params *params,
                                               os_exh_result *result, void *stream) {
  os_status extra = OS_OK;
  os_status st = guard([&] {
    OS_REQUIRE(qubo && qubo->f && result, "null argument");
    const int n = qubo->n;
    OS_REQUIRE(n >= 1 && n <= MAX_N, "exhaustive search supports 1..%d variables (got %d)", MAX_N, n);
    os_exh_params prm{};
    if (params) prm = *params;
    OS_REQUIRE(prm.fixed_high_bits >= 0 && prm.fixed_high_bits < n, "fixed_high_bits must be in [0, n)");
    if (prm.fixed_high_bits > 0)
      OS_REQUIRE(prm.prefix < (1ull << prm.fixed_high_bits), "prefix does not fit in fixed_high_bits");
    else
      OS_REQUIRE(prm.prefix == 0, "prefix given without fixed_high_bits");
    OS_REQUIRE(prm.inner_bits == 0 || prm.inner_bits == 9 || prm.inner_bits == 10,
               "inner_bits must be 0 (default), 9 or 10");
    OS_REQUIRE(prm.variant >= 0 && prm.variant <= OS_EXH_VARIANT_PACKED, "unknown variant %d", prm.variant);
    OS_REQUIRE(prm.max_minimisers <= NOALLOC_MAX_OUT,
               "max_minimisers %llu exceeds the no-allocation limit of %llu",
               (unsigned long long)prm.max_minimisers, (unsigned long long)NOALLOC_MAX_OUT);
    bool integral = true;
    double abs_sum = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = i; j < n; ++j) {
        const double v = qubo->f[(size_t)i * n + j];
        OS_REQUIRE(std::isfinite(v), "coefficient (%d,%d) is not finite", i, j);
        integral = integral && v == std::floor(v);
        abs_sum += std::fabs(v);
      }
    int kind = prm.coef_kind;
    if (kind == OS_COEF_AUTO) kind = !integral ? OS_COEF_FIXED64 : abs_sum < 2147483000.0 ? OS_COEF_INT32 : OS_COEF_INT64;
    OS_REQUIRE(kind == OS_COEF_INT32 || kind == OS_COEF_INT64,
               "the no-allocation entry point enumerates integer coefficients only (int32 or int64); "
               "use os_exhaustive_run for non-integer coefficients");
    OS_REQUIRE(integral && (kind == OS_COEF_INT64 ? abs_sum < 9.0e15 : abs_sum < 2147483000.0),
               "coefficients are not exact in the requested integer type");
    int device = 0;
    OS_CUDA(cudaGetDevice(&device));
    unsigned char *base = noalloc_scratch(device);
    cudaStream_t s = (cudaStream_t)stream;
    if (kind == OS_COEF_INT32)
      noalloc_run<int>(qubo, prm, result, kind, abs_sum, s, device, base);
    else
      noalloc_run<long long>(qubo, prm, result, kind, abs_sum, s, device, base);
    if (prm.max_minimisers > 0 && result->count > prm.max_minimisers) extra = OS_OVERFLOW_MINIMISERS;
  });
  if (st != OS_OK) return st;
  if (extra != OS_OK)
    return fail(extra, "the degenerate set holds %llu states; only %llu fit the buffer",
                (unsigned long long)result->count,
                (unsigned long long)(params ? params->max_minimisers : 0));
  return OS_OK;
}
