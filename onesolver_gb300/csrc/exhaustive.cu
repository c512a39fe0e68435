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
//   * the low G bits ("inner" bits, G = 8..10, 9 by default) are walked by
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
#include <utility>
#include <vector>

#include "common.cuh"
#include "philox.cuh"
#include "rescore.cuh"

namespace os {
namespace exh {

constexpr int G_DEFAULT = 10;        // inner (unrolled) bits
constexpr int G_MAX = 10;
constexpr int INNER_MAX = 1 << G_MAX;
constexpr int LCAP = 4;              // states kept per thread
constexpr int THREADS = 256;         // threads per CTA
constexpr int CTA_CAP = 128;         // states kept per CTA
constexpr int LOOP_BITS = 5;         // blocks per work item = 2^LOOP_BITS
constexpr int SMALL_FREE = 14;       // below: one thread per state
constexpr int MAX_N = 50;
constexpr uint64_t CAND_CAP = 1u << 20;  // fixed-point candidate buffer

__host__ __device__ constexpr int ctz_c(int t) {
  int k = 0;
  while (!((t >> k) & 1)) ++k;
  return k;
}
__host__ __device__ constexpr int gray_c(int t) { return t ^ (t >> 1); }

template <class T> struct CtaRecord {
  T min;
  unsigned count;
  unsigned ovf;
  unsigned long long minstate;
};

struct Summary {
  long long gmin;                 // minimum (quantised units for fixed64)
  unsigned long long count;       // states at the minimum
  unsigned ovf;                   // lists overflowed: collection pass needed
  unsigned pad;
  unsigned long long minstate;    // smallest state at the minimum
  double energy;                  // FP64 energy (fixed64 path)
  unsigned long long collected;   // collection pass: states written
};

template <class T> struct GrayParams {
  T kf[INNER_MAX];                // inner step constants (kf[0] unused)
  const T *q;                     // n x n symmetric coefficients
  const T *kf_g;                  // global copy of kf (slow path)
  int n;                          // row length (all variables)
  int loop_bits;                  // blocks per item = 2^loop_bits
  int item_bits;                  // number of items = 2^item_bits
  int pad;
  unsigned long long prefix_state;  // fixed top bits, in place
  unsigned long long nstates;     // small kernel: states enumerated
  unsigned long long *work;       // work-queue counter
  long long *gbest;               // best energy found so far (pruning bound)
  uint32_t seed;                  // descent starting points
  unsigned long long fixed_mask;  // variables fixed by the shard prefix
  unsigned long long var_mask;    // (1 << n) - 1
  CtaRecord<T> *cta;              // one record per CTA
  unsigned long long *cta_states; // CTA_CAP per CTA
  // collection pass
  const Summary *summary;         // gmin of the first pass
  long long window;               // collect E <= gmin + window
  unsigned long long *out_count;  // all states found
  unsigned long long *out_pos;    // states written
  unsigned long long *out_states;
  unsigned long long out_cap;
  unsigned long long *out_minstate;
};

template <class T> __device__ __forceinline__ T tmax();
template <> __device__ __forceinline__ int tmax<int>() { return INT_MAX; }
template <> __device__ __forceinline__ long long tmax<long long>() { return LLONG_MAX; }

// One unrolled inner step; t, k and the direction are template constants.
template <class T, int G, int t>
__device__ __forceinline__ void inner_step(T &E, T &m, const T (&c)[G], const GrayParams<T> &P) {
  constexpr int k = ctz_c(t);
  constexpr bool up = (gray_c(t) >> k) & 1;
  E += P.kf[t] + (up ? c[k] : -c[k]);
  m = min(m, E);
}

template <class T, int G, int... Is>
__device__ __forceinline__ void inner_block_impl(T &E, T &m, const T (&c)[G], const GrayParams<T> &P,
                                                 std::integer_sequence<int, Is...>) {
  (inner_step<T, G, Is + 1>(E, m, c, P), ...);
}

// The 2^G - 1 inner steps of one block, from inner state 0.
template <class T, int G>
__device__ __forceinline__ void inner_block(T &E, T &m, const T (&c)[G], const GrayParams<T> &P) {
  inner_block_impl<T, G>(E, m, c, P, std::make_integer_sequence<int, (1 << G) - 1>{});
}

// Energy of a full state from scratch (set-bit pairs).
template <class T>
__device__ __forceinline__ T energy_from_scratch(const T *__restrict__ q, int n,
                                                 unsigned long long x) {
  T E = 0;
  unsigned long long r = x;
  while (r) {
    int i = __ffsll((long long)r) - 1;
    r &= r - 1;
    const T *row = q + (size_t)i * n;
    E += row[i];
    unsigned long long r2 = r;
    while (r2) {
      int j = __ffsll((long long)r2) - 1;
      r2 &= r2 - 1;
      E += row[j];
    }
  }
  return E;
}

template <class T> struct ThreadBest {
  T best;
  int cnt;
  unsigned long long minstate;
  unsigned long long list[LCAP];
};

// Inner couplings passed by value to the slow path, so that the hot loop's
// copy never has its address taken and stays in registers.
template <class T, int G> struct CVec {
  T v[G];
};

struct CollectState {
  unsigned long long count;
  unsigned long long minstate;
  bool full;
};

template <class T>
__device__ __forceinline__ void note_state(ThreadBest<T> &tb, unsigned long long s, T e) {
  if (e == tb.best) {
    if (tb.cnt < LCAP) tb.list[tb.cnt] = s;
    ++tb.cnt;
    tb.minstate = min(tb.minstate, s);
  }
}

template <class T>
__device__ __forceinline__ void collect_state(CollectState &cs, const GrayParams<T> &P,
                                              unsigned long long s, T e, T thr) {
  if (e <= thr) {
    ++cs.count;
    cs.minstate = min(cs.minstate, s);
    if (!cs.full) {
      unsigned long long pos = atomicAdd(P.out_pos, 1ull);
      if (pos < P.out_cap)
        P.out_states[pos] = s;
      else
        cs.full = true;
    }
  }
}

// Greedy descent from a random state: repeatedly flip the single variable
// that lowers the energy most, until none does. The energy reached is that
// of a real state, so it is a valid upper bound on the minimum; it seeds the
// per-thread pruning bound so that blocks are walked again only when they
// reach the best energy known (a warp pays for the slow walk whenever any of
// its lanes needs it).
template <class T>
__device__ __noinline__ T descent_bound(const GrayParams<T> &P, uint32_t tid) {
  const int n = P.n;
  const T *__restrict__ q = P.q;
  const Philox4 r = philox4x32_10(tid, 0u, 0u, 0xE5000000u, P.seed, 0x9E3779B9u);
  const unsigned long long rnd = ((unsigned long long)r.x << 32) | r.y;
  unsigned long long x = P.prefix_state | (rnd & ~P.fixed_mask & P.var_mask);
  T h[MAX_N];
  for (int j = 0; j < n; ++j) {
    T a = 0;
    for (int i = 0; i < n; ++i)
      if (i != j && ((x >> i) & 1ull)) a += q[(size_t)j * n + i];
    h[j] = a;
  }
  T E = energy_from_scratch(q, n, x);
  for (int it = 0; it < 4 * n; ++it) {
    T best_d = 0;
    int best_i = -1;
    for (int i = 0; i < n; ++i) {
      if ((P.fixed_mask >> i) & 1ull) continue;
      const T loc = q[(size_t)i * n + i] + h[i];
      const T d = ((x >> i) & 1ull) ? -loc : loc;
      if (d < best_d) {
        best_d = d;
        best_i = i;
      }
    }
    if (best_i < 0) break;
    const bool was = (x >> best_i) & 1ull;
    x ^= 1ull << best_i;
    E += best_d;
    for (int j = 0; j < n; ++j)
      if (j != best_i) h[j] += was ? -q[(size_t)best_i * n + j] : q[(size_t)best_i * n + j];
  }
  return E;
}

// Slow path: walk one block again, state by state.
template <class T, int G, bool COLLECT>
__device__ __noinline__ void revisit_block(const GrayParams<T> &P, const CVec<T, G> c,
                                           unsigned long long x_outer, T Estart, ThreadBest<T> &tb,
                                           CollectState &cs, T thr) {
  T e = Estart;
  unsigned long long s = x_outer;
  if (COLLECT) collect_state(cs, P, s, e, thr); else note_state(tb, s, e);
  for (int t = 1; t < (1 << G); ++t) {
    const int k = __ffs(t) - 1;
    const bool up = ((t ^ (t >> 1)) >> k) & 1;
    T ck = 0;
#pragma unroll
    for (int j = 0; j < G; ++j)
      if (j == k) ck = c.v[j];
    e += P.kf_g[t] + (up ? ck : -ck);
    s ^= 1ull << k;
    if (COLLECT) collect_state(cs, P, s, e, thr); else note_state(tb, s, e);
  }
}

template <class T, int G, bool COLLECT>
__device__ __forceinline__ void process_item(unsigned long long item, const GrayParams<T> &P,
                                             ThreadBest<T> &tb, CollectState &cs, T thr) {
  const int n = P.n;
  const T *__restrict__ q = P.q;
  unsigned long long x = P.prefix_state | (item << (G + P.loop_bits));
  T E = energy_from_scratch(q, n, x);
  T c[G];
#pragma unroll
  for (int i = 0; i < G; ++i) c[i] = 0;
  {
    unsigned long long r = x;
    while (r) {
      int j = __ffsll((long long)r) - 1;
      r &= r - 1;
      const T *row = q + (size_t)j * n;
#pragma unroll
      for (int i = 0; i < G; ++i) c[i] += row[i];
    }
  }
  const T top_diag = q[(size_t)(G - 1) * n + (G - 1)];
  const unsigned nblocks = 1u << P.loop_bits;
  for (unsigned B = 0; B < nblocks; ++B) {
    const T Estart = E;
    T m = E;
    inner_block<T, G>(E, m, c, P);
    if (!COLLECT && (B & 7u) == 7u) {
      // Tighten the bound with the best energy any thread has published.
      const long long g = *reinterpret_cast<volatile long long *>(P.gbest);
      if (g < (long long)tb.best) {
        tb.best = (T)g;
        tb.cnt = 0;
        tb.minstate = ~0ull;
      }
    }
    if (COLLECT ? (m <= thr) : (m <= tb.best)) {
      if (!COLLECT && m < tb.best) {
        tb.best = m;
        tb.cnt = 0;
        tb.minstate = ~0ull;
        atomicMin(P.gbest, (long long)m);
      }
      CVec<T, G> cv;
#pragma unroll
      for (int i = 0; i < G; ++i) cv.v[i] = c[i];
      revisit_block<T, G, COLLECT>(P, cv, x, Estart, tb, cs, thr);
    }
    if (B + 1 < nblocks) {
      // Clear the top inner bit (the block ends at inner state 1 << (G-1)),
      // then flip outer bit G + ctz(B+1) from inner state 0.
      E -= top_diag + c[G - 1];
      const int mb = G + __ffs((int)(B + 1)) - 1;
      const unsigned long long bm = 1ull << mb;
      const bool was = (x & bm) != 0;
      const T *row = q + (size_t)mb * n;
      T sum = row[mb];
      unsigned long long r = x & ~bm;
      while (r) {
        int j = __ffsll((long long)r) - 1;
        r &= r - 1;
        sum += row[j];
      }
      E += was ? -sum : sum;
      x ^= bm;
#pragma unroll
      for (int i = 0; i < G; ++i) c[i] += was ? -row[i] : row[i];
    }
  }
}

// CTA reduction of the per-thread bests into one record per CTA.
template <class T>
__device__ __forceinline__ void cta_reduce(const GrayParams<T> &P, ThreadBest<T> &tb) {
  __shared__ T s_wmin[THREADS / 32];
  __shared__ T s_min;
  __shared__ unsigned s_count, s_ovf;
  __shared__ unsigned long long s_minstate;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T w = tb.cnt > 0 ? tb.best : tmax<T>();
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) w = min(w, __shfl_xor_sync(0xffffffffu, w, off));
  if (lane == 0) s_wmin[warp] = w;
  __syncthreads();
  if (threadIdx.x == 0) {
    T mm = tmax<T>();
    for (int i = 0; i < THREADS / 32; ++i) mm = min(mm, s_wmin[i]);
    s_min = mm;
    s_count = 0;
    s_ovf = 0;
    s_minstate = ~0ull;
  }
  __syncthreads();
  const T cmin = s_min;
  if (tb.cnt > 0 && tb.best == cmin) {
    unsigned idx = atomicAdd(&s_count, (unsigned)tb.cnt);
    if (tb.cnt > LCAP) atomicOr(&s_ovf, 1u);
    atomicMin(&s_minstate, tb.minstate);
    const int kept = min(tb.cnt, LCAP);
    for (int e = 0; e < kept; ++e)
      if (idx + e < CTA_CAP) P.cta_states[(size_t)blockIdx.x * CTA_CAP + idx + e] = tb.list[e];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    CtaRecord<T> rec;
    rec.min = cmin;
    rec.count = s_count;
    rec.ovf = (s_ovf || s_count > CTA_CAP) ? 1u : 0u;
    rec.minstate = s_minstate;
    P.cta[blockIdx.x] = rec;
  }
}

template <class T, int G, bool COLLECT>
__global__ void __launch_bounds__(THREADS) gray_kernel(const __grid_constant__ GrayParams<T> P) {
  ThreadBest<T> tb;
  tb.best = tmax<T>();
  tb.cnt = 0;
  tb.minstate = ~0ull;
  CollectState cs{0ull, ~0ull, false};
  T thr = 0;
  if (COLLECT) {
    thr = (T)(P.summary->gmin + P.window);
  } else {
    // Seed the pruning bound: one greedy descent per thread, reduced over
    // the CTA and published to the global bound.
    __shared__ long long s_bound;
    if (threadIdx.x == 0) s_bound = LLONG_MAX;
    __syncthreads();
    const T d = descent_bound(P, blockIdx.x * blockDim.x + threadIdx.x);
    atomicMin(&s_bound, (long long)d);
    __syncthreads();
    if (threadIdx.x == 0) atomicMin(P.gbest, s_bound);
    const long long g = *reinterpret_cast<volatile long long *>(P.gbest);
    tb.best = (T)min(s_bound, g);
  }
  const unsigned long long items = 1ull << P.item_bits;
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(P.work, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= items) break;
    const unsigned long long item = base + lane;
    if (item < items) process_item<T, G, COLLECT>(item, P, tb, cs, thr);
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
  bool small = false;
  unsigned long long prefix_state = 0;
  int ctas = 0;
  unsigned long long out_cap = 1;
  unsigned long long user_cap = 0;
  long long window = 0;
  int launches = 0;
  bool fixed_path_overflow = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // around the enumeration pass
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

template <class T>
void fill_params(os_exh_plan *p, GrayParams<T> &P, const std::vector<T> &q,
                 DevBuf<T> &dq, DevBuf<T> &dkf) {
  const int n = p->n;
  std::vector<T> kf(INNER_MAX, 0);
  if (!p->small) inner_constants(q.data(), n, p->G, kf.data());
  dq.alloc(q.size());
  OS_CUDA(cudaMemcpy(dq.get(), q.data(), sizeof(T) * q.size(), cudaMemcpyHostToDevice));
  dkf.alloc(INNER_MAX);
  OS_CUDA(cudaMemcpy(dkf.get(), kf.data(), sizeof(T) * INNER_MAX, cudaMemcpyHostToDevice));
  for (int t = 0; t < INNER_MAX; ++t) P.kf[t] = kf[t];
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

// Launch gray_kernel<T, G, COLLECT> for a runtime G.
template <class T, bool COLLECT>
void launch_gray(int G, int grid, cudaStream_t s, const GrayParams<T> &P) {
  switch (G) {
    case 8: gray_kernel<T, 8, COLLECT><<<grid, THREADS, 0, s>>>(P); break;
    case 9: gray_kernel<T, 9, COLLECT><<<grid, THREADS, 0, s>>>(P); break;
    case 10: gray_kernel<T, 10, COLLECT><<<grid, THREADS, 0, s>>>(P); break;
    default: throw_error(OS_INVALID_ARG, "inner_bits must be 8, 9 or 10");
  }
}

template <class T> int gray_occupancy(int G) {
  int occ = 0;
  switch (G) {
    case 8: OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<T, 8, false>, THREADS, 0)); break;
    case 9: OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<T, 9, false>, THREADS, 0)); break;
    default: OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<T, 10, false>, THREADS, 0)); break;
  }
  return occ < 1 ? 1 : occ;
}

template <class T> int grid_for(os_exh_plan *p, const GrayParams<T> &P) {
  if (p->small) return (int)ceil_div_u64(P.nstates, THREADS);
  const int occ = gray_occupancy<T>(p->G);
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
      launch_gray<T, true>(p->G, p->ctas, s, P);
    else
      launch_gray<T, false>(p->G, p->ctas, s, P);
  }
  OS_CUDA(cudaGetLastError());
  ++p->launches;
}

template <class T> void execute_typed(os_exh_plan *p, GrayParams<T> &P) {
  cudaStream_t s = p->ctx->stream;
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
    activate(ctx);
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
    OS_REQUIRE(prm.inner_bits == 0 || (prm.inner_bits >= 8 && prm.inner_bits <= G_MAX),
               "inner_bits must be 0 (default), 8, 9 or 10");
    if (kind == OS_COEF_INT32)
      OS_REQUIRE(integral && abs_sum < 2147483000.0, "coefficients are not int32-exact");
    if (kind == OS_COEF_INT64)
      OS_REQUIRE(integral && abs_sum < 9.0e15, "coefficients are not int64-exact");

    auto *p = new os_exh_plan();
    try {
      p->ctx = ctx;
      p->n = n;
      p->fixed = prm.fixed_high_bits;
      p->free_bits = n - prm.fixed_high_bits;
      p->kind = kind;
      p->small = p->free_bits < SMALL_FREE;
      p->G = prm.inner_bits ? prm.inner_bits : G_DEFAULT;
      p->prefix_state = prm.fixed_high_bits ? (prm.prefix << p->free_bits) : 0ull;
      p->user_cap = prm.max_minimisers;
      p->out_cap = std::max<unsigned long long>(prm.max_minimisers, 1ull);
      p->counters.alloc(C_N);
      OS_CUDA(cudaEventCreate(&p->ev0));
      OS_CUDA(cudaEventCreate(&p->ev1));
      p->summary.alloc(1);
      p->out_states.alloc(p->out_cap);

      if (kind == OS_COEF_INT32) {
        std::vector<int> q(f.size());
        for (size_t i = 0; i < f.size(); ++i) q[i] = (int)f[i];
        // Record buffers sized after the grid is known.
        p->rec.alloc(sizeof(CtaRecord<int>) * 1);
        fill_params(p, p->p32, q, p->q32, p->kf32);
        p->ctas = grid_for(p, p->p32);
        p->rec.alloc(sizeof(CtaRecord<int>) * p->ctas);
        p->cta_states.alloc((size_t)p->ctas * CTA_CAP);
        fill_params(p, p->p32, q, p->q32, p->kf32);
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
          p->d_f.alloc(f.size());
          OS_CUDA(cudaMemcpy(p->d_f.get(), f.data(), sizeof(double) * f.size(), cudaMemcpyHostToDevice));
          p->cand.alloc(CAND_CAP);
          p->cand_e.alloc(CAND_CAP);
        }
        p->rec.alloc(sizeof(CtaRecord<long long>) * 1);
        fill_params(p, p->p64, q, p->q64, p->kf64);
        p->ctas = grid_for(p, p->p64);
        p->rec.alloc(sizeof(CtaRecord<long long>) * p->ctas);
        p->cta_states.alloc((size_t)p->ctas * CTA_CAP);
        fill_params(p, p->p64, q, p->q64, p->kf64);
      }
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
                 cudaStream_t s, int device, unsigned char *base) {
  const int n = qubo->n;
  const int free_bits = n - prm.fixed_high_bits;
  const bool small = free_bits < SMALL_FREE;
  // Host staging on the stack: coefficients and step constants.
  T q[MAX_N * MAX_N];
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j)
      q[(size_t)i * n + j] = q[(size_t)j * n + i] = (T)qubo->f[(size_t)i * n + j];
  constexpr int G = G_DEFAULT;
  GrayParams<T> P{};
  T kf[INNER_MAX];
  if (!small) inner_constants(q, n, G, kf);
  else for (int t = 0; t < INNER_MAX; ++t) kf[t] = 0;
  for (int t = 0; t < INNER_MAX; ++t) P.kf[t] = kf[t];
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
    OS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gray_kernel<T, G, false>, THREADS, 0));
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
    gray_kernel<T, G, false><<<ctas, THREADS, 0, s>>>(P);
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
      gray_kernel<T, G, true><<<ctas, THREADS, 0, s>>>(P);
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
      noalloc_run<int>(qubo, prm, result, kind, s, device, base);
    else
      noalloc_run<long long>(qubo, prm, result, kind, s, device, base);
    if (prm.max_minimisers > 0 && result->count > prm.max_minimisers) extra = OS_OVERFLOW_MINIMISERS;
  });
  if (st != OS_OK) return st;
  if (extra != OS_OK)
    return fail(extra, "the degenerate set holds %llu states; only %llu fit the buffer",
                (unsigned long long)result->count,
                (unsigned long long)(params ? params->max_minimisers : 0));
  return OS_OK;
}
