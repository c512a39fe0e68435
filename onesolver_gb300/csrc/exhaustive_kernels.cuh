// exhaustive_kernels.cuh -- the Gray-code enumeration kernel of the
// exhaustive search (see exhaustive.cu for the algorithm), shared by the
// translation units that instantiate it for each coefficient type and inner
// width.
#ifndef ONESOLVER_EXHAUSTIVE_KERNELS_CUH_
#define ONESOLVER_EXHAUSTIVE_KERNELS_CUH_

#include <climits>
#include <cstdint>
#include <type_traits>
#include <utility>

#include "common.cuh"
#include "philox.cuh"

namespace os {
namespace exh {

constexpr int G_DEFAULT = 10;        // inner (unrolled) bits
constexpr int OS_EXH_VARIANT_ADD_MIN = 1;  // three-input add + min (ALU pipe)
constexpr int OS_EXH_VARIANT_FUSED = 2;    // FMA-pipe multiply-add + fused add-min
constexpr int OS_EXH_VARIANT_DEFAULT = OS_EXH_VARIANT_FUSED;
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
  T ks[INNER_MAX];                // prefix sums ks[t] = kf[1] + ... + kf[t]
  T one;                          // 1, as a runtime value
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
//   MODE 0: E is the state's energy: E += K[t] +/- c[k] (one three-input
//           add), m = min(m, E).
//   MODE 1: E carries only the outer-coupling part, E += c[k] * (+/-1) with
//           a runtime +/-1 (an integer multiply-add, which issues on the FMA
//           pipe), and the energy E + ks[t] meets the minimum in one fused
//           add-min; the ALU pipe then carries one instruction per state.
template <class T, int G, int MODE, int t>
__device__ __forceinline__ void inner_step(T &E, T &m, const T (&c)[G], const GrayParams<T> &P, T pos,
                                           T neg) {
  constexpr int k = ctz_c(t);
  constexpr bool up = (gray_c(t) >> k) & 1;
  if constexpr (MODE == 0) {
    E += P.kf[t] + (up ? c[k] : -c[k]);
    m = min(m, E);
  } else {
    E = c[k] * (up ? pos : neg) + E;
    m = __viaddmin_s32(E, P.ks[t], m);
  }
}

template <class T, int G, int MODE, int... Is>
__device__ __forceinline__ void inner_block_impl(T &E, T &m, const T (&c)[G], const GrayParams<T> &P, T pos,
                                                 T neg, std::integer_sequence<int, Is...>) {
  (inner_step<T, G, MODE, Is + 1>(E, m, c, P, pos, neg), ...);
}

// The 2^G - 1 inner steps of one block, from inner state 0; on return E is
// the energy of the block's last state in either mode.
template <class T, int G, int MODE>
__device__ __forceinline__ void inner_block(T &E, T &m, const T (&c)[G], const GrayParams<T> &P, T pos, T neg) {
  inner_block_impl<T, G, MODE>(E, m, c, P, pos, neg, std::make_integer_sequence<int, (1 << G) - 1>{});
  if constexpr (MODE == 1) E += P.ks[(1 << G) - 1];
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

template <class T, int G, bool COLLECT, int MODE>
__device__ __forceinline__ void process_item(unsigned long long item, const GrayParams<T> &P,
                                             ThreadBest<T> &tb, CollectState &cs, T thr) {
  const T pos = P.one, neg = -P.one;
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
    inner_block<T, G, MODE>(E, m, c, P, pos, neg);
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

template <class T, int G, bool COLLECT, int MODE = 0>
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
    if (item < items) process_item<T, G, COLLECT, MODE>(item, P, tb, cs, thr);
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

// Host-side launchers, one translation unit per (type, width):
// exhaustive_gray_i9.cu, exhaustive_gray_i10.cu, exhaustive_gray_l9.cu,
// exhaustive_gray_l10.cu.
template <class T, int G> void launch_gray_width(int variant, bool collect, int grid, cudaStream_t s,
                                                  const GrayParams<T> &P);
template <class T, int G> int gray_occupancy_width();

}  // namespace exh
}  // namespace os

#endif  // ONESOLVER_EXHAUSTIVE_KERNELS_CUH_
