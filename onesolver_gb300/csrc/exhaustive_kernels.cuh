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
constexpr int OS_EXH_VARIANT_PACKED = 3;   // two states per three-input add in 16-bit halves
constexpr int OS_EXH_VARIANT_DEFAULT = OS_EXH_VARIANT_FUSED;
// Packed variant: each half holds energy + PACK_BIAS in [0, 32767]; safe when
// the coefficient magnitudes (upper triangle) sum to at most PACK_MAX_ABS, so
// that every energy and every coupling sum stays within 16383.
constexpr int PACK_BIAS = 16384;
constexpr double PACK_MAX_ABS = 8000.0;
constexpr int G_MAX = 10;
constexpr int INNER_MAX = 1 << G_MAX;
constexpr int LCAP = 4;              // states kept per thread
constexpr int THREADS = 256;         // threads per CTA
constexpr int CTA_CAP = 128;         // states kept per CTA
constexpr int LOOP_BITS = 6;         // blocks per work item = 2^LOOP_BITS
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
  int kp[INNER_MAX];              // kf[t] in both 16-bit halves (packed variant)
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
//   (MODE 2, the packed variant, has its own block walk: inner_block_packed.)
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

// MODE 2: one block of 2^G inner states for two walks at once. E and c
// hold two values as x_b * 65536 + x_a, both energies biased into
// [0, 32767], so plain 32-bit adds update both halves exactly (a packed sum
// is a sum of packed values) and the per-half minimum is one 16x2
// instruction. Every step is the MODE 0 update on both walks,
// E += kf[t] +/- c[k], one three-input add whose constant (kf[t] in both
// halves) comes from the parameter bank; every two steps (four states) one
// three-input per-half minimum. Both run on the ALU pipe, 0.75 instructions
// per state. (Constant-bank operands are what decide this form: the 16-bit
// fused add-min and the multiply-add cannot take one without a separate
// constant load per step.)
template <int G, int t>
__device__ __forceinline__ void packed_step(int &E, const int (&c)[G], const GrayParams<int> &P) {
  constexpr int k = ctz_c(t);
  constexpr bool up = (gray_c(t) >> k) & 1;
  E = E + P.kp[t] + (up ? c[k] : -c[k]);
}

template <int G, int t>
__device__ __forceinline__ void packed_pair(int &E, int &m, const int (&c)[G], const GrayParams<int> &P) {
  packed_step<G, t>(E, c, P);
  if constexpr (t + 1 < (1 << G)) {
    const int e1 = E;
    packed_step<G, t + 1>(E, c, P);
    m = (int)__vimin3_s16x2((unsigned)m, (unsigned)e1, (unsigned)E);
  } else {
    m = (int)__vimin3_s16x2((unsigned)m, (unsigned)E, (unsigned)E);
  }
}

template <int G, int... Is>
__device__ __forceinline__ void packed_block_impl(int &E, int &m, const int (&c)[G], const GrayParams<int> &P,
                                                  std::integer_sequence<int, Is...>) {
  (packed_pair<G, 2 * Is + 1>(E, m, c, P), ...);
}

// Minimum (per half) over the block that starts at packed energy E with
// packed outer couplings c.
template <int G>
__device__ __forceinline__ int inner_block_packed(int E, const int (&c)[G], const GrayParams<int> &P) {
  int m = E;
  packed_block_impl<G>(E, m, c, P, std::make_integer_sequence<int, (1 << (G - 1))>{});
  return m;
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
//
// The 32 lanes of a warp run one descent together: lane l keeps the local
// fields of variables l and l + 32, and each step's flip (the largest
// decrease, the lowest index among equals) comes from a warp argmin, so a
// descent costs O(n) steps of a few instructions per lane instead of O(n^2)
// serial work per thread. Every lane returns the same energy.
template <class T>
__device__ __noinline__ T descent_bound_warp(const GrayParams<T> &P, uint32_t wid) {
  const int lane = threadIdx.x & 31;
  const int n = P.n;
  const T *__restrict__ q = P.q;
  const Philox4 r = philox4x32_10(wid, 1u, 0u, 0xE5000000u, P.seed, 0x9E3779B9u);
  const unsigned long long rnd = ((unsigned long long)r.x << 32) | r.y;
  unsigned long long x = P.prefix_state | (rnd & ~P.fixed_mask & P.var_mask);
  const int j0 = lane, j1 = lane + 32;
  const bool v0 = j0 < n && !((P.fixed_mask >> j0) & 1ull);
  const bool v1 = j1 < n && !((P.fixed_mask >> j1) & 1ull);
  T h0 = 0, h1 = 0;
  for (int i = 0; i < n; ++i) {
    if (!((x >> i) & 1ull)) continue;
    if (j0 < n && i != j0) h0 += q[(size_t)j0 * n + i];
    if (j1 < n && i != j1) h1 += q[(size_t)j1 * n + i];
  }
  T E = energy_from_scratch(q, n, x);
  for (int it = 0; it < 4 * n; ++it) {
    T bd = 0;
    int bi = INT_MAX;
    if (v0) {
      const T loc = q[(size_t)j0 * n + j0] + h0;
      const T d = ((x >> j0) & 1ull) ? -loc : loc;
      if (d < bd) {
        bd = d;
        bi = j0;
      }
    }
    if (v1) {
      const T loc = q[(size_t)j1 * n + j1] + h1;
      const T d = ((x >> j1) & 1ull) ? -loc : loc;
      if (d < bd) {
        bd = d;
        bi = j1;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const T od = __shfl_xor_sync(0xffffffffu, bd, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (od < bd || (od == bd && oi < bi)) {
        bd = od;
        bi = oi;
      }
    }
    if (bi == INT_MAX) break;  // warp-uniform: no flip lowers the energy
    const bool was = (x >> bi) & 1ull;
    x ^= 1ull << bi;
    E += bd;
    const T *row = q + (size_t)bi * n;
    if (j0 < n && j0 != bi) h0 += was ? -row[j0] : row[j0];
    if (j1 < n && j1 != bi) h1 += was ? -row[j1] : row[j1];
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

// MODE 2: an item's 2^loop_bits blocks as 2^(loop_bits-1) pairs walked
// together: half a has the top loop bit (`top`) clear, half b set; the two
// flip the same outer bits (all below `top`), so one row sum serves both and
// the coupling vectors and block-start energies stay packed between blocks
// (x_b * 65536 + x_a; c_b = c_a + Q[top][.]). A block pair whose smaller
// half-minimum reaches the bound is walked again state by state, each half
// that reaches it on its own, exactly as MODE 1 does.
//
// Between block pairs one of the W = loop_bits - 1 walked bits G + w flips.
// Its energy delta splits into bw[w] (its diagonal and its couplings to the
// item's fixed set bits, summed once per item in the pass that builds the
// coupling vector) plus its couplings to the other walked bits that are set
// (at most W - 1 loads), instead of a row sum over every set bit per flip.
template <int G>
__device__ __forceinline__ void process_item_packed(unsigned long long item, const GrayParams<int> &P,
                                                    ThreadBest<int> &tb, CollectState &cs) {
  const int n = P.n;
  const int *__restrict__ q = P.q;
  const int top = G + P.loop_bits - 1;
  const int *__restrict__ rowt = q + (size_t)top * n;
  unsigned long long xa = P.prefix_state | (item << (G + P.loop_bits));
  const int Ea = energy_from_scratch(q, n, xa);
  const int W = P.loop_bits - 1;  // walked bits G .. G + W - 1 (W <= LOOP_BITS - 1)
  int ca[G];
#pragma unroll
  for (int i = 0; i < G; ++i) ca[i] = 0;
  int sumt = rowt[top];
  int bw[LOOP_BITS - 1];
#pragma unroll
  for (int w = 0; w < LOOP_BITS - 1; ++w) bw[w] = w < W ? q[(size_t)(G + w) * n + G + w] : 0;
  {
    unsigned long long r = xa;
    while (r) {
      const int j = __ffsll((long long)r) - 1;
      r &= r - 1;
      const int *row = q + (size_t)j * n;
#pragma unroll
      for (int i = 0; i < G; ++i) ca[i] += row[i];
#pragma unroll
      for (int w = 0; w < LOOP_BITS - 1; ++w)
        if (w < W) bw[w] += row[G + w];
      sumt += rowt[j];
    }
  }
  int c2[G];
#pragma unroll
  for (int i = 0; i < G; ++i) c2[i] = (ca[i] + rowt[i]) * 65536 + ca[i];
  int E2s = (Ea + sumt + PACK_BIAS) * 65536 + (Ea + PACK_BIAS);
  const unsigned npairs = 1u << (P.loop_bits - 1);
  for (unsigned B = 0; B < npairs; ++B) {
    const int m = inner_block_packed<G>(E2s, c2, P);
    if ((B & 7u) == 7u) {
      const long long g = *reinterpret_cast<volatile long long *>(P.gbest);
      if (g < (long long)tb.best) {
        tb.best = (int)g;
        tb.cnt = 0;
        tb.minstate = ~0ull;
      }
    }
    const int ma = (int)((unsigned)m & 0xFFFFu) - PACK_BIAS;
    const int mb = (int)((unsigned)m >> 16) - PACK_BIAS;
    const int mm = min(ma, mb);
    if (mm <= tb.best) {
      if (mm < tb.best) {
        tb.best = mm;
        tb.cnt = 0;
        tb.minstate = ~0ull;
        atomicMin(P.gbest, (long long)mm);
      }
      CVec<int, G> cv;
      if (ma <= tb.best) {
#pragma unroll
        for (int i = 0; i < G; ++i) cv.v[i] = (int)(short)(c2[i] & 0xFFFF);
        revisit_block<int, G, false>(P, cv, xa, (int)((unsigned)E2s & 0xFFFFu) - PACK_BIAS, tb, cs, 0);
      }
      if (mb <= tb.best) {
#pragma unroll
        for (int i = 0; i < G; ++i) cv.v[i] = (c2[i] - (int)(short)(c2[i] & 0xFFFF)) >> 16;
        revisit_block<int, G, false>(P, cv, xa | (1ull << top), (int)((unsigned)E2s >> 16) - PACK_BIAS, tb, cs,
                                     0);
      }
    }
    if (B + 1 < npairs) {
      const int w = __ffs((int)(B + 1)) - 1;
      const int mbit = G + w;
      const unsigned long long bm = 1ull << mbit;
      const bool was = (xa & bm) != 0;
      const int *row = q + (size_t)mbit * n;
      const unsigned walked = (unsigned)(xa >> G) & ((1u << W) - 1u) & ~(1u << w);
      int sum = 0;
#pragma unroll
      for (int v = 0; v < LOOP_BITS - 1; ++v) {
        if (v == w) sum += bw[v];
        if ((walked >> v) & 1u) sum += row[G + v];
      }
      const int sum2 = sum * 65537 + row[top] * 65536;  // half b also has `top` set
      E2s += was ? -sum2 : sum2;
      xa ^= bm;
      const int s65537 = was ? -65537 : 65537;
#pragma unroll
      for (int i = 0; i < G; ++i) c2[i] += row[i] * s65537;
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
__global__ void __launch_bounds__(THREADS, sizeof(T) == 4 ? 5 : 1) gray_kernel(const __grid_constant__ GrayParams<T> P) {
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
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const T d = min(descent_bound_warp(P, 2 * w), descent_bound_warp(P, 2 * w + 1));
    if ((threadIdx.x & 31) == 0) atomicMin(&s_bound, (long long)d);
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
    if (item < items) {
      if constexpr (MODE == 2)
        process_item_packed<G>(item, P, tb, cs);
      else
        process_item<T, G, COLLECT, MODE>(item, P, tb, cs, thr);
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

// Host-side launchers, one translation unit per (type, width):
// exhaustive_gray_i9.cu, exhaustive_gray_i10.cu, exhaustive_gray_l9.cu,
// exhaustive_gray_l10.cu.
template <class T, int G> void launch_gray_width(int variant, bool collect, int grid, cudaStream_t s,
                                                  const GrayParams<T> &P);
template <class T, int G> int gray_occupancy_width(int variant);

}  // namespace exh
}  // namespace os

#endif  // ONESOLVER_EXHAUSTIVE_KERNELS_CUH_
