// sa_kernels.cuh -- the dense simulated-annealing sweep kernels.
//
// Replaces the SYCL kernel of sa::anneal
// (include/simulated_annealing/annealing.hpp:85-126). The reference runs one
// work-item per trajectory and recomputes the full O(n^2) FP64 energy after
// every attempt (:104). Here every trajectory keeps FP32 local fields
// h_j = sum_{i != j} Q_ij x_i, so an attempt at site k costs
//   dE_k = (1 - 2 x_k) (Q_kk + h_k)
// and an accepted flip adds +/- row k of the coupling matrix to the fields.
//
// Layout: one warp per trajectory. Sites are grouped by 128; in group g lane
// l owns the four consecutive sites g*128 + 4l + j (j = 0..3), and "slot"
// s = 4g + j is the set of 32 sites { g*128 + 4l + j : l = 0..31 }. A lane's
// fields sit in registers as FP32 pairs (slots 2q, 2q+1 in one 64-bit
// register) and its spins in one bitmask (bit s). A flip's row update then
// reads the lane's four coupling values of a group with one 128-bit load and
// adds them with two paired FP32 FMAs (fma.rn.f32x2). The slot loop is
// unrolled so every register index is a compile-time constant.
//
// Coupling rows are stored in slot order (row p = s*32 + l holds the
// couplings of site slot_site(s, l), columns in site order), so the rows of
// the sites of one slot are contiguous in memory.
//
// Sequential sweeps visit the slots in order and, within a slot, the lanes in
// order: a fixed permutation of the sites inside each group of 128. The 32
// sites of a slot are decided together: each lane evaluates its own site with
// the current fields; a warp ballot of the accepting lanes gives the next
// site in sweep order that flips. The fields are updated with that site's
// row, and only the lanes after it re-evaluate (the earlier lanes' decisions
// are final because nothing before them changed). A slot therefore costs
// (1 + accepted flips) ballot rounds, and a rejected attempt costs no field
// work.
//
// Acceptance uses the threshold form of the Metropolis test: with
// u ~ U(0,1) from Philox, the reference rule exp((E - E') / beta) > u is
// dE < -beta ln u and the physical rule exp(-beta dE) > u is
// dE < -ln(u) / beta.
//
// Replay (verification) mode: every sweep kernel has a REPLAY instantiation
// that reads the threshold of each attempt (and, for random sites, the site)
// from caller-given arrays instead of drawing it from Philox, and the
// initialisation kernels can take caller-given initial spins. Everything else
// (visit order, ballot rounds, field updates, energy and best-state
// bookkeeping, tiles, resyncs) is the production code path, so a replay on
// integer coefficients, where the FP32 fields and energies are exact, must
// reproduce a CPU transcription of the reference's Metropolis loop
// (annealing.hpp:97-123) in the kernel's site order bit for bit.
#ifndef ONESOLVER_SA_KERNELS_CUH_
#define ONESOLVER_SA_KERNELS_CUH_

#include <cstdint>

#include "philox.cuh"
#include "rescore.cuh"
#include "tma.cuh"

namespace os {
namespace sa {

constexpr unsigned FULL = 0xffffffffu;

// Site owned by `lane` in slot `s`.
__host__ __device__ __forceinline__ int slot_site(int s, int lane) {
  return ((s >> 2) << 7) + (lane << 2) + (s & 3);
}
// Slot and lane of a site.
__host__ __device__ __forceinline__ int site_slot(int k) { return ((k >> 7) << 2) + (k & 3); }
__host__ __device__ __forceinline__ int site_lane(int k) { return (k & 127) >> 2; }

struct DenseArgs {
  const float *c;          // ld x ld couplings (zero diagonal), rows in slot order
  const float *diag;       // ld, site order
  int n, nslots, ld;
  int spb;                 // steps per beta
  const double *beta;      // schedule (device)
  int step_begin, step_end;
  int acceptance;          // os_acceptance
  int traj_count;          // trajectories in this launch
  int traj_offset;         // global index of the first trajectory (RNG)
  uint32_t seed_lo, seed_hi, instance;
  float *h;                // [traj][nslots/2][32] FP32 pairs (slots 2q, 2q+1)
  unsigned long long *x;   // [traj][32] lane masks
  unsigned long long *xbest;
  float *e;                // [traj] tracked energy
  float *ebest;            // [traj]
  unsigned long long *accepted;  // [traj]
  int *status;             // set to 1 when a bounded wait ran out
  // Replay mode only (REPLAY kernels): thresholds and sites of trajectory 0
  // of this launch; sequential sweeps read thr[(t * nsteps + step) * n +
  // site], random sites thr[t * nsteps + step] and rsite[t * nsteps + step].
  const float *thr;
  const int *rsite;
  int nsteps;              // steps of the whole run (row length of thr, rsite)
};

__device__ __forceinline__ float select4(const Philox4 &r, int j) {
  const uint32_t w = j == 0 ? r.x : j == 1 ? r.y : j == 2 ? r.z : r.w;
  return u01_open(w);
}

__device__ __forceinline__ float threshold(float u, float b, int acceptance) {
  const float l = __logf(u);  // < 0
  return acceptance == OS_ACCEPT_REFERENCE ? -b * l : -l / b;
}

__device__ __forceinline__ unsigned long long splat2(float x) {
  const unsigned long long u = __float_as_uint(x);
  return (u << 32) | u;
}

// acc = a * b + acc on both FP32 halves.
__device__ __forceinline__ void ffma2(unsigned long long &acc, unsigned long long a, unsigned long long b) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(a), "l"(b));
}

// One lane's FP32 fields, as pairs.
template <int SLOTS> struct Fields {
  static_assert(SLOTS % 4 == 0, "slots come in groups of four");
  unsigned long long p[SLOTS / 2];

  __device__ __forceinline__ float get(int s) const {
    return (s & 1) ? __uint_as_float((unsigned)(p[s >> 1] >> 32)) : __uint_as_float((unsigned)p[s >> 1]);
  }
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int q = 0; q < SLOTS / 2; ++q) p[q] = 0ull;
  }
  // Field pairs of trajectory t: [t][nslots/2][32] 64-bit words.
  __device__ __forceinline__ static unsigned long long *base(float *h, long long t, int nslots, int lane) {
    return reinterpret_cast<unsigned long long *>(h) + (size_t)t * (nslots / 2) * 32 + lane;
  }
  __device__ __forceinline__ void load(const unsigned long long *src, int nslots) {
#pragma unroll
    for (int q = 0; q < SLOTS / 2; ++q) p[q] = 2 * q < nslots ? src[q * 32] : 0ull;
  }
  __device__ __forceinline__ void store(unsigned long long *dst, int nslots) const {
#pragma unroll
    for (int q = 0; q < SLOTS / 2; ++q)
      if (2 * q < nslots) dst[q * 32] = p[q];
  }
  // fields += sgn * row; `row_lane` = the row's first element + 4 * lane
  // (shared memory: 128-bit shared loads). ALL: nslots == SLOTS, so no group
  // is padding and the per-group test goes away.
  template <bool ALL = false>
  __device__ __forceinline__ void add_row(const float *row_lane, float sgn, int nslots) {
    const unsigned long long s2 = splat2(sgn);
#pragma unroll
    for (int g = 0; g < SLOTS / 4; ++g) {
      if (ALL || 4 * g < nslots) {
        const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(row_lane + g * 128);
        ffma2(p[2 * g], v.x, s2);
        ffma2(p[2 * g + 1], v.y, s2);
      }
    }
  }
  // Same from global memory through the read-only path.
  __device__ __forceinline__ void add_row_global(const float *row_lane, float sgn, int nslots) {
    const unsigned long long s2 = splat2(sgn);
#pragma unroll
    for (int g = 0; g < SLOTS / 4; ++g) {
      if (4 * g < nslots) {
        const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(row_lane + g * 128));
        ffma2(p[2 * g], v.x, s2);
        ffma2(p[2 * g + 1], v.y, s2);
      }
    }
  }
};

// Sequential-order sweeps over [step_begin, step_end), one trajectory per
// warp, rows read from global memory (used when two staged row tiles do not
// fit in shared memory).
template <int SLOTS, bool REPLAY = false>
__global__ void __launch_bounds__(128) sa_dense_seq_kernel(const __grid_constant__ DenseArgs a) {
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= a.traj_count) return;
  const int nslots = a.nslots;
  Fields<SLOTS> F;
  unsigned long long *hq = Fields<SLOTS>::base(a.h, t, nslots, lane);
  F.load(hq, nslots);
  unsigned long long xl = a.x[(size_t)t * 32 + lane];
  unsigned long long xb = a.xbest[(size_t)t * 32 + lane];
  float E = a.e[t], Eb = a.ebest[t];
  unsigned long long acc = 0;
  const uint32_t tg = (uint32_t)(a.traj_offset + t);
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSweep;

  for (int step = a.step_begin; step < a.step_end; ++step) {
    const float b = (float)a.beta[step / a.spb];
    Philox4 r{0, 0, 0, 0};
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      if (s >= nslots) break;
      const int site = slot_site(s, lane);
      const bool valid = site < a.n;
      float theta;
      if constexpr (REPLAY) {
        theta = valid ? a.thr[((size_t)t * a.nsteps + step) * a.n + site] : 0.f;
      } else {
        if ((s & 3) == 0)
          r = philox4x32_10((uint32_t)((s >> 2) * 32 + lane), (uint32_t)step, tg, c3, a.seed_lo, a.seed_hi);
        theta = threshold(select4(r, s & 3), b, a.acceptance);
      }
      const float d = a.diag[site];
      const unsigned xs0 = __ballot_sync(FULL, (xl >> s) & 1ull);  // spins at the start of the slot
      int p = 0;
      for (;;) {
        const bool xs = (xl >> s) & 1ull;
        const float loc = d + F.get(s);
        const float dE = xs ? -loc : loc;
        const unsigned mask = __ballot_sync(FULL, valid && lane >= p && dE < theta);
        if (!mask) break;
        const int i = __ffs(mask) - 1;
        const float dEi = __shfl_sync(FULL, dE, i);
        const bool xi = (xs0 >> i) & 1u;
        F.add_row_global(a.c + (size_t)(s * 32 + i) * a.ld + 4 * lane, xi ? -1.f : 1.f, nslots);
        if (lane == i) xl ^= 1ull << s;
        E += dEi;
        ++acc;
        if (E < Eb) {
          Eb = E;
          xb = xl;
        }
        p = i + 1;
      }
    }
  }
  F.store(hq, nslots);
  a.x[(size_t)t * 32 + lane] = xl;
  a.xbest[(size_t)t * 32 + lane] = xb;
  if (lane == 0) {
    a.e[t] = E;
    a.ebest[t] = Eb;
    a.accepted[t] += acc;
  }
}

// Random-order steps (the reference's one random site per step,
// annealing.hpp:97-101) for one trajectory per warp.
template <int SLOTS, bool REPLAY = false>
__global__ void __launch_bounds__(128) sa_dense_rand_kernel(const __grid_constant__ DenseArgs a) {
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= a.traj_count) return;
  const int nslots = a.nslots;
  Fields<SLOTS> F;
  unsigned long long *hq = Fields<SLOTS>::base(a.h, t, nslots, lane);
  F.load(hq, nslots);
  unsigned long long xl = a.x[(size_t)t * 32 + lane];
  unsigned long long xb = a.xbest[(size_t)t * 32 + lane];
  float E = a.e[t], Eb = a.ebest[t];
  unsigned long long acc = 0;
  const uint32_t tg = (uint32_t)(a.traj_offset + t);
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSite;
  Philox4 r{0, 0, 0, 0};
  for (int step = a.step_begin; step < a.step_end; ++step) {
    int k;
    float theta;
    if constexpr (REPLAY) {
      k = a.rsite[(size_t)t * a.nsteps + step];
      theta = a.thr[(size_t)t * a.nsteps + step];
    } else {
      const float b = (float)a.beta[step / a.spb];
      if ((step & 1) == 0 || step == a.step_begin)
        r = philox4x32_10((uint32_t)(step >> 1), 0u, tg, c3, a.seed_lo, a.seed_hi);
      const bool second = step & 1;
      const uint32_t wk = second ? r.z : r.x;
      const uint32_t wu = second ? r.w : r.y;
      k = (int)__umulhi(wk, (uint32_t)a.n);
      theta = threshold(u01_open(wu), b, a.acceptance);
    }
    const int slot = site_slot(k), owner = site_lane(k);
    float hv = 0.f;
#pragma unroll
    for (int s = 0; s < SLOTS; ++s)
      if (s == slot) hv = F.get(s);
    const bool xs = (xl >> slot) & 1ull;
    const float loc = a.diag[slot_site(slot, lane)] + hv;
    const float dEl = xs ? -loc : loc;
    const float dE = __shfl_sync(FULL, dEl, owner);
    const bool xk = __shfl_sync(FULL, xs, owner);
    if (dE < theta) {
      F.add_row_global(a.c + (size_t)(slot * 32 + owner) * a.ld + 4 * lane, xk ? -1.f : 1.f, nslots);
      if (lane == owner) xl ^= 1ull << slot;
      E += dE;
      ++acc;
      if (E < Eb) {
        Eb = E;
        xb = xl;
      }
    }
  }
  F.store(hq, nslots);
  a.x[(size_t)t * 32 + lane] = xl;
  a.xbest[(size_t)t * 32 + lane] = xb;
  if (lane == 0) {
    a.e[t] = E;
    a.ebest[t] = Eb;
    a.accepted[t] += acc;
  }
}

// Sequential sweeps with the coupling rows staged in shared memory.
//
// A CTA runs W trajectories (one warp each) of the same instance in lockstep
// over half-slots of 16 sites. The 16 coupling rows of a half-slot (16 x ld
// FP32, contiguous in global memory) arrive by one bulk async copy (TMA) into
// one of two buffers while the previous half-slot is processed, and every
// warp of the CTA takes its flip rows from that tile: the rows are read from
// L2 once per CTA instead of once per accepted flip per trajectory, and no
// flip waits on a global load. Tiles run round-robin through the sweep, so
// the first tiles of the next sweep stream in during the last ones of the
// current sweep.
constexpr int TILE_ROWS = 16;
constexpr uint32_t TILE_WAIT_LIMIT = 1u << 26;
// Largest padded row length whose two 16-row tiles fit in shared memory.
constexpr int TILE_MAX_LD = 1792;

// One item: the W trajectories of `a` (pointers already at the item's first
// trajectory, warp w runs trajectory w), steps [step_begin, step_end).
// `tiles` holds two buffers of TILE_ROWS x ld floats, `bar` their mbarriers,
// `parity` their phase bits (kept by the caller across items). Returns false
// when a bounded wait ran out (uniformly for the whole CTA).
template <int SLOTS, bool ALL, bool REPLAY>
__device__ __forceinline__ bool tile_item_impl(const DenseArgs &a, float *tiles, uint64_t *bar,
                                               uint32_t (&parity)[2]) {
  const int lane = threadIdx.x & 31;
  const int t = threadIdx.x >> 5;
  const bool active = t < a.traj_count;
  const int nslots = a.nslots, ld = a.ld;
  const size_t tile_floats = (size_t)TILE_ROWS * ld;
  const uint32_t tile_bytes = (uint32_t)(tile_floats * sizeof(float));
  const int halves = 2 * nslots;
  const long long total = (long long)(a.step_end - a.step_begin) * halves;

  Fields<SLOTS> F;
  unsigned long long xl = 0, xb = 0;
  float E = 0.f, Eb = 0.f;
  unsigned long long *hq = Fields<SLOTS>::base(a.h, t, nslots, lane);
  if (active) {
    F.load(hq, nslots);
    xl = a.x[(size_t)t * 32 + lane];
    xb = a.xbest[(size_t)t * 32 + lane];
    E = a.e[t];
    Eb = a.ebest[t];
  } else {
    F.zero();
  }
  unsigned long long acc = 0;
  const uint32_t tg = (uint32_t)(a.traj_offset + t);
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSweep;

  auto issue = [&](long long g) {
    const int hs = (int)(g % halves);
    const int b = (int)(g & 1);
    mbar_arrive_expect_tx(&bar[b], tile_bytes);
    bulk_load(tiles + (size_t)b * tile_floats, a.c + (size_t)hs * TILE_ROWS * ld, tile_bytes, &bar[b]);
  };
  if (threadIdx.x == 0) {
    if (total > 0) issue(0);
    if (total > 1) issue(1);
  }
  long long g = 0;
  for (int step = a.step_begin; step < a.step_end; ++step) {
    const float b = (float)a.beta[step / a.spb];
    Philox4 r{0, 0, 0, 0};
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      if (s >= nslots) break;
      const int site = slot_site(s, lane);
      const bool valid = site < a.n;
      float theta;
      if constexpr (REPLAY) {
        theta = (active && valid) ? a.thr[((size_t)t * a.nsteps + step) * a.n + site] : 0.f;
      } else {
        if ((s & 3) == 0)
          r = philox4x32_10((uint32_t)((s >> 2) * 32 + lane), (uint32_t)step, tg, c3, a.seed_lo, a.seed_hi);
        theta = threshold(select4(r, s & 3), b, a.acceptance);
      }
      const float d = a.diag[site];
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const bool ok = mbar_wait_bounded(&bar[half], parity[half], TILE_WAIT_LIMIT);
        parity[half] ^= 1u;
        if (active && ok) {
          const float *tile = tiles + (size_t)half * tile_floats;
          int p = half * TILE_ROWS;
          const int pend = p + TILE_ROWS;
          // Spins of the slot at the start of the half: a lane's spin only
          // changes when that lane flips, after which it is past p.
          const unsigned xs0 = __ballot_sync(FULL, (xl >> s) & 1ull);
          for (;;) {
            const bool xs = (xl >> s) & 1ull;
            const float loc = d + F.get(s);
            const float dE = xs ? -loc : loc;
            const unsigned mask = __ballot_sync(FULL, valid && lane >= p && lane < pend && dE < theta);
            if (!mask) break;
            const int i = __ffs(mask) - 1;
            const float dEi = __shfl_sync(FULL, dE, i);
            const bool xi = (xs0 >> i) & 1u;
            F.template add_row<ALL>(tile + (size_t)(i - half * TILE_ROWS) * ld + 4 * lane, xi ? -1.f : 1.f, nslots);
            if (lane == i) xl ^= 1ull << s;
            E += dEi;
            ++acc;
            if (E < Eb) {
              Eb = E;
              xb = xl;
            }
            p = i + 1;
          }
        }
        // Every warp is done with this buffer; refill it with tile g + 2.
        if (__syncthreads_or(!ok)) {
          // Let copies still in flight land (bounded) before returning: the
          // phases of tile g (whose wait ran out; its parity bit is already
          // flipped) and of tile g + 1 (when the run has it; else the wait
          // just runs out).
          if (threadIdx.x == 0) {
            for (int b2 = 0; b2 < 2; ++b2)
              mbar_wait_bounded(&bar[b2], parity[b2] ^ (b2 == half ? 1u : 0u), TILE_WAIT_LIMIT);
            if (a.status) atomicExch(a.status, 1);
          }
          return false;
        }
        if (threadIdx.x == 0 && g + 2 < total) issue(g + 2);
        ++g;
      }
    }
  }
  if (active) {
    F.store(hq, nslots);
    a.x[(size_t)t * 32 + lane] = xl;
    a.xbest[(size_t)t * 32 + lane] = xb;
    if (lane == 0) {
      a.e[t] = E;
      a.ebest[t] = Eb;
      a.accepted[t] += acc;
    }
  }
  return true;
}

// An instance whose slot count fills the kernel's class (nslots == SLOTS)
// takes the variant without per-group padding tests (8% faster at
// n = 1024); the others keep the tests.
template <int SLOTS, bool REPLAY = false>
__device__ __forceinline__ bool tile_item(const DenseArgs &a, float *tiles, uint64_t *bar, uint32_t (&parity)[2]) {
  return a.nslots == SLOTS ? tile_item_impl<SLOTS, true, REPLAY>(a, tiles, bar, parity)
                           : tile_item_impl<SLOTS, false, REPLAY>(a, tiles, bar, parity);
}

__device__ __forceinline__ void init_tile_barriers(uint64_t *bar) {
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
}

// One CTA per block of W trajectories of one instance.
template <int SLOTS, bool REPLAY = false>
__global__ void __launch_bounds__(512) sa_dense_tile_kernel(const __grid_constant__ DenseArgs a) {
  extern __shared__ __align__(128) unsigned char tile_smem[];
  __shared__ __align__(8) uint64_t bar[2];
  init_tile_barriers(bar);
  const int W = blockDim.x >> 5;
  const size_t first = (size_t)blockIdx.x * W;
  DenseArgs it = a;
  it.traj_count = a.traj_count - (int)first < W ? a.traj_count - (int)first : W;
  it.traj_offset = a.traj_offset + (int)first;
  it.h = a.h + first * a.nslots * 32;
  it.x = a.x + first * 32;
  it.xbest = a.xbest + first * 32;
  it.e = a.e + first;
  it.ebest = a.ebest + first;
  it.accepted = a.accepted + first;
  if constexpr (REPLAY) it.thr = a.thr + first * a.nsteps * a.n;
  uint32_t parity[2] = {0u, 0u};
  tile_item<SLOTS, REPLAY>(it, reinterpret_cast<float *>(tile_smem), bar, parity);
}

constexpr int TILE_MAX_BUFS = 3;
constexpr size_t TILE_SMEM_BUDGET = (size_t)220 * 1024;
// Tile buffers of a staged sweep of rows of ld floats, and their bytes.
__host__ __device__ __forceinline__ int tile_buffers(int ld) {
  return (size_t)TILE_MAX_BUFS * TILE_ROWS * ld * sizeof(float) <= TILE_SMEM_BUDGET ? TILE_MAX_BUFS : 2;
}
__host__ __device__ __forceinline__ size_t tile_smem_bytes(int ld) {
  return (size_t)tile_buffers(ld) * TILE_ROWS * ld * sizeof(float);
}
// Shared state of the tile pipeline.
struct TileSync {
  uint64_t full[TILE_MAX_BUFS];    // a buffer's copy has landed (transaction bytes)
  unsigned done[TILE_MAX_BUFS];    // warps done with a buffer's current tile
  unsigned issued[TILE_MAX_BUFS];  // copies issued into a buffer since launch (one phase each)
  int fail;                        // a bounded wait ran out
};

// Wait for buffer b's copy of the given phase; false once any warp's wait has
// run out (TILE_WAIT_LIMIT polls, then the flag is set for all).
__device__ __forceinline__ bool tile_wait(TileSync *ts, int b, uint32_t parity) {
  for (uint32_t i = 0; i < TILE_WAIT_LIMIT; ++i) {
    if (mbar_try_wait(&ts->full[b], parity)) return true;
    if (*reinterpret_cast<volatile int *>(&ts->fail)) return false;
  }
  *reinterpret_cast<volatile int *>(&ts->fail) = 1;
  return false;
}

// The batched kernel's form of the staged sweep: the same sweep as
// tile_item_impl, with NB = 3 tile buffers where three fit and no CTA-wide
// barrier between half-slots: each warp counts itself done with a buffer,
// and the last warp to finish a tile issues the copy of the tile NB
// half-slots later into it, so a warp with few flips in a half-slot runs
// ahead of one with many (by up to NB - 1 tiles) instead of waiting for it.
// With 16 trajectories per CTA (the slowest of 16 warps sets a half-slot's
// pace under a barrier) this is 7% faster on the batched configuration; the
// dense kernel, 4 trajectories per CTA on SK n = 1,024, keeps the barrier
// form above, which measured 12% faster there than this one.
template <int SLOTS, bool ALL, bool REPLAY>
__device__ __forceinline__ bool batch_tile_item_impl(const DenseArgs &a, float *tiles, TileSync *ts,
                                               uint32_t &phase) {
  const int lane = threadIdx.x & 31;
  const int t = threadIdx.x >> 5;
  const bool active = t < a.traj_count;
  const int nslots = a.nslots, ld = a.ld;
  const size_t tile_floats = (size_t)TILE_ROWS * ld;
  const uint32_t tile_bytes = (uint32_t)(tile_floats * sizeof(float));
  const int halves = 2 * nslots;
  const long long total = (long long)(a.step_end - a.step_begin) * halves;
  const int NB = tile_buffers(ld);
  const unsigned nwarps = blockDim.x >> 5;

  Fields<SLOTS> F;
  unsigned long long xl = 0, xb = 0;
  float E = 0.f, Eb = 0.f;
  unsigned long long *hq = Fields<SLOTS>::base(a.h, t, nslots, lane);
  if (active) {
    F.load(hq, nslots);
    xl = a.x[(size_t)t * 32 + lane];
    xb = a.xbest[(size_t)t * 32 + lane];
    E = a.e[t];
    Eb = a.ebest[t];
  } else {
    F.zero();
  }
  unsigned long long acc = 0;
  const uint32_t tg = (uint32_t)(a.traj_offset + t);
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSweep;

  // Tile g (half-slot g mod halves of the run) goes to buffer g mod NB.
  auto issue = [&](long long g, int b) {
    const int hs = (int)(g % halves);
    ++ts->issued[b];
    mbar_arrive_expect_tx(&ts->full[b], tile_bytes);
    bulk_load(tiles + (size_t)b * tile_floats, a.c + (size_t)hs * TILE_ROWS * ld, tile_bytes, &ts->full[b]);
  };
  if (threadIdx.x == 0)
    for (int g0 = 0; g0 < NB && g0 < total; ++g0) issue(g0, g0);
  long long g = 0;
  int buf = 0;  // buffer of tile g
  bool failed = false;
  for (int step = a.step_begin; step < a.step_end; ++step) {
    const float b = (float)a.beta[step / a.spb];
    Philox4 r{0, 0, 0, 0};
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      if (s >= nslots) break;
      const int site = slot_site(s, lane);
      const bool valid = site < a.n;
      float theta;
      if constexpr (REPLAY) {
        theta = (active && valid) ? a.thr[((size_t)t * a.nsteps + step) * a.n + site] : 0.f;
      } else {
        if ((s & 3) == 0)
          r = philox4x32_10((uint32_t)((s >> 2) * 32 + lane), (uint32_t)step, tg, c3, a.seed_lo, a.seed_hi);
        theta = threshold(select4(r, s & 3), b, a.acceptance);
      }
      const float d = a.diag[site];
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const bool ok = !failed && tile_wait(ts, buf, (phase >> buf) & 1u);
        phase ^= 1u << buf;
        failed = !ok;
        if (active && ok) {
          const float *tile = tiles + (size_t)buf * tile_floats;
          int p = half * TILE_ROWS;
          const int pend = p + TILE_ROWS;
          // Spins of the slot at the start of the half: a lane's spin only
          // changes when that lane flips, after which it is past p.
          const unsigned xs0 = __ballot_sync(FULL, (xl >> s) & 1ull);
          for (;;) {
            const bool xs = (xl >> s) & 1ull;
            const float loc = d + F.get(s);
            const float dE = xs ? -loc : loc;
            const unsigned mask = __ballot_sync(FULL, valid && lane >= p && lane < pend && dE < theta);
            if (!mask) break;
            const int i = __ffs(mask) - 1;
            const float dEi = __shfl_sync(FULL, dE, i);
            const bool xi = (xs0 >> i) & 1u;
            F.template add_row<ALL>(tile + (size_t)(i - half * TILE_ROWS) * ld + 4 * lane, xi ? -1.f : 1.f, nslots);
            if (lane == i) xl ^= 1ull << s;
            E += dEi;
            ++acc;
            if (E < Eb) {
              Eb = E;
              xb = xl;
            }
            p = i + 1;
          }
        }
        // This warp is done with buffer buf; the last warp to finish it
        // refills it with tile g + NB.
        __syncwarp();
        if (lane == 0) {
          __threadfence_block();
          if (atomicAdd(&ts->done[buf], 1u) == nwarps - 1) {
            ts->done[buf] = 0;
            __threadfence_block();
            if (g + NB < total && !*reinterpret_cast<volatile int *>(&ts->fail)) issue(g + NB, buf);
          }
        }
        ++g;
        buf = buf + 1 == NB ? 0 : buf + 1;
      }
    }
  }
  if (__syncthreads_or(failed)) {
    // Let copies still in flight land (bounded) before returning. A buffer
    // is refilled only after every warp's wait for its previous copy
    // succeeded, so at most its last issued copy is in flight: wait for
    // that copy's phase. (The warps' `phase` bits also count the tiles they
    // skipped after the failure, so they do not name it.)
    if (threadIdx.x == 0) {
      for (int b2 = 0; b2 < NB; ++b2)
        if (ts->issued[b2]) mbar_wait_bounded(&ts->full[b2], (ts->issued[b2] - 1u) & 1u, TILE_WAIT_LIMIT);
      if (a.status) atomicExch(a.status, 1);
    }
    return false;
  }
  if (active) {
    F.store(hq, nslots);
    a.x[(size_t)t * 32 + lane] = xl;
    a.xbest[(size_t)t * 32 + lane] = xb;
    if (lane == 0) {
      a.e[t] = E;
      a.ebest[t] = Eb;
      a.accepted[t] += acc;
    }
  }
  return true;
}

// An instance whose slot count fills the kernel's class (nslots == SLOTS)
// takes the variant without per-group padding tests (8% faster at
// n = 1024); the others keep the tests.
template <int SLOTS, bool REPLAY = false>
__device__ __forceinline__ bool batch_tile_item(const DenseArgs &a, float *tiles, TileSync *ts, uint32_t &phase) {
  return a.nslots == SLOTS ? batch_tile_item_impl<SLOTS, true, REPLAY>(a, tiles, ts, phase)
                           : batch_tile_item_impl<SLOTS, false, REPLAY>(a, tiles, ts, phase);
}

__device__ __forceinline__ void init_tile_sync(TileSync *ts) {
  if (threadIdx.x == 0) {
    for (int b = 0; b < TILE_MAX_BUFS; ++b) {
      mbar_init(&ts->full[b], 1);
      ts->done[b] = 0;
      ts->issued[b] = 0;
    }
    ts->fail = 0;
    mbar_fence_init();
  }
  __syncthreads();
}

// Many instances in one persistent launch: items are (instance, block of W
// trajectories), taken largest first from a global counter.
struct BatchInstance {
  const float *c;
  const float *diag;
  const double *c64;
  const double *d64;
  const double *f;
  int n, nslots, ld, T;
  long long h_off;      // first field of the instance's first trajectory
  long long traj_base;  // global index of its first trajectory
};

struct BatchArgs {
  const BatchInstance *inst;
  const int2 *items;           // (instance, first trajectory within it)
  int num_items;
  unsigned int *work;          // item counter
  int W;
  const double *beta;
  int spb, step_begin, step_end, acceptance;
  uint32_t seed_lo, seed_hi;
  float *h;
  unsigned long long *x, *xbest;
  float *e, *ebest;
  unsigned long long *accepted;
  int *status;
  // Replay mode only: thresholds of all trajectories of all instances,
  // instance after instance, [T][nsteps][n_k] each; trajectory g's block
  // starts at nsteps * state_off[g].
  const float *thr;
  const long long *state_off;
  int nsteps;
};

template <int SLOTS, bool REPLAY = false>
__global__ void __launch_bounds__(512) sa_batch_tile_kernel(const __grid_constant__ BatchArgs B) {
  extern __shared__ __align__(128) unsigned char tile_smem[];
  __shared__ __align__(8) TileSync ts;
  __shared__ int s_item;
  init_tile_sync(&ts);
  uint32_t phase = 0u;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(B.work, 1u);
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item >= B.num_items) break;
    const int2 id = B.items[item];
    const BatchInstance in = B.inst[id.x];
    const long long g0 = in.traj_base + id.y;   // global trajectory index
    DenseArgs a;
    a.c = in.c;
    a.diag = in.diag;
    a.n = in.n;
    a.nslots = in.nslots;
    a.ld = in.ld;
    a.spb = B.spb;
    a.beta = B.beta;
    a.step_begin = B.step_begin;
    a.step_end = B.step_end;
    a.acceptance = B.acceptance;
    a.traj_count = in.T - id.y < B.W ? in.T - id.y : B.W;
    a.traj_offset = id.y;
    a.seed_lo = B.seed_lo;
    a.seed_hi = B.seed_hi;
    a.instance = (uint32_t)id.x;
    a.h = B.h + in.h_off + (long long)id.y * in.nslots * 32;
    a.x = B.x + g0 * 32;
    a.xbest = B.xbest + g0 * 32;
    a.e = B.e + g0;
    a.ebest = B.ebest + g0;
    a.accepted = B.accepted + g0;
    a.status = B.status;
    if constexpr (REPLAY) {
      a.thr = B.thr + (long long)B.nsteps * B.state_off[g0];
      a.nsteps = B.nsteps;
    }
    if (!batch_tile_item<SLOTS, REPLAY>(a, reinterpret_cast<float *>(tile_smem), &ts, phase)) break;
  }
}

struct ResyncArgs {
  const double *c64;       // ld x ld FP64 couplings (zero diagonal), site order
  const double *d64;       // ld
  int n, nslots, ld;
  int init;                // 1: draw the initial spins first
  const float *init_prob;  // optional warm start (n)
  int traj_count, traj_offset;
  uint32_t seed_lo, seed_hi, instance;
  float *h;
  unsigned long long *x;
  unsigned long long *xbest;
  float *e;
  float *ebest;
  unsigned long long *drift_bits;  // max |h32 - h64| as ordered FP64 bits
  const uint8_t *init_bits;        // optional initial spins [traj][n] (replay mode)
};

// FP64 field resync (and initialisation) of trajectory t of `a`:
// h_j = sum_{i set, i != j} Q_ij in FP64 from the current spins, the drift of
// the FP32 fields against it, and the FP64 energy E = sum_{i set} (Q_ii + h_i/2).
// RNG index of the trajectory: a.traj_offset + t.
template <int SLOTS>
__device__ __forceinline__ void resync_traj(const ResyncArgs &a, int t) {
  const int lane = threadIdx.x & 31;
  const int nslots = a.nslots;
  unsigned long long xl;
  if (a.init) {
    xl = 0;
    const uint32_t tg = (uint32_t)(a.traj_offset + t);
    const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamInit;
    Philox4 r{0, 0, 0, 0};
    for (int s = 0; s < nslots; ++s) {
      if ((s & 3) == 0)
        r = philox4x32_10((uint32_t)((s >> 2) * 32 + lane), 0u, tg, c3, a.seed_lo, a.seed_hi);
      const int site = slot_site(s, lane);
      if (site >= a.n) continue;
      const uint32_t w = (s & 3) == 0 ? r.x : (s & 3) == 1 ? r.y : (s & 3) == 2 ? r.z : r.w;
      bool bit = a.init_prob ? (u01_open(w) < a.init_prob[site]) : (w >> 31) != 0;
      if (a.init_bits) bit = a.init_bits[(size_t)t * a.n + site] != 0;
      if (bit) xl |= 1ull << s;
    }
  } else {
    xl = a.x[(size_t)t * 32 + lane];
  }
  double h64[SLOTS];
#pragma unroll
  for (int s = 0; s < SLOTS; ++s) h64[s] = 0.0;
  for (int s = 0; s < nslots; ++s) {
    unsigned m = __ballot_sync(FULL, (xl >> s) & 1ull);
    while (m) {
      const int i = __ffs(m) - 1;
      m &= m - 1;
      const double *row = a.c64 + (size_t)slot_site(s, i) * a.ld + 4 * lane;
#pragma unroll
      for (int s2 = 0; s2 < SLOTS; ++s2)
        if (s2 < nslots) h64[s2] += row[(s2 >> 2) * 128 + (s2 & 3)];
    }
  }
  double epart = 0.0, drift = 0.0;
  unsigned long long *hq = Fields<SLOTS>::base(a.h, t, nslots, lane);
#pragma unroll
  for (int q = 0; q < SLOTS / 2; ++q) {
    if (2 * q >= nslots) break;
    const unsigned long long old = hq[q * 32];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int s = 2 * q + e;
      const int site = slot_site(s, lane);
      if (site < a.n) {
        const float h32 = e ? __uint_as_float((unsigned)(old >> 32)) : __uint_as_float((unsigned)old);
        if (!a.init) drift = fmax(drift, fabs((double)h32 - h64[s]));
        if ((xl >> s) & 1ull) epart += a.d64[site] + 0.5 * h64[s];
      }
    }
    hq[q * 32] = ((unsigned long long)__float_as_uint((float)h64[2 * q + 1]) << 32) |
                 __float_as_uint((float)h64[2 * q]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    epart += __shfl_xor_sync(FULL, epart, off);
    drift = fmax(drift, __shfl_xor_sync(FULL, drift, off));
  }
  a.x[(size_t)t * 32 + lane] = xl;
  if (a.init) a.xbest[(size_t)t * 32 + lane] = xl;
  if (lane == 0) {
    a.e[t] = (float)epart;
    if (a.init) a.ebest[t] = (float)epart;
    if (!a.init && a.drift_bits)
      atomicMax(a.drift_bits, (unsigned long long)__double_as_longlong(drift));
  }
}

template <int SLOTS>
__global__ void __launch_bounds__(128) sa_dense_resync_kernel(const __grid_constant__ ResyncArgs a) {
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= a.traj_count) return;
  resync_traj<SLOTS>(a, t);
}

// Batched resync: one warp per trajectory of any instance.
struct BatchResyncArgs {
  const BatchInstance *inst;
  const int *traj_inst;        // instance of each global trajectory
  long long total;
  int init;
  uint32_t seed_lo, seed_hi;
  float *h;
  unsigned long long *x, *xbest;
  float *e, *ebest;
  unsigned long long *drift_bits;
  // Replay mode only: initial spins of all trajectories, instance after
  // instance ([T][n_k] each); trajectory g's row starts at state_off[g].
  const uint8_t *init_bits;
  const long long *state_off;
};

template <int SLOTS>
__global__ void __launch_bounds__(128) sa_batch_resync_kernel(const __grid_constant__ BatchResyncArgs B) {
  const long long gt = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (gt >= B.total) return;
  const int k = B.traj_inst[gt];
  const BatchInstance in = B.inst[k];
  const int t = (int)(gt - in.traj_base);
  ResyncArgs a;
  a.c64 = in.c64;
  a.d64 = in.d64;
  a.n = in.n;
  a.nslots = in.nslots;
  a.ld = in.ld;
  a.init = B.init;
  a.init_prob = nullptr;
  a.traj_count = in.T;
  a.traj_offset = 0;
  a.seed_lo = B.seed_lo;
  a.seed_hi = B.seed_hi;
  a.instance = (uint32_t)k;
  a.h = B.h + in.h_off;
  a.x = B.x + in.traj_base * 32;
  a.xbest = B.xbest + in.traj_base * 32;
  a.e = B.e + in.traj_base;
  a.ebest = B.ebest + in.traj_base;
  a.drift_bits = B.drift_bits;
  a.init_bits = B.init_bits ? B.init_bits + B.state_off[in.traj_base] : nullptr;
  resync_traj<SLOTS>(a, t);
}

// Spin of site k from the lane masks of one trajectory.
__device__ __forceinline__ uint8_t spin_of(const unsigned long long *xm, int k) {
  return (uint8_t)((xm[site_lane(k)] >> site_slot(k)) & 1ull);
}

// Batched best states -> bytes and FP64 re-score (one CTA of RESCORE_WARPS
// warps per trajectory, rescore_energy_block).
static __global__ void __launch_bounds__(RESCORE_WARPS * 32) sa_batch_rescore_kernel(
    const BatchInstance *__restrict__ inst, const int *__restrict__ traj_inst,
    const long long *__restrict__ state_off, long long total, const unsigned long long *__restrict__ xbest,
    uint8_t *__restrict__ states, double *__restrict__ e64) {
  __shared__ unsigned xw[64];
  __shared__ double red[RESCORE_WARPS];
  const long long gt = blockIdx.x;
  if (gt >= total) return;
  const BatchInstance in = inst[traj_inst[gt]];
  uint8_t *out = states + state_off[gt];
  for (int site = threadIdx.x; site < in.n; site += blockDim.x) out[site] = spin_of(xbest + gt * 32, site);
  __syncthreads();
  const double e = rescore_energy_block(in.f, in.n, out, xw, red);
  if (threadIdx.x == 0) e64[gt] = e;
}

// Best states as one byte per variable, for the FP64 re-score.
static __global__ void unpack_states_kernel(const unsigned long long *__restrict__ xbest, int n, int traj_count,
                                            uint8_t *__restrict__ out) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)traj_count * n) return;
  const int t = (int)(idx / n), site = (int)(idx % n);
  out[idx] = spin_of(xbest + (size_t)t * 32, site);
}

}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_KERNELS_CUH_
