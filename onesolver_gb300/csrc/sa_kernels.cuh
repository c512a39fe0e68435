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
// Layout: one warp per trajectory. Lane l owns sites s*32 + l for the slots
// s < nslots; their fields sit in registers (h[s]) and their spins in one
// lane-private bitmask (bit s). The slot loop is unrolled so every register
// index is a compile-time constant.
//
// Sequential sweeps: the 32 sites of a slot are decided together. Each lane
// evaluates its own site with the current fields; a warp ballot of the
// accepting lanes gives the next site in sweep order that flips. The fields
// are updated with that site's row, and only the lanes after it re-evaluate
// (the earlier lanes' decisions are final because nothing before them
// changed). A slot therefore costs (1 + accepted flips) ballot rounds, and a
// rejected attempt costs no field work.
//
// Acceptance uses the threshold form of the Metropolis test: with
// u ~ U(0,1) from Philox, the reference rule exp((E - E') / beta) > u is
// dE < -beta ln u and the physical rule exp(-beta dE) > u is
// dE < -ln(u) / beta.
#ifndef ONESOLVER_SA_KERNELS_CUH_
#define ONESOLVER_SA_KERNELS_CUH_

#include <cstdint>

#include "philox.cuh"
#include "tma.cuh"

namespace os {
namespace sa {

constexpr unsigned FULL = 0xffffffffu;

struct DenseArgs {
  const float *c;          // ld x ld couplings (zero diagonal)
  const float *diag;       // ld
  int n, nslots, ld;
  int spb;                 // steps per beta
  const double *beta;      // schedule (device)
  int step_begin, step_end;
  int acceptance;          // os_acceptance
  int traj_count;          // trajectories in this launch
  int traj_offset;         // global index of the first trajectory (RNG)
  uint32_t seed_lo, seed_hi, instance;
  float *h;                // [traj][nslots][32]
  unsigned long long *x;   // [traj][32] lane masks
  unsigned long long *xbest;
  float *e;                // [traj] tracked energy
  float *ebest;            // [traj]
  unsigned long long *accepted;  // [traj]
  int *status;             // set to 1 when a bounded wait ran out
};

__device__ __forceinline__ float select4(const Philox4 &r, int j) {
  const uint32_t w = j == 0 ? r.x : j == 1 ? r.y : j == 2 ? r.z : r.w;
  return u01_open(w);
}

__device__ __forceinline__ float threshold(float u, float b, int acceptance) {
  const float l = __logf(u);  // < 0
  return acceptance == OS_ACCEPT_REFERENCE ? -b * l : -l / b;
}

// Sequential-order sweeps over [step_begin, step_end) for one trajectory per
// warp.
template <int SLOTS>
__global__ void __launch_bounds__(128) sa_dense_seq_kernel(const __grid_constant__ DenseArgs a) {
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= a.traj_count) return;
  const int nslots = a.nslots;
  float h[SLOTS];
  float *hp = a.h + (size_t)t * nslots * 32 + lane;
#pragma unroll
  for (int s = 0; s < SLOTS; ++s) h[s] = s < nslots ? hp[s * 32] : 0.f;
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
      if ((s & 3) == 0)
        r = philox4x32_10((uint32_t)((s >> 2) * 32 + lane), (uint32_t)step, tg, c3, a.seed_lo,
                          a.seed_hi);
      const float theta = threshold(select4(r, s & 3), b, a.acceptance);
      const int site = s * 32 + lane;
      const bool valid = site < a.n;
      const float d = a.diag[site];
      int p = 0;
      for (;;) {
        const bool xs = (xl >> s) & 1ull;
        const float loc = d + h[s];
        const float dE = xs ? -loc : loc;
        const unsigned mask = __ballot_sync(FULL, valid && lane >= p && dE < theta);
        if (!mask) break;
        const int i = __ffs(mask) - 1;
        const float dEi = __shfl_sync(FULL, dE, i);
        const bool xi = __shfl_sync(FULL, xs, i);
        const float sgn = xi ? -1.f : 1.f;
        const float *row = a.c + (size_t)(s * 32 + i) * a.ld + lane;
#pragma unroll
        for (int s2 = 0; s2 < SLOTS; ++s2)
          if (s2 < nslots) h[s2] = fmaf(sgn, __ldg(row + s2 * 32), h[s2]);
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
#pragma unroll
  for (int s = 0; s < SLOTS; ++s)
    if (s < nslots) hp[s * 32] = h[s];
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
template <int SLOTS>
__global__ void __launch_bounds__(128) sa_dense_rand_kernel(const __grid_constant__ DenseArgs a) {
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= a.traj_count) return;
  const int nslots = a.nslots;
  float h[SLOTS];
  float *hp = a.h + (size_t)t * nslots * 32 + lane;
#pragma unroll
  for (int s = 0; s < SLOTS; ++s) h[s] = s < nslots ? hp[s * 32] : 0.f;
  unsigned long long xl = a.x[(size_t)t * 32 + lane];
  unsigned long long xb = a.xbest[(size_t)t * 32 + lane];
  float E = a.e[t], Eb = a.ebest[t];
  unsigned long long acc = 0;
  const uint32_t tg = (uint32_t)(a.traj_offset + t);
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSite;
  Philox4 r{0, 0, 0, 0};
  for (int step = a.step_begin; step < a.step_end; ++step) {
    const float b = (float)a.beta[step / a.spb];
    if ((step & 1) == 0 || step == a.step_begin)
      r = philox4x32_10((uint32_t)(step >> 1), 0u, tg, c3, a.seed_lo, a.seed_hi);
    const bool second = step & 1;
    const uint32_t wk = second ? r.z : r.x;
    const uint32_t wu = second ? r.w : r.y;
    const int k = (int)__umulhi(wk, (uint32_t)a.n);
    const float theta = threshold(u01_open(wu), b, a.acceptance);
    const int slot = k >> 5, owner = k & 31;
    float hv = 0.f;
#pragma unroll
    for (int s = 0; s < SLOTS; ++s)
      if (s == slot) hv = h[s];
    const bool xs = (xl >> slot) & 1ull;
    const float loc = a.diag[k] + hv;
    const float dEl = xs ? -loc : loc;
    const float dE = __shfl_sync(FULL, dEl, owner);
    const bool xk = __shfl_sync(FULL, xs, owner);
    if (dE < theta) {
      const float sgn = xk ? -1.f : 1.f;
      const float *row = a.c + (size_t)k * a.ld + lane;
#pragma unroll
      for (int s2 = 0; s2 < SLOTS; ++s2)
        if (s2 < nslots) h[s2] = fmaf(sgn, __ldg(row + s2 * 32), h[s2]);
      if (lane == owner) xl ^= 1ull << slot;
      E += dE;
      ++acc;
      if (E < Eb) {
        Eb = E;
        xb = xl;
      }
    }
  }
#pragma unroll
  for (int s = 0; s < SLOTS; ++s)
    if (s < nslots) hp[s * 32] = h[s];
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

template <int SLOTS>
__global__ void __launch_bounds__(256) sa_dense_tile_kernel(const __grid_constant__ DenseArgs a) {
  extern __shared__ __align__(128) unsigned char tile_smem[];
  __shared__ __align__(8) uint64_t bar[2];
  float *tiles = reinterpret_cast<float *>(tile_smem);
  const int lane = threadIdx.x & 31;
  const int W = blockDim.x >> 5;
  const int t = blockIdx.x * W + (threadIdx.x >> 5);
  const bool active = t < a.traj_count;
  const int nslots = a.nslots, ld = a.ld;
  const size_t tile_floats = (size_t)TILE_ROWS * ld;
  const uint32_t tile_bytes = (uint32_t)(tile_floats * sizeof(float));
  const int halves = 2 * nslots;
  const long long total = (long long)(a.step_end - a.step_begin) * halves;

  float h[SLOTS];
  unsigned long long xl = 0, xb = 0;
  float E = 0.f, Eb = 0.f;
  float *hp = a.h + (size_t)t * nslots * 32 + lane;
  if (active) {
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) h[s] = s < nslots ? hp[s * 32] : 0.f;
    xl = a.x[(size_t)t * 32 + lane];
    xb = a.xbest[(size_t)t * 32 + lane];
    E = a.e[t];
    Eb = a.ebest[t];
  } else {
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) h[s] = 0.f;
  }
  unsigned long long acc = 0;
  const uint32_t tg = (uint32_t)(a.traj_offset + t);
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSweep;

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
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
  uint32_t parity[2] = {0u, 0u};
  long long g = 0;
  bool failed = false;
  for (int step = a.step_begin; step < a.step_end && !failed; ++step) {
    const float b = (float)a.beta[step / a.spb];
    Philox4 r{0, 0, 0, 0};
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      if (s >= nslots || failed) break;
      if ((s & 3) == 0)
        r = philox4x32_10((uint32_t)((s >> 2) * 32 + lane), (uint32_t)step, tg, c3, a.seed_lo, a.seed_hi);
      const float theta = threshold(select4(r, s & 3), b, a.acceptance);
      const int site = s * 32 + lane;
      const bool valid = site < a.n;
      const float d = a.diag[site];
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const bool ok = mbar_wait_bounded(&bar[half], parity[half], TILE_WAIT_LIMIT);
        parity[half] ^= 1u;
        if (active && ok) {
          const float *tile = tiles + (size_t)half * tile_floats;
          int p = half * TILE_ROWS;
          const int pend = p + TILE_ROWS;
          for (;;) {
            const bool xs = (xl >> s) & 1ull;
            const float loc = d + h[s];
            const float dE = xs ? -loc : loc;
            const unsigned mask = __ballot_sync(FULL, valid && lane >= p && lane < pend && dE < theta);
            if (!mask) break;
            const int i = __ffs(mask) - 1;
            const float dEi = __shfl_sync(FULL, dE, i);
            const bool xi = __shfl_sync(FULL, xs, i);
            const float sgn = xi ? -1.f : 1.f;
            const float *row = tile + (size_t)(i - half * TILE_ROWS) * ld + lane;
#pragma unroll
            for (int s2 = 0; s2 < SLOTS; ++s2)
              if (s2 < nslots) h[s2] = fmaf(sgn, row[s2 * 32], h[s2]);
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
          failed = true;
          break;
        }
        if (threadIdx.x == 0 && g + 2 < total) issue(g + 2);
        ++g;
      }
    }
  }
  if (failed) {
    // Let copies still in flight land (bounded) before the CTA's shared
    // memory is released, and report the timeout.
    if (threadIdx.x == 0) {
      for (int b2 = 0; b2 < 2; ++b2) mbar_wait_bounded(&bar[b2], parity[b2], TILE_WAIT_LIMIT);
      if (a.status) atomicExch(a.status, 1);
    }
    return;
  }
  if (active) {
#pragma unroll
    for (int s = 0; s < SLOTS; ++s)
      if (s < nslots) hp[s * 32] = h[s];
    a.x[(size_t)t * 32 + lane] = xl;
    a.xbest[(size_t)t * 32 + lane] = xb;
    if (lane == 0) {
      a.e[t] = E;
      a.ebest[t] = Eb;
      a.accepted[t] += acc;
    }
  }
}

struct ResyncArgs {
  const double *c64;       // ld x ld FP64 couplings (zero diagonal)
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
};

// FP64 field resync (and initialisation): h_j = sum_{i set, i != j} Q_ij in
// FP64 from the current spins, the drift of the FP32 fields against it, and
// the FP64 energy E = sum_{i set} (Q_ii + h_i / 2).
template <int SLOTS>
__global__ void __launch_bounds__(128) sa_dense_resync_kernel(const __grid_constant__ ResyncArgs a) {
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= a.traj_count) return;
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
      const int site = s * 32 + lane;
      if (site >= a.n) continue;
      const uint32_t w = (s & 3) == 0 ? r.x : (s & 3) == 1 ? r.y : (s & 3) == 2 ? r.z : r.w;
      bool bit = a.init_prob ? (u01_open(w) < a.init_prob[site]) : (w >> 31) != 0;
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
      const double *row = a.c64 + (size_t)(s * 32 + i) * a.ld + lane;
#pragma unroll
      for (int s2 = 0; s2 < SLOTS; ++s2)
        if (s2 < nslots) h64[s2] += row[s2 * 32];
    }
  }
  double epart = 0.0, drift = 0.0;
  float *hp = a.h + (size_t)t * nslots * 32 + lane;
#pragma unroll
  for (int s = 0; s < SLOTS; ++s) {
    if (s >= nslots) break;
    const int site = s * 32 + lane;
    if (site < a.n) {
      if (!a.init) drift = fmax(drift, fabs((double)hp[s * 32] - h64[s]));
      if ((xl >> s) & 1ull) epart += a.d64[site] + 0.5 * h64[s];
    }
    hp[s * 32] = (float)h64[s];
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

// Best states as one byte per variable, for the FP64 re-score.
__global__ void unpack_states_kernel(const unsigned long long *__restrict__ xbest, int n,
                                     int traj_count, uint8_t *__restrict__ out) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)traj_count * n) return;
  const int t = (int)(idx / n), site = (int)(idx % n);
  out[idx] = (uint8_t)((xbest[(size_t)t * 32 + (site & 31)] >> (site >> 5)) & 1ull);
}

}  // namespace sa
}  // namespace os

#endif  // ONESOLVER_SA_KERNELS_CUH_
