// sa_init.cu -- initial spins and local fields of the dense annealing plans
// on the tensor cores.
//
// The reference starts every trajectory from fair coins
// (include/simulated_annealing/annealing.hpp:91-93) and evaluates energies
// from scratch; here each trajectory needs its FP32 local fields
// h_j = sum_{i != j} Q_ij x_i before the first sweep. For all trajectories at
// once that is one product H = X C (T x n by n x n) with X in {0, 1}: it runs
// on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation).
// The FP32 couplings are split into three BF16 terms, c = c_hi + c_mid + c_lo
// exactly (8 + 8 + 8 significand bits), and K runs over the three terms, so
// every product is exact and only the FP32 accumulation rounds: the fields
// agree with an FP32 sum of the couplings, as the sweeps keep them. The
// periodic resyncs (FP64, sa_dense_resync_kernel) measure the drift against
// FP64 fields as before.
//
// The initial spins are the same Philox draws as the FP64 initialisation
// (stream kStreamInit, one call per group of four slots and lane), so a
// seed starts from the same states on either path.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "philox.cuh"
#include "sa_common.cuh"
#include "sa_init.cuh"
#include "sa_kernels.cuh"
#include "sa_plan.cuh"

namespace os {
namespace sa {

namespace {

constexpr int IM = 64, IN = 64, IK = 32;  // CTA tile of the product
constexpr int INIT_CHUNK = 8192;          // trajectories per product (bounds X)

__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// B = [c_hi; c_mid; c_lo] (3 ld x ld, row k' = term * ld + site i) from the
// FP64 couplings in site order.
__global__ void split_kernel(const double *__restrict__ c64, int ld, __nv_bfloat16 *__restrict__ b) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nn = (size_t)ld * ld;
  if (idx >= nn) return;
  const float v = (float)c64[idx];
  const __nv_bfloat16 hi = __float2bfloat16(v);
  const float r1 = v - __bfloat162float(hi);
  const __nv_bfloat16 mid = __float2bfloat16(r1);
  const float r2 = r1 - __bfloat162float(mid);
  b[idx] = hi;
  b[nn + idx] = mid;
  b[2 * nn + idx] = __float2bfloat16(r2);
}

// Initial spins of trajectories [t0, t0 + count): lane masks (x, xbest) and
// the 0/1 rows of X (site order, ld wide). A warp per trajectory.
__global__ void init_spins_kernel(const InitArgs a, int t0, int count, __nv_bfloat16 *__restrict__ X) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= count) return;
  const int t = t0 + w;
  const uint32_t tg = (uint32_t)(a.traj_offset + t);
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamInit;
  unsigned long long xl = 0;
  Philox4 r{0, 0, 0, 0};
  __nv_bfloat16 *row = X + (size_t)w * a.ld;
  const __nv_bfloat16 one = __float2bfloat16(1.f), zero = __float2bfloat16(0.f);
  for (int s = 0; s < a.nslots; ++s) {
    if ((s & 3) == 0) r = philox4x32_10((uint32_t)((s >> 2) * 32 + lane), 0u, tg, c3, a.seed_lo, a.seed_hi);
    const int site = slot_site(s, lane);
    bool bit = false;
    if (site < a.n) {
      const uint32_t v = (s & 3) == 0 ? r.x : (s & 3) == 1 ? r.y : (s & 3) == 2 ? r.z : r.w;
      bit = a.init_prob ? (u01_open(v) < a.init_prob[site]) : (v >> 31) != 0;
    }
    if (bit) xl |= 1ull << s;
    row[site] = bit ? one : zero;
  }
  a.x[(size_t)t * 32 + lane] = xl;
  a.xbest[(size_t)t * 32 + lane] = xl;
}

// H = X [c_hi; c_mid; c_lo] for trajectories [t0, t0 + count): CTA tile of
// 64 trajectories x 64 sites, 4 warps of 16 rows, K step 32 over 3 ld. The
// fields go straight into the sweep kernels' layout ([t][nslots/2][32] FP32
// pairs, slot s = site_slot(j) in half s & 1 of pair s >> 1, lane site_lane(j)).
__global__ void __launch_bounds__(128) init_gemm_kernel(const __nv_bfloat16 *__restrict__ X,
                                                        const __nv_bfloat16 *__restrict__ B, int ld, int nslots,
                                                        int t0, int count, float *__restrict__ h) {
  __shared__ __nv_bfloat16 sA[IM][IK + 8];
  __shared__ __nv_bfloat16 sB[IK][IN + 8];
  const int row0 = blockIdx.x * IM, col0 = blockIdx.y * IN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tg = lane & 3;
  float acc[IN / 8][4];
#pragma unroll
  for (int j = 0; j < IN / 8; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
  const int K = 3 * ld;
  for (int k0 = 0; k0 < K; k0 += IK) {
    const int kx = k0 % ld;  // column of X for this K step (the three terms share X)
    for (int i = threadIdx.x; i < IM * IK; i += blockDim.x) {
      const int r = i / IK, c = i % IK;
      sA[r][c] = X[(size_t)(row0 + r) * ld + kx + c];
    }
    for (int i = threadIdx.x; i < IK * IN; i += blockDim.x) {
      const int r = i / IN, c = i % IN;
      sB[r][c] = B[(size_t)(k0 + r) * ld + col0 + c];
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < IK; kk += 16) {
      uint32_t a[4];
      const int ar = warp * 16 + g;
      a[0] = pack(sA[ar][kk + tg * 2], sA[ar][kk + tg * 2 + 1]);
      a[1] = pack(sA[ar + 8][kk + tg * 2], sA[ar + 8][kk + tg * 2 + 1]);
      a[2] = pack(sA[ar][kk + tg * 2 + 8], sA[ar][kk + tg * 2 + 9]);
      a[3] = pack(sA[ar + 8][kk + tg * 2 + 8], sA[ar + 8][kk + tg * 2 + 9]);
#pragma unroll
      for (int j = 0; j < IN / 8; ++j) {
        uint32_t b[2];
        const int bc = j * 8 + g;
        b[0] = pack(sB[kk + tg * 2][bc], sB[kk + tg * 2 + 1][bc]);
        b[1] = pack(sB[kk + tg * 2 + 8][bc], sB[kk + tg * 2 + 9][bc]);
        mma_16816(acc[j], a, b);
      }
    }
    __syncthreads();
  }
  const int rows[2] = {row0 + warp * 16 + g, row0 + warp * 16 + g + 8};
#pragma unroll
  for (int j = 0; j < IN / 8; ++j) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = rows[e >> 1];
      if (r >= count) continue;
      const int site = col0 + j * 8 + tg * 2 + (e & 1);
      const int s = site_slot(site), l = site_lane(site);
      const size_t pair = ((size_t)(t0 + r) * (nslots / 2) + (s >> 1)) * 32 + l;
      h[2 * pair + (s & 1)] = acc[j][e];
    }
  }
}

// Tracked energies E = sum_{i set} (Q_ii + h_i / 2) of trajectories
// [t0, t0 + count) from the new fields, in FP64. A warp per trajectory.
__global__ void init_energy_kernel(const InitArgs a, int t0, int count) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= count) return;
  const int t = t0 + w;
  const unsigned long long xl = a.x[(size_t)t * 32 + lane];
  double e = 0.0;
  for (int s = 0; s < a.nslots; ++s) {
    if (!((xl >> s) & 1ull)) continue;
    const int site = slot_site(s, lane);
    const size_t pair = ((size_t)t * (a.nslots / 2) + (s >> 1)) * 32 + lane;
    e += a.d64[site] + 0.5 * (double)a.h[2 * pair + (s & 1)];
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) e += __shfl_xor_sync(0xffffffffu, e, off);
  if (lane == 0) {
    a.e[t] = (float)e;
    a.ebest[t] = (float)e;
  }
}

}  // namespace

void dense_init_prepare(os_sa_plan *p, cudaStream_t s) {
  const size_t nn = (size_t)p->ld * p->ld;
  p->bsplit.alloc(3 * nn);
  split_kernel<<<(unsigned)ceil_div_u64(nn, 256), 256, 0, s>>>(p->c64.get(), p->ld, p->bsplit.get());
  OS_CUDA(cudaGetLastError());
  const int rows = std::min(p->T, INIT_CHUNK);
  p->xmat.alloc((size_t)(rows + IM - 1) / IM * IM * p->ld);
}

int dense_init_tc(os_sa_plan *p, const InitArgs &a, cudaStream_t s) {
  const int chunk = std::min(p->T, INIT_CHUNK);
  const size_t xrows = (size_t)(chunk + IM - 1) / IM * IM;
  int launches = 0;
  for (int t0 = 0; t0 < p->T; t0 += chunk) {
    const int count = std::min(chunk, p->T - t0);
    OS_CUDA(cudaMemsetAsync(p->xmat.get(), 0, sizeof(__nv_bfloat16) * xrows * p->ld, s));
    init_spins_kernel<<<(count + 3) / 4, 128, 0, s>>>(a, t0, count, p->xmat.get());
    OS_CUDA(cudaGetLastError());
    dim3 grid((unsigned)((count + IM - 1) / IM), (unsigned)(p->ld / IN));
    init_gemm_kernel<<<grid, 128, 0, s>>>(p->xmat.get(), p->bsplit.get(), p->ld, p->nslots, t0, count, a.h);
    OS_CUDA(cudaGetLastError());
    init_energy_kernel<<<(count + 3) / 4, 128, 0, s>>>(a, t0, count);
    OS_CUDA(cudaGetLastError());
    launches += 3;
  }
  return launches;
}

}  // namespace sa
}  // namespace os
