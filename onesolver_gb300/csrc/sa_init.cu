// sa_init.cu -- initial spins and local fields of the dense annealing plans
// on the tensor cores.
//
// The reference starts every trajectory from fair coins
// (include/simulated_annealing/annealing.hpp:91-93) and evaluates energies
// from scratch; here each trajectory needs its FP32 local fields
// h_j = sum_{i != j} Q_ij x_i before the first sweep. For all trajectories at
// once that is one product H = X C (T x n by n x n) with X in {0, 1}: it runs
// on the 5th-generation tensor cores (tcgen05.mma kind::f16, BF16 operands,
// FP32 accumulator in tensor memory). The FP32 couplings are split into three
// BF16 terms, c = c_hi + c_mid + c_lo exactly (8 + 8 + 8 significand bits),
// and K runs over the three terms, so every product is exact and only the
// FP32 accumulation rounds: the fields agree with an FP32 sum of the
// couplings, as the sweeps keep them. The periodic resyncs (FP64,
// sa_dense_resync_kernel) measure the drift against FP64 fields as before.
//
// CTA tile: 128 trajectories x 128 sites, accumulator in 128 TMEM columns.
// K advances in chunks of 64: the 4 warps stage the chunk's rows of X and of
// the split couplings (both K-major) into one of two shared-memory buffers
// as 8 x 16-byte core matrices, one elected thread issues four K = 16 MMAs
// and commits them to the buffer's mbarrier, which frees the buffer for the
// chunk after next. The epilogue reads the accumulator with tcgen05.ld (warp
// w: trajectories 32 w .. 32 w + 31) and writes the fields straight into the
// sweep kernels' register layout.
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
#include "tc05.cuh"

namespace os {
namespace sa {

namespace {

constexpr int IM = 128, IN = 128, IK = 64;  // CTA tile of the product, K chunk
constexpr int INIT_CHUNK = 8192;            // trajectories per product (bounds X)
constexpr uint32_t INIT_WAIT_LIMIT = 1u << 26;
constexpr int INIT_SMEM = 2 * (IM + IN) * IK * 2;  // two stages of A and B chunks (64 KB)

// Split couplings, K-major for the product: row j (site) holds
// [c_hi(C_j), c_mid(C_j), c_lo(C_j)] (3 ld wide); C is symmetric, so row j of
// C is also its column j.
__global__ void split_kernel(const double *__restrict__ c64, int ld, __nv_bfloat16 *__restrict__ b) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nn = (size_t)ld * ld;
  if (idx >= nn) return;
  const size_t j = idx / ld, i = idx % ld;
  const float v = (float)c64[idx];
  const __nv_bfloat16 hi = __float2bfloat16(v);
  const float r1 = v - __bfloat162float(hi);
  const __nv_bfloat16 mid = __float2bfloat16(r1);
  const float r2 = r1 - __bfloat162float(mid);
  __nv_bfloat16 *row = b + j * 3 * ld;
  row[i] = hi;
  row[ld + i] = mid;
  row[2 * ld + i] = __float2bfloat16(r2);
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
      if (a.init_bits) bit = a.init_bits[(size_t)t * a.n + site] != 0;
    }
    if (bit) xl |= 1ull << s;
    row[site] = bit ? one : zero;
  }
  a.x[(size_t)t * 32 + lane] = xl;
  a.xbest[(size_t)t * 32 + lane] = xl;
}

// H = X [c_hi | c_mid | c_lo]^T for trajectories [t0, t0 + count): CTA
// (x, y) covers trajectories t0 + 128 x .. + 127 and sites 128 y .. + 127.
// X: xrows x ld (rows past count are zero), Bt: ld x 3 ld. On a bounded wait
// running out the CTA stops, frees its TMEM and sets *status.
__global__ void __launch_bounds__(128) init_gemm_kernel(const __nv_bfloat16 *__restrict__ X,
                                                        const __nv_bfloat16 *__restrict__ Bt, int ld, int nslots,
                                                        int t0, int count, float *__restrict__ h,
                                                        int *__restrict__ status) {
  extern __shared__ __align__(1024) unsigned char init_smem[];  // INIT_SMEM bytes
  // stage b: A chunk at b * 16 KB, B chunk at 32 KB + b * 16 KB
  auto sA = [&](int b) { return init_smem + b * (IM * IK * 2); };
  auto sB = [&](int b) { return init_smem + 2 * (IM * IK * 2) + b * (IN * IK * 2); };
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * IM, col0 = blockIdx.y * IN;
  if (warp == 0) {
    tc05::tmem_alloc(&tmem_base, IN);
    tc05::tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tmem = tmem_base;
  constexpr uint32_t idesc = tc05::idesc_bf16_f32(IM, IN);
  const int K = 3 * ld, nchunks = K / IK;
  bool bad = false;
  for (int c = 0; c < nchunks; ++c) {
    const int b = c & 1;
    if (c >= 2) {  // the MMAs of chunk c - 2 have released buffer b
      const bool ok = mbar_wait_bounded(&bar[b], (uint32_t)(((c - 2) >> 1) & 1), INIT_WAIT_LIMIT);
      if (__syncthreads_or(!ok)) {
        bad = true;
        break;
      }
    }
    const int k0 = c * IK, kx = k0 % ld;
    for (int p = tid; p < IM * (IK / 8); p += 128) {
      const int r = p >> 3, kg = p & 7;
      *reinterpret_cast<uint4 *>(sA(b) + tc05::core_offset(r, kg)) =
          *reinterpret_cast<const uint4 *>(X + (size_t)(row0 + r) * ld + kx + kg * 8);
      *reinterpret_cast<uint4 *>(sB(b) + tc05::core_offset(r, kg)) =
          *reinterpret_cast<const uint4 *>(Bt + (size_t)(col0 + r) * K + k0 + kg * 8);
    }
    tc05::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc05::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < IK / 16; ++kk) {
        const uint64_t ad = tc05::smem_desc(smem_u32(sA(b)) + kk * 256, 128, 1024);
        const uint64_t bd = tc05::smem_desc(smem_u32(sB(b)) + kk * 256, 128, 1024);
        tc05::mma_bf16(tmem, ad, bd, idesc, (c > 0 || kk > 0) ? 1u : 0u);
      }
      tc05::commit(&bar[b]);
    }
  }
  if (!bad) {  // the last commit covers every MMA issued before it
    const int c = nchunks - 1;
    const bool ok = mbar_wait_bounded(&bar[c & 1], (uint32_t)((c >> 1) & 1), INIT_WAIT_LIMIT);
    bad = __syncthreads_or(!ok);
  }
  tc05::fence_after_sync();
  if (!bad) {
    const int r = 32 * warp + lane;  // accumulator row = TMEM lane
    const int t = row0 + r;
#pragma unroll 1
    for (int c4 = 0; c4 < IN / 32; ++c4) {
      uint32_t v[32];
      tc05::ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(c4 * 32), v);
      tc05::wait_ld();
      if (t < count) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int site = col0 + c4 * 32 + j;
          const int s = site_slot(site), l = site_lane(site);
          const size_t pair = ((size_t)(t0 + t) * (nslots / 2) + (s >> 1)) * 32 + l;
          h[2 * pair + (s & 1)] = __uint_as_float(v[j]);
        }
      }
    }
  } else if (tid == 0 && status) {
    atomicExch(status, 1);
  }
  tc05::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc05::fence_after_sync();
    tc05::tmem_dealloc(tmem, IN);
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
  OS_CUDA(cudaFuncSetAttribute(init_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, INIT_SMEM));
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
    init_gemm_kernel<<<grid, 128, INIT_SMEM, s>>>(p->xmat.get(), p->bsplit.get(), p->ld, p->nslots, t0, count,
                                                  a.h, p->status.get());
    OS_CUDA(cudaGetLastError());
    init_energy_kernel<<<(count + 3) / 4, 128, 0, s>>>(a, t0, count);
    OS_CUDA(cudaGetLastError());
    launches += 3;
  }
  return launches;
}

}  // namespace sa
}  // namespace os
