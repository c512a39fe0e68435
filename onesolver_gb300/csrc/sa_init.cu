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
// Output tile: 128 trajectories x 128 sites, its K range (3 ld) split over
// a cluster of 4 CTAs, one per K quarter, each with its own 128 x 128 FP32
// accumulator in 128 TMEM columns. K advances in chunks of 64 through a
// 6-stage ring: one thread issues the chunk's two TMA tensor copies (the
// rows of X and of the split couplings, K-major, 128-byte swizzle) on the
// stage's `full` mbarrier, another issues four K = 16 MMAs once they have
// landed and commits them to the stage's `empty` mbarrier, which lets the
// copy thread refill it. When every CTA's MMAs are done (cluster barrier),
// CTA r gathers column group r (32 sites) of the tile: the other three send
// their partials of it into its shared memory (distributed shared memory),
// and it adds the four in rank order, so the sums do not depend on timing,
// and writes the fields straight into the sweep kernels' register layout.
//
// The initial spins are the same Philox draws as the FP64 initialisation
// (stream kStreamInit, one call per group of four slots and lane), so a
// seed starts from the same states on either path.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

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

constexpr int IM = 128, IN = 128, IK = 64;  // output tile of the product, K chunk
constexpr int INIT_CHUNK = 8192;            // trajectories per product (bounds X)
constexpr uint32_t INIT_WAIT_LIMIT = 1u << 26;
constexpr int INIT_STAGES = 6, INIT_SPLIT = 4;          // ring depth; CTAs (K quarters) per tile
constexpr int INIT_STAGE_BYTES = (IM + IN) * IK * 2;    // A and B chunks of one stage (32 KB)
constexpr int INIT_RECV_STRIDE = 36;  // floats per received partial row (32 + 4: conflict-free 16-byte stores)
constexpr int INIT_SMEM = INIT_STAGES * INIT_STAGE_BYTES + 1024;  // + room to align the ring to 1024 bytes
static_assert((INIT_SPLIT - 1) * IM * INIT_RECV_STRIDE * 4 <= INIT_STAGES * INIT_STAGE_BYTES,
              "the received partials reuse the ring");

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

// H = X [c_hi | c_mid | c_lo]^T for trajectories [t0, t0 + count): the
// cluster at (x, y) covers trajectories t0 + 128 x .. + 127 and sites
// 128 y .. + 127, CTA z of it K chunks [z nch / 4, (z + 1) nch / 4) of the
// nch = 3 ld / 64. tmx: X (xrows x ld), tmb: Bt (ld x 3 ld), boxes of
// 64 x 128 with the 128-byte swizzle. On a bounded wait running out the
// CTA still takes part in both cluster barriers, skips its writes, frees its
// TMEM and sets *status.
__global__ void __cluster_dims__(1, 1, INIT_SPLIT) __launch_bounds__(128, 1)
    init_gemm_kernel(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmb, int ld,
                     int nslots, int t0, int count, float *__restrict__ h, int *__restrict__ status) {
  extern __shared__ unsigned char init_raw[];  // INIT_SMEM bytes
  unsigned char *ring =
      init_raw + ((1024u - (smem_u32(init_raw) & 1023u)) & 1023u);  // TMA 128-byte swizzle: 1024-byte aligned
  auto sA = [&](int s) { return ring + s * INIT_STAGE_BYTES; };
  auto sB = [&](int s) { return ring + s * INIT_STAGE_BYTES + IM * IK * 2; };
  __shared__ __align__(8) uint64_t full[INIT_STAGES], empty[INIT_STAGES], done;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rank = (int)tc05::cluster_ctarank();
  const int row0 = blockIdx.x * IM, col0 = blockIdx.y * IN;
  const int nch = 3 * ld / IK, c_begin = rank * nch / INIT_SPLIT, c_end = (rank + 1) * nch / INIT_SPLIT;
  if (warp == 0) {
    tc05::tmem_alloc(&tmem_base, IN);
    tc05::tmem_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < INIT_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    mbar_fence_init();
  }
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tmem = tmem_base;
  constexpr uint32_t idesc = tc05::idesc_bf16_f32(IM, IN);
  bool bad = false;
  if (warp == 0 && lane == 0) {  // copies
    int issued = 0;
    for (int c = c_begin; c < c_end; ++c) {
      const int i = c - c_begin, s = i % INIT_STAGES, u = i / INIT_STAGES;
      if (u > 0 && !mbar_wait_bounded(&empty[s], (uint32_t)((u - 1) & 1), INIT_WAIT_LIMIT)) {
        bad = true;
        break;
      }
      mbar_arrive_expect_tx(&full[s], INIT_STAGE_BYTES);
      const int k0 = c * IK;
      tma_load_2d(sA(s), &tmx, k0 % ld, row0, &full[s]);
      tma_load_2d(sB(s), &tmb, k0, col0, &full[s]);
      issued = i + 1;
    }
    // Let the copies land (bounded) before the CTA goes on to reuse the ring
    // or exit: after a failure the MMA thread may have stopped consuming
    // them. A stage is reloaded only after the MMAs released its previous
    // copy, so only its last copy can be pending.
    for (int s = 0; s < INIT_STAGES && s < issued; ++s) {
      const int last = s + ((issued - 1 - s) / INIT_STAGES) * INIT_STAGES;
      if (!mbar_wait_bounded(&full[s], (uint32_t)((last / INIT_STAGES) & 1), INIT_WAIT_LIMIT)) bad = true;
    }
  } else if (warp == 1 && lane == 0) {  // MMAs
    for (int c = c_begin; c < c_end; ++c) {
      const int i = c - c_begin, s = i % INIT_STAGES, u = i / INIT_STAGES;
      if (!mbar_wait_bounded(&full[s], (uint32_t)(u & 1), INIT_WAIT_LIMIT)) {
        bad = true;
        break;
      }
      tc05::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < IK / 16; ++kk) {
        const uint64_t ad = tc05::smem_desc_sw128(smem_u32(sA(s)) + kk * 32);
        const uint64_t bd = tc05::smem_desc_sw128(smem_u32(sB(s)) + kk * 32);
        tc05::mma_bf16(tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
      }
      tc05::commit(&empty[s]);
    }
    tc05::commit(&done);  // arrives once every MMA issued above has completed
  }
  if (!mbar_wait_bounded(&done, 0u, INIT_WAIT_LIMIT)) bad = true;
  bad = __syncthreads_or(bad);
  tc05::fence_after_sync();
  // Every CTA's MMAs are complete: its ring may receive partials.
  tc05::cluster_sync();
  const int r = 32 * warp + lane;  // accumulator row = TMEM lane
  uint32_t own[32];
#pragma unroll 1
  for (int g = 0; g < INIT_SPLIT; ++g) {
    uint32_t v[32];
    tc05::ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(g * 32), v);
    tc05::wait_ld();
    if (g == rank) {
#pragma unroll
      for (int j = 0; j < 32; ++j) own[j] = v[j];
    } else {
      const int slot = rank < g ? rank : rank - 1;
      const uint32_t dst =
          tc05::mapa(smem_u32(ring) + (uint32_t)((slot * IM + r) * INIT_RECV_STRIDE * 4), (uint32_t)g);
#pragma unroll
      for (int q = 0; q < 8; ++q) tc05::st_cluster_v4(dst + q * 16, v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
  }
  // Every partial has been delivered.
  tc05::cluster_sync();
  const int t = row0 + r;
  if (!bad && t < count) {
    const float *recv = reinterpret_cast<const float *>(ring);
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      float acc = 0.f;
#pragma unroll
      for (int src = 0; src < INIT_SPLIT; ++src) {
        const float p = src == rank ? __uint_as_float(own[j])
                                    : recv[((src < rank ? src : src - 1) * IM + r) * INIT_RECV_STRIDE + j];
        acc = src == 0 ? p : acc + p;
      }
      const int site = col0 + 32 * rank + j;
      const int s = site_slot(site), l = site_lane(site);
      const size_t pair = ((size_t)(t0 + t) * (nslots / 2) + (s >> 1)) * 32 + l;
      h[2 * pair + (s & 1)] = acc;
    }
  }
  if (bad && tid == 0 && status) atomicExch(status, 1);
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

// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point
// query (no link against the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    OS_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q));
    OS_REQUIRE(q == cudaDriverEntryPointSuccess && f != nullptr, "cuTensorMapEncodeTiled is not available");
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }
  return fn;
}

// Tensor map of a row-major BF16 matrix (rows x cols, 16-byte aligned rows)
// read in boxes of 64 columns x 128 rows with the 128-byte swizzle.
static void encode_bf16_map(void *out, const __nv_bfloat16 *base, uint64_t rows, uint64_t cols) {
  CUtensorMap m;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {cols * sizeof(__nv_bfloat16)};
  const cuuint32_t box[2] = {(cuuint32_t)IK, (cuuint32_t)IM};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(base),
                                          dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  OS_REQUIRE(r == CUDA_SUCCESS, "tensor map encoding failed (%d)", (int)r);
  std::memcpy(out, &m, sizeof m);
}

void dense_init_prepare(os_sa_plan *p, cudaStream_t s) {
  static_assert(sizeof(CUtensorMap) == sizeof(p->init_tmap[0]), "tensor map size");
  OS_CUDA(cudaFuncSetAttribute(init_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, INIT_SMEM));
  const size_t nn = (size_t)p->ld * p->ld;
  p->bsplit.alloc_on(3 * nn, p->ctx->pool, s);
  split_kernel<<<(unsigned)ceil_div_u64(nn, 256), 256, 0, s>>>(p->c64.get(), p->ld, p->bsplit.get());
  OS_CUDA(cudaGetLastError());
  const int rows = std::min(p->T, INIT_CHUNK);
  const size_t xrows = (size_t)(rows + IM - 1) / IM * IM;
  p->xmat.alloc_on(xrows * p->ld, p->ctx->pool, s);
  encode_bf16_map(p->init_tmap[0], p->xmat.get(), xrows, (uint64_t)p->ld);
  encode_bf16_map(p->init_tmap[1], p->bsplit.get(), (uint64_t)p->ld, 3 * (uint64_t)p->ld);
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
    dim3 grid((unsigned)((count + IM - 1) / IM), (unsigned)(p->ld / IN), INIT_SPLIT);
    init_gemm_kernel<<<grid, 128, INIT_SMEM, s>>>(*reinterpret_cast<const CUtensorMap *>(p->init_tmap[0]),
                                                  *reinterpret_cast<const CUtensorMap *>(p->init_tmap[1]), p->ld,
                                                  p->nslots, t0, count, a.h, p->status.get());
    OS_CUDA(cudaGetLastError());
    init_energy_kernel<<<(count + 3) / 4, 128, 0, s>>>(a, t0, count);
    OS_CUDA(cudaGetLastError());
    launches += 3;
  }
  return launches;
}

}  // namespace sa
}  // namespace os
