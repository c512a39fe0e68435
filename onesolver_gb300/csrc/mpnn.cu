// mpnn.cu -- the learned warm start: a small message-passing network over the
// coupling matrix that predicts per-spin probabilities P(x_i = 1), trained
// on the GPU by the library's own forward, backward and Adam kernels.
//
// No reference counterpart: the reference always starts trajectories from
// fair coins (include/simulated_annealing/annealing.hpp:91-93). Its output
// feeds os_sa_params.init_prob; plain random-init annealing stays the
// fallback and the yardstick of the energy gap.
//
// Network (H hidden units, L message-passing layers, n spins):
//   C^      = C / (rms(C) sqrt(n))           off-diagonal couplings, BF16
//   X       = [1, d_i / s, r_i / s, [i == 0], u_i] node features: diagonal
//             d_i, row sum r_i of C, scale s = rms(C) sqrt(n); spin 0 is the
//             anchor; u = sqrt(n) v sign(v_0), v the unit vector that power
//             iteration on (sigma I - C / s) reaches (FP32 products, FP64
//             norms; spec_step_kernel):
//             the low end of the coupling spectrum, which the ground states of
//             field-free couplings follow (min over s of s^T C s)
//   H0      = relu(X W_in + b_in)
//   M_l     = C^ H_{l-1}                      (n x n) x (n x H) BF16 tensor cores
//   H_l     = relu(H_{l-1} Ws_l + M_l Wm_l + b_l),   l = 1..L
//   logit   = H_L w_out + b_out,  p = sigmoid(logit)
//   loss    = mean BCE(p_i, y_i)
// A QUBO from a field-free Ising model has the global flip symmetry
// E(x) = E(1 - x) + const; for such instances labels are oriented to agree
// with the spectral feature (sum_i (2 y_i - 1) u_i >= 0; y_0 = 1 on an exact
// tie), and the prediction is in that orientation. General QUBOs keep their
// labels as given.
//
// The (n x n) x (n x H) products run on the 5th-generation tensor cores
// (tcgen05.mma kind::f16, BF16 x BF16 -> FP32 in tensor memory); the small
// (n x H) x (H x H) products, the weight gradients and the element-wise parts
// run on FP32 CUDA cores.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"
#include "philox.cuh"
#include "sa_plan.cuh"
#include "tc05.cuh"

namespace os {
namespace mpnn {

constexpr int FEAT = 5;
constexpr int SPEC_RHO_ITERS = 16;   // power iterations on C^ for its spectral radius
constexpr int SPEC_ITERS = 96;       // power iterations on (sigma I - C^), sigma = 1.05 rho

// ---------------------------------------------------------------------------
// C^ (np x np, BF16, row-major) times Hb (np x 64, BF16), on the
// 5th-generation tensor cores: out (np x 64, FP32, row-major).
//
// Hb is passed transposed (HbT, 64 x np), so both operands are K-major. A CTA
// computes 128 rows x 64 columns over one K range of `ks` (split K: CTA
// (x, y) covers rows [128 x, 128 x + 128) and K [y ks, (y + 1) ks), and writes
// its partial product to out + y * np * 64). K advances in chunks of 64: the
// 4 warps stage the chunk's A (128 x 64) and B (64 x 64) tiles into one of
// two shared-memory buffers as 8-row x 16-byte core matrices (tc05.cuh), one
// elected thread issues four K = 16 tcgen05.mma (kind::f16, BF16 x BF16 ->
// FP32) into a 128 x 64 accumulator in 64 TMEM columns and commits them to
// the buffer's mbarrier, which frees it for the chunk after next. The
// epilogue reads the accumulator with tcgen05.ld (warp w: rows 32 w ..
// 32 w + 31). Rows past np are staged as zeros and not stored. Every wait is
// bounded; on a wait running out the CTA stops, frees its TMEM and sets
// *status.
// ---------------------------------------------------------------------------
constexpr int GN = 64;                                   // hidden width the kernels are built for
constexpr int TM = 128, TK = 64;
constexpr int TC_STAGE_A = TM * TK * 2, TC_STAGE_B = GN * TK * 2;
constexpr int TC_SMEM = 2 * (TC_STAGE_A + TC_STAGE_B);   // 48 KB
constexpr uint32_t TC_WAIT_LIMIT = 1u << 26;

__global__ void __launch_bounds__(128) gemm_ch_kernel(const __nv_bfloat16 *__restrict__ A, int np, int ks,
                                                      const __nv_bfloat16 *__restrict__ BT, float *__restrict__ out,
                                                      int *__restrict__ status) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  auto sA = [&](int b) { return tc_smem + b * TC_STAGE_A; };
  auto sB = [&](int b) { return tc_smem + 2 * TC_STAGE_A + b * TC_STAGE_B; };
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * TM, kb = blockIdx.y * ks;
  out += (size_t)blockIdx.y * np * GN;
  if (warp == 0) {
    tc05::tmem_alloc(&tmem_base, GN);
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
  constexpr uint32_t idesc = tc05::idesc_bf16_f32(TM, GN);
  const int nchunks = ks / TK;
  bool bad = false;
  int committed = 0;  // chunks whose MMAs were issued and committed
  for (int c = 0; c < nchunks; ++c) {
    const int b = c & 1;
    if (c >= 2) {  // the MMAs of chunk c - 2 have released buffer b
      const bool ok = mbar_wait_bounded(&bar[b], (uint32_t)(((c - 2) >> 1) & 1), TC_WAIT_LIMIT);
      if (__syncthreads_or(!ok)) {
        bad = true;
        break;
      }
    }
    const int k0 = kb + c * TK;
    for (int p = tid; p < TM * (TK / 8); p += 128) {
      const int r = p >> 3, kg = p & 7, row = row0 + r;
      const uint4 v = row < np ? *reinterpret_cast<const uint4 *>(A + (size_t)row * np + k0 + kg * 8)
                               : make_uint4(0u, 0u, 0u, 0u);
      *reinterpret_cast<uint4 *>(sA(b) + tc05::core_offset(r, kg)) = v;
    }
    for (int p = tid; p < GN * (TK / 8); p += 128) {
      const int r = p >> 3, kg = p & 7;
      *reinterpret_cast<uint4 *>(sB(b) + tc05::core_offset(r, kg)) =
          *reinterpret_cast<const uint4 *>(BT + (size_t)r * np + k0 + kg * 8);
    }
    tc05::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc05::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk) {
        const uint64_t ad = tc05::smem_desc(smem_u32(sA(b)) + kk * 256, 128, 1024);
        const uint64_t bd = tc05::smem_desc(smem_u32(sB(b)) + kk * 256, 128, 1024);
        tc05::mma_bf16(tmem, ad, bd, idesc, (c > 0 || kk > 0) ? 1u : 0u);
      }
      tc05::commit(&bar[b]);
    }
    committed = c + 1;
  }
  if (!bad) {  // the last commit covers every MMA issued before it
    const int c = nchunks - 1;
    const bool ok = mbar_wait_bounded(&bar[c & 1], (uint32_t)((c >> 1) & 1), TC_WAIT_LIMIT);
    bad = __syncthreads_or(!ok);
  }
  if (bad && tid == 0 && committed > 0) {
    // Let MMAs still in flight finish (bounded) before the accumulator is
    // freed; the last commit covers all of them.
    const int c = committed - 1;
    mbar_wait_bounded(&bar[c & 1], (uint32_t)((c >> 1) & 1), TC_WAIT_LIMIT);
  }
  tc05::fence_after_sync();
  if (!bad) {
    const int row = row0 + 32 * warp + lane;  // accumulator row = TMEM lane
#pragma unroll 1
    for (int c2 = 0; c2 < GN / 32; ++c2) {
      uint32_t v[32];
      tc05::ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(c2 * 32), v);
      tc05::wait_ld();
      if (row < np) {
#pragma unroll
        for (int j = 0; j < 32; ++j) out[(size_t)row * GN + c2 * 32 + j] = __uint_as_float(v[j]);
      }
    }
  } else if (tid == 0 && status) {
    atomicExch(status, 1);
  }
  tc05::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc05::fence_after_sync();
    tc05::tmem_dealloc(tmem, GN);
  }
}

// out[i] = sum over the S partial products, in split order.
__global__ void sum_parts_kernel(const float *__restrict__ part, int S, size_t count, float *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float v = part[i];
  for (int y = 1; y < S; ++y) v += part[(size_t)y * count + i];
  out[i] = v;
}

// ---------------------------------------------------------------------------
// Small FP32 kernels
// ---------------------------------------------------------------------------

// out[n x Hh] = A[n x K] W[K x Hh] (+ B[n x K] W2[K x Hh]) (+ bias), optional relu.
__global__ void linear_kernel(const float *__restrict__ A, const float *__restrict__ W, const float *__restrict__ B,
                              const float *__restrict__ W2, const float *__restrict__ bias, int n, int K, int Hh,
                              int relu, float *__restrict__ pre, float *__restrict__ out) {
  const int i = blockIdx.x;
  const int h = threadIdx.x;
  if (i >= n || h >= Hh) return;
  float acc = bias ? bias[h] : 0.f;
  for (int k = 0; k < K; ++k) acc = fmaf(A[(size_t)i * K + k], W[(size_t)k * Hh + h], acc);
  if (B)
    for (int k = 0; k < K; ++k) acc = fmaf(B[(size_t)i * K + k], W2[(size_t)k * Hh + h], acc);
  if (pre) pre[(size_t)i * Hh + h] = acc;
  out[(size_t)i * Hh + h] = relu ? fmaxf(acc, 0.f) : acc;
}

// in (rows x 64, FP32, row-major) -> out (64 x np, BF16): the transposed,
// K-major operand of gemm_ch_kernel.
__global__ void to_bf16_t_kernel(const float *__restrict__ in, __nv_bfloat16 *__restrict__ out, int rows, int np) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)rows * GN) return;
  const int r = (int)(i / GN), h = (int)(i % GN);
  out[(size_t)h * np + r] = __float2bfloat16(in[i]);
}

// logits, probabilities, loss terms and dlogit for one instance.
__global__ void head_kernel(const float *__restrict__ Hl, const float *__restrict__ w, const float *__restrict__ b,
                            const uint8_t *__restrict__ y, int n, int Hh, float *__restrict__ prob,
                            float *__restrict__ dlogit, float *__restrict__ loss_acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < n) {
    float z = b[0];
    for (int h = 0; h < Hh; ++h) z = fmaf(Hl[(size_t)i * Hh + h], w[h], z);
    const float p = 1.f / (1.f + __expf(-z));
    prob[i] = p;
    if (y) {
      const float t = y[i] ? 1.f : 0.f;
      // BCE with logits, stable form: max(z,0) - z t + log(1 + e^-|z|)
      l = fmaxf(z, 0.f) - z * t + log1pf(__expf(-fabsf(z)));
      dlogit[i] = (p - t) / (float)n;
    }
  }
  if (y && loss_acc) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_acc, l / (float)n);
  }
}

// dW[K x Hh] += A^T dZ (A: n x K, dZ: n x Hh); one thread per (k, h).
__global__ void weight_grad_kernel(const float *__restrict__ A, const float *__restrict__ dZ, int n, int K, int Hh,
                                   float *__restrict__ dW) {
  const int k = blockIdx.x, h = threadIdx.x;
  if (k >= K || h >= Hh) return;
  float acc = 0.f;
  for (int i = 0; i < n; ++i) acc = fmaf(A[(size_t)i * K + k], dZ[(size_t)i * Hh + h], acc);
  dW[(size_t)k * Hh + h] += acc;
}

__global__ void bias_grad_kernel(const float *__restrict__ dZ, int n, int Hh, float *__restrict__ db) {
  const int h = threadIdx.x;
  if (h >= Hh) return;
  float acc = 0.f;
  for (int i = 0; i < n; ++i) acc += dZ[(size_t)i * Hh + h];
  db[h] += acc;
}

// dZ = dH * (pre > 0)
__global__ void relu_back_kernel(const float *__restrict__ dH, const float *__restrict__ pre, size_t count,
                                 float *__restrict__ dZ) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dZ[i] = pre[i] > 0.f ? dH[i] : 0.f;
}

// out[n x K] = dZ[n x Hh] W^T (W: K x Hh)  (+= when accumulate)
__global__ void linear_back_kernel(const float *__restrict__ dZ, const float *__restrict__ W, int n, int K, int Hh,
                                   int accumulate, float *__restrict__ out) {
  const int i = blockIdx.x, k = threadIdx.x;
  if (i >= n || k >= K) return;
  float acc = 0.f;
  for (int h = 0; h < Hh; ++h) acc = fmaf(dZ[(size_t)i * Hh + h], W[(size_t)k * Hh + h], acc);
  out[(size_t)i * K + k] = accumulate ? out[(size_t)i * K + k] + acc : acc;
}

// dH_last = dlogit w_out^T ; dw_out += H^T dlogit ; db_out += sum dlogit
__global__ void head_back_kernel(const float *__restrict__ Hl, const float *__restrict__ dlogit,
                                 const float *__restrict__ w, int n, int Hh, float *__restrict__ dH,
                                 float *__restrict__ dw, float *__restrict__ db) {
  const int h = threadIdx.x;
  if (blockIdx.x == 0 && h < Hh) {
    float acc = 0.f;
    for (int i = 0; i < n; ++i) acc = fmaf(Hl[(size_t)i * Hh + h], dlogit[i], acc);
    dw[h] += acc;
  }
  if (blockIdx.x == 0 && h == 0) {
    float s = 0.f;
    for (int i = 0; i < n; ++i) s += dlogit[i];
    db[0] += s;
  }
  for (int i = blockIdx.x; i < n; i += gridDim.x)
    if (h < Hh) dH[(size_t)i * Hh + h] = dlogit[i] * w[h];
}

__global__ void add_kernel(float *__restrict__ a, const float *__restrict__ b, size_t count) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) a[i] += b[i];
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, size_t count, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace mpnn
}  // namespace os

using namespace os;
using namespace os::mpnn;

// One step of the power-iteration chain, a warp per row, on the FP32 copy of
// C^ (rows of `ld` floats, ld a multiple of 128, zero beyond n; v likewise
// zero beyond n): out = C v^ (mode 0) or sigma v^ - C v^ (mode 1,
// sigma = 1.05 sqrt(*rho2)), v^ = v / sqrt(*norm_in). Products accumulate in
// FP32, the scaling and the squared norm of out in FP64; one atomic per CTA
// adds the CTA's share of that norm into *norm_out. With `x` (the first
// step) the step also stores the row sum of C^ as node feature 2. FP64
// arithmetic is scarce on this part: the norm's reciprocal square root and
// sigma are formed once per CTA, the FP64 products once per row.
//
// The steps are chained by programmatic dependent launch: a step may start
// while its predecessor runs, loads its row of the matrix (which no step
// writes) into registers, and only then waits for the predecessor's results
// (griddepcontrol.wait); it releases its own successor after that wait, so a
// step's early part never overlaps a step older than its predecessor. The
// vector is read through L2 (ld.global.cg) into shared memory once per CTA.
constexpr int SPEC_WARPS = 4;
constexpr int SPEC_PRE = 8;  // float4 of the row per lane loaded before the wait (rows up to 1024)
__global__ void __launch_bounds__(SPEC_WARPS * 32) spec_step_kernel(const float *__restrict__ c, int n, int ld,
                                                                    const float *v, const double *norm_in,
                                                                    const double *rho2, int mode, float *out,
                                                                    double *norm_out, float *x) {
  extern __shared__ float4 vs[];  // ld / 4
  __shared__ double part[SPEC_WARPS], sc[2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * SPEC_WARPS + warp;
  const int q = ld >> 2;
  const float4 *cr = reinterpret_cast<const float4 *>(c + (size_t)(row < n ? row : 0) * ld);
  float4 pre[SPEC_PRE];
#pragma unroll
  for (int t = 0; t < SPEC_PRE; ++t) {
    const int j = lane + 32 * t;
    pre[t] = row < n && j < q ? __ldg(cr + j) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (threadIdx.x == 0) {
    const double nin = __ldcg(norm_in);
    sc[0] = nin > 0.0 ? 1.0 / sqrt(nin) : 0.0;
    sc[1] = mode ? 1.05 * sqrt(__ldcg(rho2)) : 0.0;
  }
  const float4 *v4 = reinterpret_cast<const float4 *>(v);
  for (int j = threadIdx.x; j < q; j += blockDim.x) vs[j] = __ldcg(v4 + j);
  __syncthreads();
  double y = 0.0;
  if (row < n) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int t = 0; t < SPEC_PRE; ++t) {
      const int j = lane + 32 * t;
      if (j < q) {
        const float4 vv = vs[j];
        a0 = fmaf(pre[t].x, vv.x, a0);
        a1 = fmaf(pre[t].y, vv.y, a1);
        a2 = fmaf(pre[t].z, vv.z, a2);
        a3 = fmaf(pre[t].w, vv.w, a3);
      }
    }
#pragma unroll 4
    for (int j = lane + 32 * SPEC_PRE; j < q; j += 32) {
      const float4 cv = __ldg(cr + j), vv = vs[j];
      a0 = fmaf(cv.x, vv.x, a0);
      a1 = fmaf(cv.y, vv.y, a1);
      a2 = fmaf(cv.z, vv.z, a2);
      a3 = fmaf(cv.w, vv.w, a3);
    }
    float acc = (a0 + a1) + (a2 + a3);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (x) {
      float ls = 0.f;
#pragma unroll
      for (int t = 0; t < SPEC_PRE; ++t) ls += (pre[t].x + pre[t].y) + (pre[t].z + pre[t].w);
      for (int j = lane + 32 * SPEC_PRE; j < q; j += 32) {
        const float4 cv = __ldg(cr + j);
        ls += (cv.x + cv.y) + (cv.z + cv.w);
      }
      double rsum = ls;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) rsum += __shfl_xor_sync(0xffffffffu, rsum, off);
      if (lane == 0) x[(size_t)row * FEAT + 2] = (float)rsum;
    }
    if (lane == 0) {
      const double vr = reinterpret_cast<const float *>(vs)[row];
      y = mode ? (sc[1] * vr - (double)acc) * sc[0] : (double)acc * sc[0];
      out[row] = (float)y;
    }
  }
  if (lane == 0) part[warp] = y * y;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < SPEC_WARPS; ++w) t += part[w];
    atomicAdd(norm_out, t);
  }
}

// u_i = sqrt(n) v^_i sign(v^_0) into column `col` of the feature matrix.
__global__ void spec_feature_kernel(const float *__restrict__ v, const double *__restrict__ norm, int n,
                                    float *__restrict__ x, int col) {
  __shared__ double fac;  // sqrt(n) sign(v_0) / |v|, formed once per CTA
  if (threadIdx.x == 0) fac = (*norm > 0.0 ? sqrt((double)n / *norm) : 0.0) * (v[0] < 0.f ? -1.0 : 1.0);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[(size_t)i * FEAT + col] = (float)(fac * (double)v[i]);
}

// One stored instance: scaled couplings (BF16, padded to np x np), features,
// optional labels.
struct MpnnInstance {
  int n = 0, np = 0;
  DevBuf<__nv_bfloat16> c;
  DevBuf<float> x;     // n x FEAT
  DevBuf<uint8_t> y;   // n (oriented labels) or empty
};

// Temporaries of staging an instance: the matrix as given, FP32 scaled
// couplings (rows padded to `ld`), power-iteration vectors, their FP64 norms,
// coefficient statistics.
struct StageTmp {
  int ld = 0;
  DevBuf<double> f, norms, stats, part;
  DevBuf<float> c32, v[3];
};

struct os_mpnn {
  os_ctx *ctx = nullptr;
  int H = 64, L = 3;
  bool orient = true;  // labels oriented with y_0 = 1
  // parameter layout (FP32): W_in[FEAT*H], b_in[H], {Ws[H*H], Wm[H*H], b[H]} x L, w_out[H], b_out[1]
  size_t nparam = 0;
  DevBuf<float> param, grad, adam_m, adam_v;
  long long adam_t = 0;
  std::vector<std::unique_ptr<MpnnInstance>> inst;
  // work buffers for n up to cap
  int cap = 0;
  DevBuf<float> X0pre, Hs, pres, M, dH, dZ, dM, prob, dlogit, loss, gpart;
  DevBuf<__nv_bfloat16> Hb;            // the message product's operand, transposed (64 x np)
  DevBuf<int> tc_status;                // set when a tensor-core kernel's bounded wait ran out
  // prediction: persistent buffers and the captured staging + forward graph
  // (valid for pgraph_n spins while the work buffers keep capacity pgraph_cap)
  std::unique_ptr<MpnnInstance> pin;
  StageTmp ptmp;
  cudaGraphExec_t pgraph = nullptr;
  int pgraph_n = 0, pgraph_cap = 0;
  ~os_mpnn() {
    if (pgraph) cudaGraphExecDestroy(pgraph);
  }

  size_t off_win() const { return 0; }
  size_t off_bin() const { return (size_t)FEAT * H; }
  size_t off_layer(int l) const { return off_bin() + H + (size_t)l * (2 * H * H + H); }
  size_t off_wout() const { return off_layer(L); }
  size_t off_bout() const { return off_wout() + H; }
};

namespace {

void ensure_work(os_mpnn *m, int np) {
  if (np <= m->cap) return;
  const size_t nh = (size_t)np * m->H;
  m->X0pre.alloc(nh);
  m->Hs.alloc(nh * (m->L + 1));
  m->pres.alloc(nh * (m->L + 1));
  m->M.alloc(nh * m->L);
  m->dH.alloc(nh);
  m->dZ.alloc(nh);
  m->dM.alloc(nh);
  m->prob.alloc(np);
  m->dlogit.alloc(np);
  m->loss.alloc(1);
  m->Hb.alloc(nh);
  m->gpart.alloc(4 * nh);
  m->tc_status.alloc(1);
  OS_CUDA(cudaMemset(m->tc_status.get(), 0, sizeof(int)));
  OS_CUDA(cudaFuncSetAttribute(gemm_ch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
  m->cap = np;
}

// out (np x 64, FP32) = A (np x np, BF16) B (np x 64, BF16, given transposed
// as BT) on the tensor cores, K split over S CTAs per 128-row block and the S
// partial products summed in order.
void gemm_ch(os_mpnn *m, const __nv_bfloat16 *A, int np, const __nv_bfloat16 *BT, float *out, cudaStream_t s) {
  const int chunks = np / TK;  // np is a multiple of 64
  const int S = chunks % 4 == 0 ? 4 : chunks % 2 == 0 ? 2 : 1;
  gemm_ch_kernel<<<dim3((unsigned)((np + TM - 1) / TM), (unsigned)S), 128, TC_SMEM, s>>>(
      A, np, np / S, BT, m->gpart.get(), m->tc_status.get());
  OS_CUDA(cudaGetLastError());
  const size_t count = (size_t)np * GN;
  sum_parts_kernel<<<(unsigned)ceil_div_u64(count, 256), 256, 0, s>>>(m->gpart.get(), S, count, out);
  OS_CUDA(cudaGetLastError());
}

// OS_TIMEOUT if a tensor-core kernel's bounded wait ran out (after a
// synchronisation of the context's stream); the flag is cleared.
void check_tc_status(os_mpnn *m) {
  int st = 0;
  OS_CUDA(cudaMemcpy(&st, m->tc_status.get(), sizeof st, cudaMemcpyDeviceToHost));
  if (st) {
    OS_CUDA(cudaMemset(m->tc_status.get(), 0, sizeof(int)));
    throw_error(OS_TIMEOUT, "a tensor-core message product's bounded wait ran out");
  }
}

// Forward pass of instance `in` (activations kept for the backward pass).
void forward(os_mpnn *m, MpnnInstance &in, cudaStream_t s) {
  const int n = in.n, np = in.np, H = m->H;
  const size_t nh = (size_t)np * H;
  float *P = m->param.get();
  OS_CUDA(cudaMemsetAsync(m->Hs.get(), 0, sizeof(float) * nh * (m->L + 1), s));
  // H0 = relu(X W_in + b_in)
  linear_kernel<<<n, H, 0, s>>>(in.x.get(), P + m->off_win(), nullptr, nullptr, P + m->off_bin(), n, FEAT, H, 1,
                                m->pres.get(), m->Hs.get());
  for (int l = 0; l < m->L; ++l) {
    const float *Hprev = m->Hs.get() + (size_t)l * nh;
    float *Ml = m->M.get() + (size_t)l * nh;
    to_bf16_t_kernel<<<(unsigned)ceil_div_u64(nh, 256), 256, 0, s>>>(Hprev, m->Hb.get(), np, np);
    gemm_ch(m, in.c.get(), np, m->Hb.get(), Ml, s);
    const float *Wl = P + m->off_layer(l);
    linear_kernel<<<n, H, 0, s>>>(Hprev, Wl, Ml, Wl + (size_t)H * H, Wl + 2 * (size_t)H * H, n, H, H, 1,
                                  m->pres.get() + (size_t)(l + 1) * nh, m->Hs.get() + (size_t)(l + 1) * nh);
  }
  OS_CUDA(cudaGetLastError());
}

// Loss and gradients (accumulated into m->grad) of one instance; the
// forward pass must have run. Element-wise work covers the n real rows; the
// padded rows of the BF16 operands are zero.
void backward(os_mpnn *m, MpnnInstance &in, cudaStream_t s) {
  const int n = in.n, np = in.np, H = m->H;
  const size_t nh = (size_t)np * H, rh = (size_t)n * H;
  const unsigned eb = (unsigned)ceil_div_u64(rh, 256);
  float *P = m->param.get(), *Gd = m->grad.get();
  const float *HL = m->Hs.get() + (size_t)m->L * nh;
  head_kernel<<<(n + 255) / 256, 256, 0, s>>>(HL, P + m->off_wout(), P + m->off_bout(), in.y.get(), n, H,
                                              m->prob.get(), m->dlogit.get(), m->loss.get());
  head_back_kernel<<<64, H, 0, s>>>(HL, m->dlogit.get(), P + m->off_wout(), n, H, m->dH.get(),
                                    Gd + m->off_wout(), Gd + m->off_bout());
  for (int l = m->L - 1; l >= 0; --l) {
    const float *Hprev = m->Hs.get() + (size_t)l * nh;
    const float *pre = m->pres.get() + (size_t)(l + 1) * nh;
    const float *Ml = m->M.get() + (size_t)l * nh;
    const float *Wl = P + m->off_layer(l);
    float *Gl = Gd + m->off_layer(l);
    relu_back_kernel<<<eb, 256, 0, s>>>(m->dH.get(), pre, rh, m->dZ.get());
    weight_grad_kernel<<<H, H, 0, s>>>(Hprev, m->dZ.get(), n, H, H, Gl);               // dWs
    weight_grad_kernel<<<H, H, 0, s>>>(Ml, m->dZ.get(), n, H, H, Gl + (size_t)H * H);  // dWm
    bias_grad_kernel<<<1, H, 0, s>>>(m->dZ.get(), n, H, Gl + 2 * (size_t)H * H);        // db
    // dM = dZ Wm^T ; dH_prev = dZ Ws^T + C^ dM  (C^ is symmetric)
    linear_back_kernel<<<n, H, 0, s>>>(m->dZ.get(), Wl + (size_t)H * H, n, H, H, 0, m->dM.get());
    linear_back_kernel<<<n, H, 0, s>>>(m->dZ.get(), Wl, n, H, H, 0, m->dH.get());
    OS_CUDA(cudaMemsetAsync(m->Hb.get(), 0, sizeof(__nv_bfloat16) * nh, s));
    to_bf16_t_kernel<<<eb, 256, 0, s>>>(m->dM.get(), m->Hb.get(), n, np);
    gemm_ch(m, in.c.get(), np, m->Hb.get(), m->dZ.get(), s);
    add_kernel<<<eb, 256, 0, s>>>(m->dH.get(), m->dZ.get(), rh);
  }
  // Input layer: dZ0 = dH0 * (pre0 > 0); dW_in = X^T dZ0; db_in = sum dZ0.
  relu_back_kernel<<<eb, 256, 0, s>>>(m->dH.get(), m->pres.get(), rh, m->dZ.get());
  weight_grad_kernel<<<FEAT, H, 0, s>>>(in.x.get(), m->dZ.get(), n, FEAT, H, Gd + m->off_win());
  bias_grad_kernel<<<1, H, 0, s>>>(m->dZ.get(), n, H, Gd + m->off_bin());
  OS_CUDA(cudaGetLastError());
}

// Start vector of the power iterations: positive, uneven, deterministic.
__host__ __device__ inline double spec_start(int i) {
  return 1.0 + 0.25 * (double)(((uint32_t)i * 2654435761u) >> 24) / 255.0;
}

// Staging works on 32 x 32 tiles (I, J) of the upper triangle: a 2-D grid of
// T x T CTAs (T = ceil(n / 32), blockIdx.y = I, blockIdx.x = J) in which the
// CTAs below the diagonal return at once. Thread (ty, tx) = (warp, lane)
// takes tile rows ty, ty + 8, ty + 16, ty + 24 at column tx.
constexpr int STAGE_TILE = 32;

// stats[0] = sum of squares of the off-diagonal upper-triangle coefficients,
// stats[1] = count of non-finite coefficients on or above the diagonal. Each
// tile's CTA writes its two partial sums to part[2 (I T + J)]; the last CTA
// to finish (counted in *done, zero at launch) adds them in index order, so
// the result does not depend on the order in which the CTAs ran.
__global__ void __launch_bounds__(256) stage_stats_kernel(const double *__restrict__ f, int n, double *part,
                                                          unsigned *done, double *__restrict__ stats) {
  const int T = gridDim.x, I = blockIdx.y, J = blockIdx.x;
  if (I > J) return;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  __shared__ double rs[8], rb[8];
  __shared__ bool last;
  double ss = 0.0, bad = 0.0;
  const int gj = J * STAGE_TILE + tx;
#pragma unroll
  for (int r = ty; r < STAGE_TILE; r += 8) {
    const int gi = I * STAGE_TILE + r;
    if (gi < n && gj < n && gj >= gi) {
      const double v = f[(size_t)gi * n + gj];
      if (!isfinite(v)) bad += 1.0;
      else if (gj > gi) ss += v * v;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ss += __shfl_xor_sync(0xffffffffu, ss, off);
    bad += __shfl_xor_sync(0xffffffffu, bad, off);
  }
  if (tx == 0) rs[ty] = ss, rb[ty] = bad;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < 8; ++w) a += rs[w], b += rb[w];
    part[2 * ((size_t)I * T + J)] = a;
    part[2 * ((size_t)I * T + J) + 1] = b;
    __threadfence();
    last = atomicAdd(done, 1u) == (unsigned)(T * (T + 1) / 2 - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < T * T; k += blockDim.x)
    if (k / T <= k % T) a += __ldcg(part + 2 * (size_t)k), b += __ldcg(part + 2 * (size_t)k + 1);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, off);
    b += __shfl_xor_sync(0xffffffffu, b, off);
  }
  if (tx == 0) rs[ty] = a, rb[ty] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < 8; ++w) ta += rs[w], tb += rb[w];
    stats[0] = ta;
    stats[1] = tb;
  }
}

// Scaled symmetric couplings C^ = C / s, s = rms * sqrt(n) from stats[0]
// over `pairs` coefficients (1 when they are all zero), from the upper
// triangle of f: BF16 with rows of np and FP32 with rows of ld (both
// zero-filled beforehand; only entries below n are written). Tile (I, J)
// writes block (I, J) and, through a shared-memory transpose, block (J, I).
// The diagonal tiles write the node features that need no row sum (the row
// sums are added by the first power-iteration step) and the start vector of
// the power iterations; CTA (0, 0) stores its squared norm, `start_norm`.
__global__ void __launch_bounds__(256) stage_build_kernel(const double *__restrict__ f, int n, int np, int ld,
                                                          double pairs, const double *__restrict__ stats,
                                                          __nv_bfloat16 *__restrict__ cb, float *__restrict__ c32,
                                                          float *__restrict__ x, float *__restrict__ v0,
                                                          double start_norm, double *__restrict__ norm0) {
  const int I = blockIdx.y, J = blockIdx.x;
  if (I > J) return;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  __shared__ double tile[STAGE_TILE][STAGE_TILE + 1];
  __shared__ double scale_s[2];  // s and 1 / s, formed once per CTA (FP64 is scarce)
  if (threadIdx.x == 0) {
    const double rms = pairs > 0 ? sqrt(stats[0] / pairs) : 0.0;
    scale_s[0] = rms > 0 ? rms * sqrt((double)n) : 1.0;
    scale_s[1] = 1.0 / scale_s[0];
  }
#pragma unroll
  for (int r = ty; r < STAGE_TILE; r += 8) {
    const int gi = I * STAGE_TILE + r, gj = J * STAGE_TILE + tx;
    tile[r][tx] = gi < n && gj < n && gi < gj ? f[(size_t)gi * n + gj] : 0.0;
  }
  __syncthreads();
  const double inv_scale = scale_s[1];
#pragma unroll
  for (int r = ty; r < STAGE_TILE; r += 8) {
    int gi = I * STAGE_TILE + r, gj = J * STAGE_TILE + tx;
    if (gi < n && gj < n) {
      const double v = (I == J && r > tx ? tile[tx][r] : tile[r][tx]) * inv_scale;
      c32[(size_t)gi * ld + gj] = (float)v;
      cb[(size_t)gi * np + gj] = __float2bfloat16((float)v);
    }
    gi = J * STAGE_TILE + r, gj = I * STAGE_TILE + tx;
    if (I < J && gi < n && gj < n) {
      const double v = tile[tx][r] * inv_scale;
      c32[(size_t)gi * ld + gj] = (float)v;
      cb[(size_t)gi * np + gj] = __float2bfloat16((float)v);
    }
  }
  if (I == J && ty == 0) {
    const int i = I * STAGE_TILE + tx;
    if (i < n) {
      float *xi = x + (size_t)i * FEAT;
      xi[0] = 1.f;
      xi[1] = (float)(f[(size_t)i * n + i] / scale_s[0]);
      xi[3] = i == 0 ? 1.f : 0.f;
      xi[4] = 0.f;
      v0[i] = (float)spec_start(i);
    }
    if (I == 0 && tx == 0) *norm0 = start_norm;
  }
}

// Stage an instance on `s`: the QUBO goes up once; scale, BF16 and FP32
// scaled couplings, node features and the spectral feature are computed on
// the device. The spectral feature (column 4): SPEC_RHO_ITERS power
// iterations on C^ estimate its spectral radius rho, then SPEC_ITERS
// iterations on (1.05 rho I - C^) from the same start vector (FP32 products
// from the L2-resident FP32 matrix, FP64 norms), no host round trip. With a label the stream is synchronised,
// the coefficients checked and the label oriented; without one the caller
// checks `tmp.stats[1]` (non-finite count) after its own synchronisation.
// Device buffers of an instance of n spins and of its staging.
void stage_alloc(MpnnInstance &in, StageTmp &tmp, int n) {
  in.n = n;
  in.np = (n + 63) / 64 * 64;
  const size_t nn = (size_t)n * n;
  tmp.ld = (n + 127) / 128 * 128;
  tmp.f.alloc(nn);
  tmp.stats.alloc(3);
  const size_t T = (n + STAGE_TILE - 1) / STAGE_TILE;
  tmp.part.alloc(2 * T * T);
  tmp.norms.alloc(SPEC_RHO_ITERS + SPEC_ITERS + 2);
  in.c.alloc((size_t)in.np * in.np);
  tmp.c32.alloc((size_t)n * tmp.ld);
  in.x.alloc((size_t)n * FEAT);
  for (auto &b : tmp.v) b.alloc(tmp.ld);
}

// Staging kernels on `s` (tmp.f already holds the matrix): no allocation and
// no host synchronisation, so the sequence can be captured into a graph.
void stage_enqueue(MpnnInstance &in, StageTmp &tmp, cudaStream_t s) {
  const int n = in.n;
  const int total = SPEC_RHO_ITERS + SPEC_ITERS + 2;
  OS_CUDA(cudaMemsetAsync(tmp.stats.get(), 0, sizeof(double) * 3, s));  // sums, non-finite count, CTA counter
  OS_CUDA(cudaMemsetAsync(tmp.norms.get(), 0, sizeof(double) * total, s));
  OS_CUDA(cudaMemsetAsync(in.c.get(), 0, sizeof(__nv_bfloat16) * in.c.count, s));
  for (auto &b : tmp.v) OS_CUDA(cudaMemsetAsync(b.get(), 0, sizeof(float) * b.count, s));
  OS_CUDA(cudaMemsetAsync(tmp.c32.get(), 0, sizeof(float) * tmp.c32.count, s));
  const int T = (n + STAGE_TILE - 1) / STAGE_TILE;
  const dim3 tiles(T, T);
  stage_stats_kernel<<<tiles, 256, 0, s>>>(tmp.f.get(), n, tmp.part.get(),
                                           reinterpret_cast<unsigned *>(tmp.stats.get() + 2), tmp.stats.get());
  OS_CUDA(cudaGetLastError());
  double start_norm = 0.0;  // of the start vector as stored (FP32), in index order
  for (int i = 0; i < n; ++i) {
    const double v = (double)(float)spec_start(i);
    start_norm += v * v;
  }
  stage_build_kernel<<<tiles, 256, 0, s>>>(tmp.f.get(), n, in.np, tmp.ld, (double)n * (n - 1) / 2,
                                           tmp.stats.get(), in.c.get(), tmp.c32.get(), in.x.get(), tmp.v[2].get(),
                                           start_norm, tmp.norms.get());
  OS_CUDA(cudaGetLastError());
  // Power iterations, one chain of SPEC_RHO_ITERS + SPEC_ITERS steps. Step k
  // of a phase reads v[k & 1] (v[2], the start vector, for k = 0) and writes
  // v[(k + 1) & 1]. Squared norms: norms[0] is the start vector's; the C^
  // phase writes norms[1 .. R] (R = SPEC_RHO_ITERS, rho^2 = norms[R]); the
  // (sigma I - C^) phase writes norms[R + 1 .. R + SPEC_ITERS], its first
  // step reading norms[0] again.
  const int R = SPEC_RHO_ITERS;
  cudaLaunchAttribute chain;
  chain.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  chain.val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((n + SPEC_WARPS - 1) / SPEC_WARPS);
  cfg.blockDim = dim3(SPEC_WARPS * 32);
  cfg.dynamicSmemBytes = sizeof(float) * tmp.ld;
  cfg.stream = s;
  cfg.attrs = &chain;
  double *norms = tmp.norms.get();
  int last = 0;
  for (int mode = 0; mode < 2; ++mode) {
    const int iters = mode ? SPEC_ITERS : R, slot0 = mode ? R : 0;
    for (int k = 0; k < iters; ++k) {
      const float *vin = k == 0 ? tmp.v[2].get() : tmp.v[k & 1].get();
      const double *nin = k == 0 ? norms : norms + slot0 + k;
      // The first step follows the staging kernels in plain stream order:
      // its matrix loads must see them complete.
      cfg.numAttrs = mode == 0 && k == 0 ? 0 : 1;
      OS_CUDA(cudaLaunchKernelEx(&cfg, spec_step_kernel, (const float *)tmp.c32.get(), n, tmp.ld, vin, nin,
                                 (const double *)(norms + R), mode, tmp.v[(k + 1) & 1].get(),
                                 norms + slot0 + k + 1, mode == 0 && k == 0 ? in.x.get() : (float *)nullptr));
    }
    last = iters & 1;
  }
  spec_feature_kernel<<<(n + 255) / 256, 256, 0, s>>>(tmp.v[last].get(), norms + R + SPEC_ITERS, n, in.x.get(),
                                                      4);
  OS_CUDA(cudaGetLastError());
}

std::unique_ptr<MpnnInstance> stage(const os_qubo_dense *q, const char *label, bool orient, cudaStream_t s,
                                    StageTmp &tmp) {
  const int n = q->n;
  OS_REQUIRE(n >= 2 && n <= 8192, "the network takes 2..8192 spins (got %d)", n);
  auto in = std::make_unique<MpnnInstance>();
  stage_alloc(*in, tmp, n);
  OS_CUDA(cudaMemcpyAsync(tmp.f.get(), q->f, sizeof(double) * (size_t)n * n, cudaMemcpyHostToDevice, s));
  stage_enqueue(*in, tmp, s);
  if (label) {
    std::vector<float> x((size_t)n * FEAT);
    double bad = 0.0;
    OS_CUDA(cudaMemcpyAsync(x.data(), in->x.get(), sizeof(float) * x.size(), cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaMemcpyAsync(&bad, tmp.stats.get() + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
    OS_REQUIRE(bad == 0.0, "the QUBO has non-finite coefficients");
    std::vector<uint8_t> y(n);
    double agree = 0.0;
    for (int i = 0; i < n; ++i) agree += (label[i] ? 1.0 : -1.0) * (double)x[(size_t)i * FEAT + 4];
    const bool flip = orient && (agree != 0.0 ? agree < 0.0 : label[0] == 0);
    for (int i = 0; i < n; ++i) y[i] = (uint8_t)((label[i] != 0) != flip);
    in->y.alloc(n);
    OS_CUDA(cudaMemcpy(in->y.get(), y.data(), n, cudaMemcpyHostToDevice));
  }
  return in;
}

void init_params(os_mpnn *m, unsigned long long seed) {
  std::vector<float> p(m->nparam, 0.f);
  // Scaled uniform initialisation from Philox (fan-in scaling).
  size_t ctr = 0;
  auto fill = [&](size_t off, int rows, int cols) {
    const float a = std::sqrt(6.f / (float)(rows + cols));
    for (int i = 0; i < rows * cols; ++i, ++ctr) {
      Philox4 r = philox4x32_10((uint32_t)ctr, (uint32_t)(ctr >> 32), 0x11u, 0x4D504E4Eu, (uint32_t)seed,
                                (uint32_t)(seed >> 32));
      const float u = ((r.x >> 8) + 0.5f) * 0x1.0p-24f;
      p[off + i] = a * (2.f * u - 1.f);
    }
  };
  fill(m->off_win(), FEAT, m->H);
  for (int l = 0; l < m->L; ++l) {
    fill(m->off_layer(l), m->H, m->H);
    fill(m->off_layer(l) + (size_t)m->H * m->H, m->H, m->H);
  }
  fill(m->off_wout(), m->H, 1);
  OS_CUDA(cudaMemcpy(m->param.get(), p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice));
  OS_CUDA(cudaMemset(m->adam_m.get(), 0, sizeof(float) * m->nparam));
  OS_CUDA(cudaMemset(m->adam_v.get(), 0, sizeof(float) * m->nparam));
  m->adam_t = 0;
}

}  // namespace

extern "C" {

os_status os_mpnn_create(os_ctx *ctx, int32_t hidden, int32_t layers, int32_t orient, uint64_t seed,
                         os_mpnn **out) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(out != nullptr, "null output");
    OS_REQUIRE(hidden == 64, "the message-passing kernels are built for 64 hidden units");
    OS_REQUIRE(layers >= 1 && layers <= 8, "layers must be 1..8");
    auto *m = new os_mpnn();
    try {
      m->ctx = ctx;
      m->H = hidden;
      m->L = layers;
      m->orient = orient != 0;
      m->nparam = m->off_bout() + 1;
      m->param.alloc(m->nparam);
      m->grad.alloc(m->nparam);
      m->adam_m.alloc(m->nparam);
      m->adam_v.alloc(m->nparam);
      init_params(m, seed);
    } catch (...) {
      delete m;
      throw;
    }
    *out = m;
  });
}

void os_mpnn_destroy(os_mpnn *m) {
  if (!m) return;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(m->ctx->stream);
  delete m;
}

int64_t os_mpnn_num_params(const os_mpnn *m) { return m ? (int64_t)m->nparam : -1; }

os_status os_mpnn_get_params(os_mpnn *m, float *out, size_t cap) {
  return guard([&] {
    OS_REQUIRE(m && out && cap >= m->nparam, "buffer holds %zu values, %zu needed", cap, m ? m->nparam : 0);
    activate(m->ctx);
    OS_CUDA(cudaStreamSynchronize(m->ctx->stream));
    OS_CUDA(cudaMemcpy(out, m->param.get(), sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
  });
}

os_status os_mpnn_set_params(os_mpnn *m, const float *in, size_t count) {
  return guard([&] {
    OS_REQUIRE(m && in && count == m->nparam, "expected %zu parameters", m ? m->nparam : 0);
    activate(m->ctx);
    OS_CUDA(cudaStreamSynchronize(m->ctx->stream));
    OS_CUDA(cudaMemcpy(m->param.get(), in, sizeof(float) * count, cudaMemcpyHostToDevice));
  });
}

os_status os_mpnn_add_instance(os_mpnn *m, const os_qubo_dense *q, const char *label, int32_t *index) {
  return guard([&] {
    OS_REQUIRE(m && q && q->f, "null argument");
    activate(m->ctx);
    StageTmp tmp;
    m->inst.push_back(stage(q, label, m->orient, m->ctx->stream, tmp));
    OS_CUDA(cudaStreamSynchronize(m->ctx->stream));
    if (index) *index = (int32_t)m->inst.size() - 1;
  });
}

os_status os_mpnn_clear_instances(os_mpnn *m) {
  return guard([&] {
    OS_REQUIRE(m != nullptr, "null model");
    activate(m->ctx);
    OS_CUDA(cudaStreamSynchronize(m->ctx->stream));
    m->inst.clear();
  });
}

os_status os_mpnn_loss_grad(os_mpnn *m, int32_t index, float *loss, float *grads, size_t cap) {
  return guard([&] {
    OS_REQUIRE(m && index >= 0 && index < (int)m->inst.size(), "no instance %d", index);
    MpnnInstance &in = *m->inst[index];
    OS_REQUIRE(in.y.count, "instance %d has no labels", index);
    activate(m->ctx);
    cudaStream_t s = m->ctx->stream;
    ensure_work(m, in.np);
    OS_CUDA(cudaMemsetAsync(m->grad.get(), 0, sizeof(float) * m->nparam, s));
    OS_CUDA(cudaMemsetAsync(m->loss.get(), 0, sizeof(float), s));
    forward(m, in, s);
    backward(m, in, s);
    if (loss) OS_CUDA(cudaMemcpyAsync(loss, m->loss.get(), sizeof(float), cudaMemcpyDeviceToHost, s));
    if (grads) {
      OS_REQUIRE(cap >= m->nparam, "gradient buffer too small");
      OS_CUDA(cudaMemcpyAsync(grads, m->grad.get(), sizeof(float) * m->nparam, cudaMemcpyDeviceToHost, s));
    }
    OS_CUDA(cudaStreamSynchronize(s));
    check_tc_status(m);
  });
}

os_status os_mpnn_train(os_mpnn *m, int32_t epochs, float lr, uint64_t shuffle_seed, float *epoch_loss) {
  return guard([&] {
    OS_REQUIRE(m && epochs >= 0 && lr > 0.f, "bad arguments");
    activate(m->ctx);
    cudaStream_t s = m->ctx->stream;
    std::vector<int> order;
    for (int i = 0; i < (int)m->inst.size(); ++i)
      if (m->inst[i]->y.count) order.push_back(i);
    OS_REQUIRE(!order.empty(), "no labelled instances");
    int npmax = 0;
    for (int i : order) npmax = std::max(npmax, m->inst[i]->np);
    ensure_work(m, npmax);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    unsigned long long st = shuffle_seed * 0x9E3779B97F4A7C15ull + 1;
    for (int e = 0; e < epochs; ++e) {
      for (size_t i = order.size(); i > 1; --i) {  // Fisher-Yates with a splitmix stream
        st += 0x9E3779B97F4A7C15ull;
        unsigned long long z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        std::swap(order[i - 1], order[z % i]);
      }
      OS_CUDA(cudaMemsetAsync(m->loss.get(), 0, sizeof(float), s));
      for (int idx : order) {
        MpnnInstance &in = *m->inst[idx];
        OS_CUDA(cudaMemsetAsync(m->grad.get(), 0, sizeof(float) * m->nparam, s));
        forward(m, in, s);
        backward(m, in, s);
        ++m->adam_t;
        const float c1 = 1.f - std::pow(b1, (float)m->adam_t), c2 = 1.f - std::pow(b2, (float)m->adam_t);
        adam_kernel<<<(unsigned)ceil_div_u64(m->nparam, 256), 256, 0, s>>>(
            m->param.get(), m->grad.get(), m->adam_m.get(), m->adam_v.get(), m->nparam, lr, b1, b2, eps, c1, c2);
        OS_CUDA(cudaGetLastError());
      }
      if (epoch_loss) {
        float l = 0.f;
        OS_CUDA(cudaMemcpyAsync(&l, m->loss.get(), sizeof(float), cudaMemcpyDeviceToHost, s));
        OS_CUDA(cudaStreamSynchronize(s));
        epoch_loss[e] = l / (float)order.size();
      }
    }
    OS_CUDA(cudaStreamSynchronize(s));
    if (m->tc_status.count) check_tc_status(m);
  });
}

}  // extern "C"

namespace {

// Persistent prediction buffers and one captured graph per size: the
// staging (from m->ptmp.f), its 112 power-iteration launches and the forward
// pass replay as one launch, which leaves P(x_i = 1) in m->prob.
void predict_prepare(os_mpnn *m, int n, cudaStream_t s) {
  if (!m->pin || m->pin->n != n) {
    m->pin = std::make_unique<MpnnInstance>();
    stage_alloc(*m->pin, m->ptmp, n);
  }
  MpnnInstance &in = *m->pin;
  ensure_work(m, in.np);
  if (m->pgraph && (m->pgraph_n != n || m->pgraph_cap != m->cap)) {
    cudaGraphExecDestroy(m->pgraph);
    m->pgraph = nullptr;
  }
  if (!m->pgraph) {
    cudaGraph_t g = nullptr;
    OS_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      stage_enqueue(in, m->ptmp, s);
      forward(m, in, s);
      const float *HL = m->Hs.get() + (size_t)m->L * in.np * m->H;
      float *P = m->param.get();
      head_kernel<<<(n + 255) / 256, 256, 0, s>>>(HL, P + m->off_wout(), P + m->off_bout(), nullptr, n, m->H,
                                                  m->prob.get(), nullptr, nullptr);
    } catch (...) {
      // leave the stream out of capture mode before reporting
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();
      throw;
    }
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    OS_CUDA(le);
    OS_CUDA(ce);
    const cudaError_t ie = cudaGraphInstantiate(&m->pgraph, g, 0);
    cudaGraphDestroy(g);
    OS_CUDA(ie);
    m->pgraph_n = n;
    m->pgraph_cap = m->cap;
  }
}

}  // namespace

extern "C" {

os_status os_mpnn_predict(os_mpnn *m, const os_qubo_dense *q, float *prob) {
  return guard([&] {
    OS_REQUIRE(m && q && q->f && prob, "null argument");
    activate(m->ctx);
    cudaStream_t s = m->ctx->stream;
    const int n = q->n;
    OS_REQUIRE(n >= 2 && n <= 8192, "the network takes 2..8192 spins (got %d)", n);
    predict_prepare(m, n, s);
    OS_CUDA(cudaMemcpyAsync(m->ptmp.f.get(), q->f, sizeof(double) * (size_t)n * n, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaGraphLaunch(m->pgraph, s));
    OS_CUDA(cudaMemcpyAsync(prob, m->prob.get(), sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    double bad = 0.0;
    OS_CUDA(cudaMemcpyAsync(&bad, m->ptmp.stats.get() + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
    check_tc_status(m);
    OS_REQUIRE(bad == 0.0, "the QUBO has non-finite coefficients");
  });
}

os_status os_sa_plan_warm_start(os_sa_plan *p, os_mpnn *m) {
  return guard([&] {
    OS_REQUIRE(p && m, "null argument");
    OS_REQUIRE(p->kind == 0, "the warm start takes a dense plan");
    OS_REQUIRE(p->ctx == m->ctx, "the plan and the network must share a context");
    activate(p->ctx);
    cudaStream_t s = p->ctx->stream;
    const int n = p->n;
    OS_REQUIRE(n >= 2 && n <= 8192, "the network takes 2..8192 spins (got %d)", n);
    predict_prepare(m, n, s);
    // The plan's matrix as given is already on the device (and was checked
    // finite when the plan was created): a device copy into the staging
    // buffer, the graph, and the probabilities straight into the plan.
    OS_CUDA(cudaMemcpyAsync(m->ptmp.f.get(), p->f.get(), sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice,
                            s));
    OS_CUDA(cudaGraphLaunch(m->pgraph, s));
    if (p->init_prob.count != (size_t)n) p->init_prob.alloc(n);
    OS_CUDA(cudaMemcpyAsync(p->init_prob.get(), m->prob.get(), sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  });
}

}  // extern "C"
