// sa_sparse.cu -- simulated annealing on sparse QUBOs (Chimera droplets).
//
// Replaces sa::anneal (include/simulated_annealing/annealing.hpp:55-140) for
// sparse instances such as the reference's Chimera benchmarks
// (benchmarks/annealing/chimera_droplets_qbsolv, 2048 spins, ~6 couplers per
// spin). The reference recomputes the full dense O(n^2) energy per attempt;
// here each trajectory keeps FP32 local fields in shared memory.
//
// Sites are coloured on the host so that no coupler joins two sites of one
// colour (Chimera is bipartite: two colours). A sweep visits the colours in
// order; all sites of a colour are attempted in parallel, which is exactly a
// sequential sweep in colour-sorted site order because the attempts within a
// colour do not interact. An accepted flip adds +/- its CSR row to the
// neighbours' fields with shared-memory atomics (neighbours of one colour
// are all of other colours, so no field read in the current colour changes).
// The energy is tracked per sweep and the best state is checked once per
// sweep. FP64 resyncs recompute the fields from the spins and record the
// drift of the FP32 fields.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <queue>
#include <vector>

#include "common.cuh"
#include "philox.cuh"
#include "sa_common.cuh"
#include "sa_plan.cuh"

namespace os {
namespace sa {

struct SparseArgs {
  const int *row_ptr;
  const int *col;
  const float *val;
  const float *diag;
  const int *color_sites;
  const int *color_ptr;
  int ncolors, n, deg_max;
  const int2 *ell;        // [n][deg_max] (neighbour site, coupling bits); site -1 past a site's degree
  const double *beta;
  int spb, step_begin, step_end, acceptance;
  int T, traj_per_cta;
  uint32_t seed_lo, seed_hi, instance;
  float *h;               // [T][n]
  uint8_t *x;             // [T][n]
  uint8_t *xbest;         // [T][n]
  double *e;              // [T]
  double *ebest;          // [T]
  unsigned long long *accepted;
};

// Neighbour updates of a warp's accepted sites, applied once the colour is
// decided (no coupler joins two sites of one colour, so the colour's own
// decisions never read a field these updates touch). `list` holds `cnt`
// entries (site << 1 | negative); lane l serves neighbour `le` of entry
// g + lr of each group of `per` entries (lr = l / deg_max, le = l % deg_max),
// so the shared-memory atomics run with nearly full warps. Four groups per
// iteration keep their table loads in flight together.
__device__ __forceinline__ void apply_updates(const uint32_t *__restrict__ list, int cnt, int per, int lr, int le,
                                              int deg_max, const int2 *__restrict__ ell, float *__restrict__ h) {
  for (int g = 0; g < cnt; g += 4 * per) {
    int2 nb[4];
    uint32_t e[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = g + u * per + lr;
      e[u] = (lr < per && r < cnt) ? list[r] : 0xffffffffu;
      nb[u] = e[u] != 0xffffffffu ? ell[(size_t)(e[u] >> 1) * deg_max + le] : make_int2(-1, 0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (nb[u].x >= 0) atomicAdd(&h[nb[u].x], (e[u] & 1u) ? -__int_as_float(nb[u].y) : __int_as_float(nb[u].y));
  }
}

__global__ void __launch_bounds__(256, 8) sa_sparse_kernel(const __grid_constant__ SparseArgs a) {
  extern __shared__ unsigned char smem[];
  const int R = a.traj_per_cta;
  const int tpt = blockDim.x / R;            // threads per trajectory (multiple of 32)
  const int slot = threadIdx.x / tpt;        // trajectory within the CTA
  const int tid = threadIdx.x % tpt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = a.n;
  float *h_all = reinterpret_cast<float *>(smem);
  uint8_t *x_all = reinterpret_cast<uint8_t *>(h_all + (size_t)R * n);
  __shared__ uint32_t s_list[8][128];   // per warp: accepted sites of the colour (<= 4 x 32)
  __shared__ float s_de[8];
  __shared__ double s_e[8], s_eb[8];
  __shared__ int s_improve[8];
  const int t = blockIdx.x * R + slot;
  const bool active = t < a.T;
  float *h = h_all + (size_t)slot * n;
  uint8_t *x = x_all + (size_t)slot * n;
  if (active) {
    for (int i = tid; i < n; i += tpt) {
      h[i] = a.h[(size_t)t * n + i];
      x[i] = a.x[(size_t)t * n + i];
    }
  }
  if (tid == 0) {
    s_de[slot] = 0.f;
    s_e[slot] = active ? a.e[t] : 0.0;
    s_eb[slot] = active ? a.ebest[t] : 0.0;
  }
  __syncthreads();
  unsigned acc = 0;
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSweep;
  const bool coop = a.deg_max <= 32;
  const int per = coop ? 32 / a.deg_max : 0;
  const int lr = coop ? lane / a.deg_max : 0, le = coop ? lane - lr * a.deg_max : 0;
  for (int step = a.step_begin; step < a.step_end; ++step) {
    const float b = (float)a.beta[step / a.spb];
    float de = 0.f;
    for (int c = 0; c < a.ncolors; ++c) {
      const int c0 = a.color_ptr[c], cnt = a.color_ptr[c + 1] - c0;
      // Warp-uniform trip count (the warp's first thread decides), so that
      // every lane takes part in the ballots; thread tid attempts the same
      // sites with the same Philox counters as a per-thread loop would.
      for (int wbase = tid - lane; wbase < cnt; wbase += 4 * tpt) {
        const int mybase = wbase + lane;
        const Philox4 r = philox4x32_10((uint32_t)(c0 + mybase), (uint32_t)step, (uint32_t)t, c3, a.seed_lo,
                                        a.seed_hi);
        int listed = 0;  // warp-uniform
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const int idx = mybase + m * tpt;
          const bool valid = active && idx < cnt;
          int k = 0;
          bool accept = false;
          bool neg = false;
          if (valid) {
            k = a.color_sites[c0 + idx];
            const uint32_t w = m == 0 ? r.x : m == 1 ? r.y : m == 2 ? r.z : r.w;
            const float l = __logf(u01_open(w));
            const float theta = a.acceptance == OS_ACCEPT_REFERENCE ? -b * l : -l / b;
            const float loc = a.diag[k] + h[k];
            const bool xk = x[k];
            const float dE = xk ? -loc : loc;
            accept = dE < theta;
            if (accept) {
              x[k] = xk ? 0 : 1;
              neg = xk;
              de += dE;
              ++acc;
            }
          }
          if (coop) {
            const unsigned M = __ballot_sync(0xffffffffu, accept);
            if (accept) s_list[warp][listed + __popc(M & ((1u << lane) - 1u))] = ((uint32_t)k << 1) | (neg ? 1u : 0u);
            listed += __popc(M);
          } else if (accept) {
            const float sgn = neg ? -1.f : 1.f;
            const int e1 = a.row_ptr[k + 1];
            for (int e = a.row_ptr[k]; e < e1; ++e) atomicAdd(&h[a.col[e]], sgn * a.val[e]);
          }
        }
        if (coop && listed) {
          __syncwarp();
          apply_updates(s_list[warp], listed, per, lr, le, a.deg_max, a.ell, h);
          __syncwarp();
        }
      }
      if (c + 1 < a.ncolors) __syncthreads();
    }
    // Sweep end: energy of each trajectory and best-state check. Each thread
    // copies only the sites it attempts itself (colour index = tid mod tpt),
    // which no other thread writes, so the copy needs no barrier after it.
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) de += __shfl_xor_sync(0xffffffffu, de, off);
    if (lane == 0) atomicAdd(&s_de[slot], de);
    __syncthreads();
    if (tid == 0) {
      const double En = s_e[slot] + (double)s_de[slot];
      const bool imp = active && En < s_eb[slot];
      s_e[slot] = En;
      if (imp) s_eb[slot] = En;
      s_improve[slot] = imp;
      s_de[slot] = 0.f;
    }
    __syncthreads();
    if (s_improve[slot]) {
      for (int c = 0; c < a.ncolors; ++c) {
        const int c0 = a.color_ptr[c], cnt = a.color_ptr[c + 1] - c0;
        for (int idx = tid; idx < cnt; idx += tpt) {
          const int k = a.color_sites[c0 + idx];
          a.xbest[(size_t)t * n + k] = x[k];
        }
      }
    }
    if (acc >= (1u << 30)) {
      atomicAdd(&a.accepted[t], (unsigned long long)acc);
      acc = 0;
    }
  }
  __syncthreads();
  if (active) {
    for (int i = tid; i < n; i += tpt) {
      a.h[(size_t)t * n + i] = h[i];
      a.x[(size_t)t * n + i] = x[i];
    }
    if (tid == 0) {
      a.e[t] = s_e[slot];
      a.ebest[t] = s_eb[slot];
    }
    // Accepted-flip count: one atomic per thread with flips.
    if (acc) atomicAdd(&a.accepted[t], (unsigned long long)acc);
  }
}

struct SparseResyncArgs {
  const int *row_ptr;
  const int *col;
  const double *val;
  const double *diag;
  int n, T, init;
  const float *init_prob;
  uint32_t seed_lo, seed_hi, instance;
  float *h;
  uint8_t *x;
  uint8_t *xbest;
  double *e;
  double *ebest;
  unsigned long long *drift_bits;
};

// Initial spins (one Philox call per four sites of a trajectory).
__global__ void sa_sparse_init_kernel(const __grid_constant__ SparseResyncArgs a) {
  const int t = blockIdx.y;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;  // group of 4 sites
  if (t >= a.T || 4 * g >= a.n) return;
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamInit;
  const Philox4 r = philox4x32_10((uint32_t)g, 0u, (uint32_t)t, c3, a.seed_lo, a.seed_hi);
  const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int k = 4 * g + m;
    if (k >= a.n) break;
    const bool bit = a.init_prob ? (u01_open(w[m]) < a.init_prob[k]) : (w[m] >> 31) != 0;
    a.x[(size_t)t * a.n + k] = bit;
  }
}

// FP64 fields from the spins, drift of the FP32 fields, FP64 energy. One
// CTA per trajectory.
__global__ void __launch_bounds__(256) sa_sparse_resync_kernel(const __grid_constant__ SparseResyncArgs a) {
  const int t = blockIdx.x;
  if (t >= a.T) return;
  const uint8_t *x = a.x + (size_t)t * a.n;
  float *h = a.h + (size_t)t * a.n;
  double epart = 0.0, drift = 0.0;
  for (int j = threadIdx.x; j < a.n; j += blockDim.x) {
    double acc = 0.0;
    for (int e = a.row_ptr[j]; e < a.row_ptr[j + 1]; ++e)
      if (x[a.col[e]]) acc += a.val[e];
    if (!a.init) drift = fmax(drift, fabs((double)h[j] - acc));
    if (x[j]) epart += a.diag[j] + 0.5 * acc;
    h[j] = (float)acc;
  }
  __shared__ double s_e[8], s_d[8];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    epart += __shfl_xor_sync(0xffffffffu, epart, off);
    drift = fmax(drift, __shfl_xor_sync(0xffffffffu, drift, off));
  }
  if ((threadIdx.x & 31) == 0) {
    s_e[threadIdx.x >> 5] = epart;
    s_d[threadIdx.x >> 5] = drift;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double es = 0.0, dm = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      es += s_e[i];
      dm = fmax(dm, s_d[i]);
    }
    a.e[t] = es;
    if (a.init) a.ebest[t] = es;
    if (!a.init && a.drift_bits) atomicMax(a.drift_bits, (unsigned long long)__double_as_longlong(dm));
  }
  if (a.init)
    for (int j = threadIdx.x; j < a.n; j += blockDim.x) a.xbest[(size_t)t * a.n + j] = x[j];
}

// FP64 energy of each best state in the reference's summation order
// (annealing.hpp:31-40): set pairs (i <= j) in row-major order; CSR columns
// are ascending so the sparse walk adds the same non-zero terms in the same
// order as the dense loop.
__global__ void sa_sparse_rescore_kernel(const int *__restrict__ row_ptr, const int *__restrict__ col,
                                         const double *__restrict__ val, const double *__restrict__ diag,
                                         int n, int T, const uint8_t *__restrict__ xs,
                                         double *__restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const uint8_t *x = xs + (size_t)t * n;
  double e = 0.0;
  for (int i = 0; i < n; ++i) {
    if (!x[i]) continue;
    e += diag[i];
    for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
      const int j = col[k];
      if (j > i && x[j]) e += val[k];
    }
  }
  out[t] = e;
}

// Colouring: BFS two-colouring when the coupling graph is bipartite,
// otherwise greedy colouring in descending-degree order.
int color_graph(int n, const std::vector<int> &rp, const std::vector<int> &cl, std::vector<int> &color) {
  color.assign(n, -1);
  bool bip = true;
  for (int s = 0; s < n && bip; ++s) {
    if (color[s] >= 0) continue;
    color[s] = 0;
    std::queue<int> q;
    q.push(s);
    while (!q.empty() && bip) {
      int v = q.front();
      q.pop();
      for (int e = rp[v]; e < rp[v + 1]; ++e) {
        int w = cl[e];
        if (color[w] < 0) {
          color[w] = 1 - color[v];
          q.push(w);
        } else if (color[w] == color[v]) {
          bip = false;
          break;
        }
      }
    }
  }
  if (bip) {
    int nc = 1;
    for (int v = 0; v < n; ++v) nc = std::max(nc, color[v] + 1);
    return nc;
  }
  std::vector<int> order(n);
  for (int v = 0; v < n; ++v) order[v] = v;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return rp[a + 1] - rp[a] > rp[b + 1] - rp[b]; });
  color.assign(n, -1);
  int nc = 0;
  std::vector<int> used;
  for (int v : order) {
    used.assign(nc + 1, 0);
    for (int e = rp[v]; e < rp[v + 1]; ++e)
      if (color[cl[e]] >= 0 && color[cl[e]] <= nc) used[color[cl[e]]] = 1;
    int c = 0;
    while (c < nc && used[c]) ++c;
    color[v] = c;
    nc = std::max(nc, c + 1);
  }
  return nc;
}

void plan_create_sparse(os_sa_plan *p, const os_qubo_csr *q) {
  OS_REQUIRE(q && q->row_ptr && q->diag, "null CSR");
  const int n = q->n;
  OS_REQUIRE(n >= 1, "empty instance");
  OS_REQUIRE(p->T <= 65535, "sparse annealing runs at most 65535 trajectories per call");
  OS_REQUIRE(q->row_ptr[0] == 0, "row_ptr[0] must be 0");
  const int nnz = q->row_ptr[n];
  OS_REQUIRE(nnz >= 0 && (nnz == 0 || (q->col && q->val)), "bad CSR arrays");
  std::vector<int> rp(q->row_ptr, q->row_ptr + n + 1), cl(q->col, q->col + nnz);
  std::vector<double> vl(q->val, q->val + nnz), dg(q->diag, q->diag + n);
  // Rows sorted by column, no diagonal entries, symmetric values.
  std::map<std::pair<int, int>, double> m;
  for (int i = 0; i < n; ++i) {
    OS_REQUIRE(rp[i + 1] >= rp[i], "row_ptr not monotone at %d", i);
    OS_REQUIRE(std::isfinite(dg[i]), "diag[%d] not finite", i);
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      OS_REQUIRE(cl[e] >= 0 && cl[e] < n && cl[e] != i, "bad column %d in row %d", cl[e], i);
      OS_REQUIRE(e == rp[i] || cl[e] > cl[e - 1], "row %d not strictly sorted", i);
      OS_REQUIRE(std::isfinite(vl[e]), "value in row %d not finite", i);
      m[{i, cl[e]}] = vl[e];
    }
  }
  for (auto &kv : m) {
    auto it = m.find({kv.first.second, kv.first.first});
    OS_REQUIRE(it != m.end() && it->second == kv.second, "CSR is not symmetric at (%d,%d)",
               kv.first.first, kv.first.second);
  }
  std::vector<int> color;
  const int nc = color_graph(n, rp, cl, color);
  std::vector<int> cptr(nc + 1, 0), csites;
  for (int v = 0; v < n; ++v) cptr[color[v] + 1]++;
  for (int c = 0; c < nc; ++c) cptr[c + 1] += cptr[c];
  csites.resize(n);
  std::vector<int> fill(cptr.begin(), cptr.end() - 1);
  for (int v = 0; v < n; ++v) csites[fill[color[v]]++] = v;
  std::vector<float> v32(vl.begin(), vl.end()), d32(dg.begin(), dg.end());

  p->n = n;
  p->nnz = nnz;
  p->ncolors = nc;
  p->deg_max = 0;
  for (int i = 0; i < n; ++i) p->deg_max = std::max(p->deg_max, rp[i + 1] - rp[i]);
  p->deg_max = std::max(p->deg_max, 1);
  {
    std::vector<int2> ell((size_t)n * p->deg_max, make_int2(-1, 0));
    for (int i = 0; i < n; ++i)
      for (int e = rp[i]; e < rp[i + 1]; ++e) {
        const float v = (float)vl[e];
        int bits;
        std::memcpy(&bits, &v, sizeof bits);
        ell[(size_t)i * p->deg_max + (e - rp[i])] = make_int2(cl[e], bits);
      }
    p->ell.alloc(ell.size());
    OS_CUDA(cudaMemcpy(p->ell.get(), ell.data(), sizeof(int2) * ell.size(), cudaMemcpyHostToDevice));
  }
  p->row_ptr.alloc(n + 1);
  p->col.alloc(nnz);
  p->val32.alloc(nnz);
  p->val64.alloc(nnz);
  p->diag32.alloc(n);
  p->diag64.alloc(n);
  p->color_sites.alloc(n);
  p->color_ptr.alloc(nc + 1);
  OS_CUDA(cudaMemcpy(p->row_ptr.get(), rp.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
  if (nnz) {
    OS_CUDA(cudaMemcpy(p->col.get(), cl.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice));
    OS_CUDA(cudaMemcpy(p->val32.get(), v32.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice));
    OS_CUDA(cudaMemcpy(p->val64.get(), vl.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice));
  }
  OS_CUDA(cudaMemcpy(p->diag32.get(), d32.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  OS_CUDA(cudaMemcpy(p->diag64.get(), dg.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  OS_CUDA(cudaMemcpy(p->color_sites.get(), csites.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  OS_CUDA(cudaMemcpy(p->color_ptr.get(), cptr.data(), sizeof(int) * (nc + 1), cudaMemcpyHostToDevice));
  const size_t T = p->T;
  p->sh.alloc(T * n);
  p->sx.alloc(T * n);
  p->sxbest.alloc(T * n);
  p->se.alloc(T);
  p->sebest.alloc(T);
  p->accepted.alloc(T);
  p->states.alloc(T * n);
  p->e64.alloc(T);
  // Threads per trajectory: one Philox call (four sites) per thread and
  // colour where the largest colour allows, 32..256; a CTA has 256 threads
  // (256 / tpt trajectories), eight CTAs per SM.
  int maxc = 1;
  for (int c = 0; c < nc; ++c) maxc = std::max(maxc, cptr[c + 1] - cptr[c]);
  int tpt = 32;
  while (tpt < 256 && tpt * 4 < maxc) tpt <<= 1;
  int R = 256 / tpt;
  const size_t per = (size_t)n * 5;
  while (R > 1 && per * R > 100 * 1024) R >>= 1;  // R <= 8 (tpt >= 32)
  OS_REQUIRE(per <= 200 * 1024, "sparse instance too large for shared memory (%d variables)", n);
  p->traj_per_cta = R;
  p->warps = tpt * R / 32;
  OS_CUDA(cudaFuncSetAttribute(sa_sparse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)std::max<size_t>(per * R, 48 * 1024)));
}

void execute_sparse(os_sa_plan *p) {
  cudaStream_t s = p->ctx->stream;
  p->launches = 0;
  const int n = p->n, T = p->T;
  OS_CUDA(cudaMemsetAsync(p->accepted.get(), 0, sizeof(unsigned long long) * T, s));
  OS_CUDA(cudaMemsetAsync(p->drift.get(), 0, sizeof(unsigned long long), s));
  SparseResyncArgs r{};
  r.row_ptr = p->row_ptr.get();
  r.col = p->col.get();
  r.val = p->val64.get();
  r.diag = p->diag64.get();
  r.n = n;
  r.T = T;
  r.init = 1;
  r.init_prob = p->init_prob.count ? p->init_prob.get() : nullptr;
  r.seed_lo = (uint32_t)p->seed;
  r.seed_hi = (uint32_t)(p->seed >> 32);
  r.instance = 0;
  r.h = p->sh.get();
  r.x = p->sx.get();
  r.xbest = p->sxbest.get();
  r.e = p->se.get();
  r.ebest = p->sebest.get();
  r.drift_bits = p->drift.get();
  dim3 ig((unsigned)ceil_div_u64((n + 3) / 4, 128), T);
  sa_sparse_init_kernel<<<ig, 128, 0, s>>>(r);
  OS_CUDA(cudaGetLastError());
  sa_sparse_resync_kernel<<<T, 256, 0, s>>>(r);
  OS_CUDA(cudaGetLastError());
  p->launches += 2;
  r.init = 0;

  SparseArgs a{};
  a.row_ptr = p->row_ptr.get();
  a.col = p->col.get();
  a.val = p->val32.get();
  a.diag = p->diag32.get();
  a.color_sites = p->color_sites.get();
  a.color_ptr = p->color_ptr.get();
  a.ncolors = p->ncolors;
  a.n = n;
  a.deg_max = p->deg_max;
  a.ell = p->ell.get();
  a.beta = p->beta.get();
  a.spb = p->spb;
  a.acceptance = p->acceptance;
  a.T = T;
  a.traj_per_cta = p->traj_per_cta;
  a.seed_lo = r.seed_lo;
  a.seed_hi = r.seed_hi;
  a.instance = 0;
  a.h = p->sh.get();
  a.x = p->sx.get();
  a.xbest = p->sxbest.get();
  a.e = p->se.get();
  a.ebest = p->sebest.get();
  a.accepted = p->accepted.get();
  const int R = p->traj_per_cta;
  const int threads = p->warps * 32;
  const size_t smem = (size_t)n * 5 * R;
  const int grid = (T + R - 1) / R;
  p->sweep_ev_used = 0;
  for (int s0 = 0; s0 < p->steps; s0 += p->chunk) {
    a.step_begin = s0;
    a.step_end = std::min(p->steps, s0 + p->chunk);
    OS_CUDA(cudaEventRecord(p->event(2 * p->sweep_ev_used), s));
    sa_sparse_kernel<<<grid, threads, smem, s>>>(a);
    OS_CUDA(cudaGetLastError());
    OS_CUDA(cudaEventRecord(p->event(2 * p->sweep_ev_used + 1), s));
    ++p->sweep_ev_used;
    sa_sparse_resync_kernel<<<T, 256, 0, s>>>(r);
    OS_CUDA(cudaGetLastError());
    p->launches += 2;
  }
  OS_CUDA(cudaMemcpyAsync(p->states.get(), p->sxbest.get(), (size_t)T * n, cudaMemcpyDeviceToDevice, s));
  sa_sparse_rescore_kernel<<<(T + 127) / 128, 128, 0, s>>>(p->row_ptr.get(), p->col.get(), p->val64.get(),
                                                           p->diag64.get(), n, T, p->states.get(),
                                                           p->e64.get());
  OS_CUDA(cudaGetLastError());
  p->launches += 1;
}

}  // namespace sa
}  // namespace os

using namespace os;
using namespace os::sa;

extern "C" {

os_status os_sa_plan_create_sparse(os_ctx *ctx, const os_qubo_csr *qubo, const os_sa_params *params,
                                   os_sa_plan **out) {
  return guard([&] {
    activate(ctx);
    OS_REQUIRE(out != nullptr, "null output");
    check_schedule(params);
    OS_REQUIRE(params->resync_every >= 0, "resync_every = -1 (no resync) is for dense plans only");
    OS_REQUIRE(qubo != nullptr, "null QUBO");
    OS_REQUIRE(params->site_order == OS_SITES_SEQUENTIAL,
               "sparse annealing sweeps all sites per step (site_order must be SEQUENTIAL)");
    auto *p = new os_sa_plan();
    try {
      p->kind = 1;
      os_sa_plan_common(p, ctx, params, qubo->n);
      plan_create_sparse(p, qubo);
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

os_status os_sa_run_sparse(os_ctx *ctx, const os_qubo_csr *qubo, const os_sa_params *params,
                           os_sa_result *result) {
  os_sa_plan *plan = nullptr;
  os_status st = os_sa_plan_create_sparse(ctx, qubo, params, &plan);
  if (st != OS_OK) return st;
  st = os_sa_plan_execute(plan);
  if (st == OS_OK) st = os_sa_plan_result(plan, result);
  os_sa_plan_destroy(plan);
  return st;
}

}  // extern "C"
