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
//
// The same sweep kernel also serves the two solvers the reference's annealing
// benchmark names as next (benchmarks/annealing/performance.md:52-59):
// parallel tempering (each replica at its own inverse temperature, replica
// exchange between launches) and population annealing (systematic resampling
// between temperatures, the copy folded into the sweep's state load).
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
  const int *temp;        // tempering: temperature index of each trajectory into beta
  // Population annealing: trajectory t starts from replica parent[t] of the
  // previous population (these arrays) and is written to h, x, xbest, e,
  // ebest; anc[t] = anc_in[parent[t]].
  const int *parent;
  const float *h_in;
  const uint8_t *x_in, *xbest_in;
  const double *e_in, *ebest_in;
  const int *anc_in;
  int *anc;
  // Replay mode only (REPLAY kernel): the threshold of every attempt,
  // thr[(t * nsteps + step) * n + site], in place of the Philox draws.
  const float *thr;
  int nsteps;
};

enum SweepMode : int { kAnneal = 0, kTemper = 1, kPopulation = 2 };

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

// MODE kAnneal: annealing, beta[step / spb] from the schedule. kTemper:
// parallel tempering, each trajectory at its own fixed inverse temperature
// beta[temp[t]] for the whole launch. kPopulation: annealing whose
// trajectories start from their resampled parents (population annealing);
// the copy rides on the launch's own state load.
template <int MODE, bool REPLAY = false>
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
  if constexpr (MODE == kPopulation) {
    const int src = active ? a.parent[t] : 0;
    if (active) {
      for (int i = tid; i < n; i += tpt) {
        h[i] = a.h_in[(size_t)src * n + i];
        x[i] = a.x_in[(size_t)src * n + i];
        a.xbest[(size_t)t * n + i] = a.xbest_in[(size_t)src * n + i];
      }
      if (tid == 0) a.anc[t] = a.anc_in[src];
    }
    if (tid == 0) {
      s_de[slot] = 0.f;
      s_e[slot] = active ? a.e_in[src] : 0.0;
      s_eb[slot] = active ? a.ebest_in[src] : 0.0;
    }
  } else {
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
  }
  __syncthreads();
  unsigned acc = 0;
  const uint32_t c3 = (a.instance & 0x0FFFFFFFu) | kStreamSweep;
  const bool coop = a.deg_max <= 32;
  const int per = coop ? 32 / a.deg_max : 0;
  const int lr = coop ? lane / a.deg_max : 0, le = coop ? lane - lr * a.deg_max : 0;
  float b_fixed = 1.f;
  if constexpr (MODE == kTemper) b_fixed = active ? (float)a.beta[a.temp[t]] : 1.f;
  for (int step = a.step_begin; step < a.step_end; ++step) {
    const float b = MODE == kTemper ? b_fixed : (float)a.beta[step / a.spb];
    const float inv_b = 1.0f / b;  // physical rule: -ln(u) * (1 / beta), no division per attempt
    float de = 0.f;
    for (int c = 0; c < a.ncolors; ++c) {
      const int c0 = a.color_ptr[c], cnt = a.color_ptr[c + 1] - c0;
      // Warp-uniform trip count (the warp's first thread decides), so that
      // every lane takes part in the ballots; thread tid attempts the same
      // sites with the same Philox counters as a per-thread loop would.
      for (int wbase = tid - lane; wbase < cnt; wbase += 4 * tpt) {
        const int mybase = wbase + lane;
        Philox4 r{0, 0, 0, 0};
        if constexpr (!REPLAY)
          r = philox4x32_10((uint32_t)(c0 + mybase), (uint32_t)step, (uint32_t)t, c3, a.seed_lo, a.seed_hi);
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
            float theta;
            if constexpr (REPLAY) {
              theta = a.thr[((size_t)t * a.nsteps + step) * n + k];
            } else {
              const uint32_t w = m == 0 ? r.x : m == 1 ? r.y : m == 2 ? r.z : r.w;
              const float l = __logf(u01_open(w));
              theta = a.acceptance == OS_ACCEPT_REFERENCE ? -b * l : -l * inv_b;
            }
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
  const uint8_t *init_bits;   // optional initial spins [T][n] (replay mode)
};

// Initial spins (one Philox call per four sites of a trajectory, or the
// caller's spins in replay mode).
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
    bool bit = a.init_prob ? (u01_open(w[m]) < a.init_prob[k]) : (w[m] >> 31) != 0;
    if (a.init_bits) bit = a.init_bits[(size_t)t * a.n + k] != 0;
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

// FP64 energy of each state (n bytes per state) under the reference's
// energy function (annealing.hpp:31-40): the set diagonal terms and the set
// pairs i < j. One warp per state: lane l sums rows l, l + 32, ... (each row's
// terms in column order), and a fixed shuffle tree adds the 32 partial sums,
// so the value differs from the serial row-major sum by rounding only.
__global__ void __launch_bounds__(256) sa_sparse_rescore_kernel(const int *__restrict__ row_ptr,
                                                                const int *__restrict__ col,
                                                                const double *__restrict__ val,
                                                                const double *__restrict__ diag, int n, int T,
                                                                const uint8_t *__restrict__ xs,
                                                                double *__restrict__ out) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= T) return;
  const uint8_t *x = xs + (size_t)w * n;
  double e = 0.0;
  for (int i = lane; i < n; i += 32) {
    if (!x[i]) continue;
    double r = diag[i];
    for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
      const int j = col[k];
      if (j > i && x[j]) r += val[k];
    }
    e += r;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) e += __shfl_xor_sync(0xffffffffu, e, off);
  if (lane == 0) out[w] = e;
}

static unsigned rescore_blocks(int T) { return (unsigned)ceil_div_u64((unsigned long long)T * 32, 256); }

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
  p->host_color_sites = csites;
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
  for (auto fn : {sa_sparse_kernel<kAnneal>, sa_sparse_kernel<kTemper>, sa_sparse_kernel<kPopulation>,
                  sa_sparse_kernel<kAnneal, true>})
    OS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)std::max<size_t>(per * R, 48 * 1024)));
}

// Resets the counters, draws the initial spins and computes their FP64
// fields and energies; returns the resync arguments (init = 0) for later
// resyncs.
static SparseResyncArgs start_sparse(os_sa_plan *p) {
  cudaStream_t s = p->ctx->stream;
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
  r.init_bits = p->replay ? p->rp_init.get() : nullptr;
  dim3 ig((unsigned)ceil_div_u64((n + 3) / 4, 128), T);
  sa_sparse_init_kernel<<<ig, 128, 0, s>>>(r);
  OS_CUDA(cudaGetLastError());
  sa_sparse_resync_kernel<<<T, 256, 0, s>>>(r);
  OS_CUDA(cudaGetLastError());
  p->launches += 2;
  r.init = 0;
  return r;
}

static SparseArgs sweep_args(os_sa_plan *p, const SparseResyncArgs &r) {
  SparseArgs a{};
  a.row_ptr = p->row_ptr.get();
  a.col = p->col.get();
  a.val = p->val32.get();
  a.diag = p->diag32.get();
  a.color_sites = p->color_sites.get();
  a.color_ptr = p->color_ptr.get();
  a.ncolors = p->ncolors;
  a.n = p->n;
  a.deg_max = p->deg_max;
  a.ell = p->ell.get();
  a.beta = p->beta.get();
  a.spb = p->spb;
  a.acceptance = p->acceptance;
  a.T = p->T;
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
  a.temp = nullptr;
  a.thr = p->replay ? p->rp_thr.get() : nullptr;
  a.nsteps = p->steps;
  return a;
}

// FP64 re-score of the best state of every trajectory into p->e64.
static void finish_sparse(os_sa_plan *p) {
  cudaStream_t s = p->ctx->stream;
  const int n = p->n, T = p->T;
  OS_CUDA(cudaMemcpyAsync(p->states.get(), p->sxbest.get(), (size_t)T * n, cudaMemcpyDeviceToDevice, s));
  sa_sparse_rescore_kernel<<<rescore_blocks(T), 256, 0, s>>>(p->row_ptr.get(), p->col.get(), p->val64.get(),
                                                           p->diag64.get(), n, T, p->states.get(),
                                                           p->e64.get());
  OS_CUDA(cudaGetLastError());
  p->launches += 1;
}

void execute_sparse(os_sa_plan *p) {
  cudaStream_t s = p->ctx->stream;
  p->launches = 0;
  const int n = p->n, T = p->T;
  const SparseResyncArgs r = start_sparse(p);
  SparseArgs a = sweep_args(p, r);
  const int R = p->traj_per_cta;
  const int threads = p->warps * 32;
  const size_t smem = (size_t)n * 5 * R;
  const int grid = (T + R - 1) / R;
  p->sweep_ev_used = 0;
  for (int s0 = 0; s0 < p->steps; s0 += p->chunk) {
    a.step_begin = s0;
    a.step_end = std::min(p->steps, s0 + p->chunk);
    OS_CUDA(cudaEventRecord(p->event(2 * p->sweep_ev_used), s));
    if (p->replay)
      sa_sparse_kernel<kAnneal, true><<<grid, threads, smem, s>>>(a);
    else
      sa_sparse_kernel<kAnneal><<<grid, threads, smem, s>>>(a);
    OS_CUDA(cudaGetLastError());
    OS_CUDA(cudaEventRecord(p->event(2 * p->sweep_ev_used + 1), s));
    ++p->sweep_ev_used;
    sa_sparse_resync_kernel<<<T, 256, 0, s>>>(r);
    OS_CUDA(cudaGetLastError());
    p->launches += 2;
  }
  finish_sparse(p);
}

// ---------------------------------------------------------------------------
// Parallel tempering (replica exchange; Swendsen and Wang, PRL 57 (1986);
// Hukushima and Nemoto, J. Phys. Soc. Jpn. 65 (1996)). No counterpart in the
// reference, whose annealing benchmark names it as the next solver
// (benchmarks/annealing/performance.md:52-59). Replicas keep their spins and
// fields; exchanges swap temperature labels only, so a round costs the sweep
// launch plus one thread per chain.
// ---------------------------------------------------------------------------

struct ExchangeArgs {
  const double *beta;          // [nt] inverse temperatures
  const double *e;             // [chains * nt] current energies
  int *temp;                   // [chains * nt] temperature index of each replica
  int *traj_at;                // [chains][nt] replica at each temperature
  unsigned long long *swaps;   // [nt - 1] accepted exchanges per pair
  int chains, nt, round0, rounds;
  uint32_t seed_lo, seed_hi;
};

// Rounds round0 .. round0 + rounds - 1 of the exchange step, one warp per
// chain: the pairs (k, k+1) of a round, k = round mod 2, k + 2, ..., are
// disjoint, so lane l takes the pairs k = round mod 2 + 2 (l + 32 i) and the
// round needs one pass of loads; the pair swaps when
// ln u < (beta[k+1] - beta[k]) * (E_cold - E_hot), i.e. with probability
// min(1, exp(...)), u from Philox (pair, round, chain) and drawn only when
// the exponent is negative.
__global__ void pt_exchange_kernel(const __grid_constant__ ExchangeArgs a) {
  const int lane = threadIdx.x & 31;
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // warp-uniform
  if (c >= a.chains) return;
  int *at = a.traj_at + c * a.nt;
  for (int r = a.round0; r < a.round0 + a.rounds; ++r) {
    for (int k = (r & 1) + 2 * lane; k + 1 < a.nt; k += 64) {
      const int hot = at[k], cold = at[k + 1];
      const double d = (a.beta[k + 1] - a.beta[k]) * (a.e[cold] - a.e[hot]);
      bool swap = d >= 0.0;
      if (!swap) {
        const Philox4 p = philox4x32_10((uint32_t)k, (uint32_t)r, (uint32_t)c, kStreamExchange, a.seed_lo,
                                        a.seed_hi);
        swap = log(u01_open64(p.x)) < d;
      }
      if (swap) {
        at[k] = cold;
        at[k + 1] = hot;
        a.temp[cold] = k;
        a.temp[hot] = k + 1;
        atomicAdd(&a.swaps[k], 1ull);
      }
    }
    __syncwarp();  // the next round reads pairs that other lanes wrote
  }
}

// Grid of the exchange kernel: 4 chains (warps) per 128-thread block.
static unsigned exchange_blocks(unsigned long long chains) { return (unsigned)ceil_div_u64(chains, 4); }

// Replica t = chain * nt + r starts at temperature r.
__global__ void pt_identity_kernel(int *temp, int *traj_at, int total, int nt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  temp[t] = t % nt;
  traj_at[t] = t;
}

static void check_ladder(const double *beta, int nt) {
  OS_REQUIRE(beta != nullptr && nt >= 1, "empty temperature ladder");
  for (int k = 0; k < nt; ++k) {
    OS_REQUIRE(std::isfinite(beta[k]) && beta[k] >= 0.0, "beta[%d] must be finite and >= 0", k);
    OS_REQUIRE(k == 0 || beta[k] >= beta[k - 1], "beta must be non-decreasing (beta[%d] < beta[%d])", k, k - 1);
  }
}

struct PtRun {
  os_sa_plan p;                // sparse buffers; T = chains * nt, beta = the ladder
  int chains = 0, nt = 0, rounds = 0, spr = 0, resync = 0;
  os::DevBuf<int> temp, traj_at;
  os::DevBuf<unsigned long long> swaps;
  os::DevBuf<double> efinal;   // FP64 energies of the final states
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~PtRun() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
};

// Host-only checks of the tempering parameters (no device needed).
static void check_pt_params(const os_qubo_csr *q, const os_pt_params *prm) {
  OS_REQUIRE(prm != nullptr && q != nullptr, "null argument");
  check_ladder(prm->beta, prm->num_temps);
  OS_REQUIRE(prm->num_chains >= 1, "num_chains must be positive");
  OS_REQUIRE(prm->num_rounds >= 1 && prm->sweeps_per_round >= 1, "num_rounds and sweeps_per_round must be positive");
  OS_REQUIRE(prm->resync_every >= 0, "resync_every must be >= 0");
  const unsigned long long total = (unsigned long long)prm->num_chains * (unsigned long long)prm->num_temps;
  OS_REQUIRE(total <= 65535, "parallel tempering runs at most 65535 replicas (chains x temperatures)");
  const long long steps = (long long)prm->num_rounds * prm->sweeps_per_round;
  OS_REQUIRE(steps < (1ll << 31), "too many sweeps (%lld)", steps);
}

static void pt_create(PtRun &pr, os_ctx *ctx, const os_qubo_csr *q, const os_pt_params *prm) {
  check_pt_params(q, prm);
  const unsigned long long total = (unsigned long long)prm->num_chains * (unsigned long long)prm->num_temps;
  const long long steps = (long long)prm->num_rounds * prm->sweeps_per_round;
  os_sa_params sp{};
  sp.beta = prm->beta;
  sp.num_iter = prm->num_temps;
  sp.sweeps_per_beta = 1;
  sp.num_tries = (uint32_t)total;
  sp.seed = prm->seed;
  sp.acceptance = OS_ACCEPT_PHYSICAL;
  sp.site_order = OS_SITES_SEQUENTIAL;
  sp.resync_every = 0;
  sp.init_prob = nullptr;
  pr.p.kind = 1;
  os_sa_plan_common(&pr.p, ctx, &sp, q->n);
  plan_create_sparse(&pr.p, q);
  pr.p.steps = (int)steps;
  pr.chains = (int)prm->num_chains;
  pr.nt = prm->num_temps;
  pr.rounds = prm->num_rounds;
  pr.spr = prm->sweeps_per_round;
  pr.resync = prm->resync_every;
  pr.temp.alloc(total);
  pr.traj_at.alloc(total);
  pr.swaps.alloc(std::max(pr.nt - 1, 1));
  pr.efinal.alloc(total);
  for (auto &e : pr.ev) OS_CUDA(cudaEventCreate(&e));
}

static void pt_execute(PtRun &pr) {
  os_sa_plan *p = &pr.p;
  cudaStream_t s = p->ctx->stream;
  p->launches = 0;
  const int n = p->n, T = p->T;
  OS_CUDA(cudaMemsetAsync(pr.swaps.get(), 0, sizeof(unsigned long long) * pr.swaps.count, s));
  pt_identity_kernel<<<(T + 127) / 128, 128, 0, s>>>(pr.temp.get(), pr.traj_at.get(), T, pr.nt);
  OS_CUDA(cudaGetLastError());
  const SparseResyncArgs r = start_sparse(p);
  SparseArgs a = sweep_args(p, r);
  a.temp = pr.temp.get();
  ExchangeArgs x{};
  x.beta = p->beta.get();
  x.e = p->se.get();
  x.temp = pr.temp.get();
  x.traj_at = pr.traj_at.get();
  x.swaps = pr.swaps.get();
  x.chains = pr.chains;
  x.nt = pr.nt;
  x.rounds = 1;
  x.seed_lo = r.seed_lo;
  x.seed_hi = r.seed_hi;
  const int R = p->traj_per_cta;
  const int threads = p->warps * 32;
  const size_t smem = (size_t)n * 5 * R;
  const int grid = (T + R - 1) / R;
  OS_CUDA(cudaEventRecord(pr.ev[0], s));
  for (int round = 0; round < pr.rounds; ++round) {
    a.step_begin = round * pr.spr;
    a.step_end = a.step_begin + pr.spr;
    sa_sparse_kernel<kTemper><<<grid, threads, smem, s>>>(a);
    OS_CUDA(cudaGetLastError());
    ++p->launches;
    if (pr.nt > 1) {
      x.round0 = round;
      pt_exchange_kernel<<<exchange_blocks(pr.chains), 128, 0, s>>>(x);
      OS_CUDA(cudaGetLastError());
      ++p->launches;
    }
    // Same resync points as an anneal whose chunk is resync_every rounds.
    if ((pr.resync > 0 && (round + 1) % pr.resync == 0) || round + 1 == pr.rounds) {
      sa_sparse_resync_kernel<<<T, 256, 0, s>>>(r);
      OS_CUDA(cudaGetLastError());
      ++p->launches;
    }
  }
  OS_CUDA(cudaEventRecord(pr.ev[1], s));
  finish_sparse(p);
  sa_sparse_rescore_kernel<<<rescore_blocks(T), 256, 0, s>>>(p->row_ptr.get(), p->col.get(), p->val64.get(),
                                                           p->diag64.get(), n, T, p->sx.get(), pr.efinal.get());
  OS_CUDA(cudaGetLastError());
  ++p->launches;
}

static void pt_result(PtRun &pr, os_pt_result *res) {
  OS_REQUIRE(res != nullptr, "null result");
  os_sa_plan *p = &pr.p;
  OS_CUDA(cudaStreamSynchronize(p->ctx->stream));
  const int T = p->T, n = p->n;
  std::vector<double> e(T);
  OS_CUDA(cudaMemcpy(e.data(), p->e64.get(), sizeof(double) * T, cudaMemcpyDeviceToHost));
  std::vector<unsigned long long> acc(T);
  OS_CUDA(cudaMemcpy(acc.data(), p->accepted.get(), sizeof(unsigned long long) * T, cudaMemcpyDeviceToHost));
  unsigned long long drift_bits = 0;
  OS_CUDA(cudaMemcpy(&drift_bits, p->drift.get(), sizeof drift_bits, cudaMemcpyDeviceToHost));
  const int best = argmin_first(e);
  if (res->state) OS_CUDA(cudaMemcpy(res->state, p->states.get() + (size_t)best * n, n, cudaMemcpyDeviceToHost));
  res->energy = e[best];
  if (res->chain_energies)
    for (int c = 0; c < pr.chains; ++c) {
      double m = e[(size_t)c * pr.nt];
      for (int k = 1; k < pr.nt; ++k) m = std::min(m, e[(size_t)c * pr.nt + k]);
      res->chain_energies[c] = m;
    }
  if (res->final_temps)
    OS_CUDA(cudaMemcpy(res->final_temps, pr.temp.get(), sizeof(int) * T, cudaMemcpyDeviceToHost));
  if (res->final_energies)
    OS_CUDA(cudaMemcpy(res->final_energies, pr.efinal.get(), sizeof(double) * T, cudaMemcpyDeviceToHost));
  if (res->final_states) OS_CUDA(cudaMemcpy(res->final_states, p->sx.get(), (size_t)T * n, cudaMemcpyDeviceToHost));
  if (pr.nt > 1 && res->swaps_accepted)
    OS_CUDA(cudaMemcpy(res->swaps_accepted, pr.swaps.get(), sizeof(unsigned long long) * (pr.nt - 1),
                       cudaMemcpyDeviceToHost));
  if (res->swaps_attempted)
    for (int k = 0; k + 1 < pr.nt; ++k)  // rounds with round mod 2 == k mod 2
      res->swaps_attempted[k] = (unsigned long long)pr.chains * (unsigned long long)((pr.rounds + 1 - (k & 1)) / 2);
  double drift;
  std::memcpy(&drift, &drift_bits, sizeof drift);
  res->max_field_drift = drift;
  res->attempts = (unsigned long long)p->steps * (unsigned long long)n * (unsigned long long)T;
  unsigned long long total = 0;
  for (auto v : acc) total += v;
  res->accepted = total;
  float ms = 0.f;
  OS_CUDA(cudaEventElapsedTime(&ms, pr.ev[0], pr.ev[1]));
  res->device_ms = ms;
}

// ---------------------------------------------------------------------------
// Population annealing (Hukushima and Iba, AIP Conf. Proc. 690 (2003);
// Machta, PRE 82 (2010)). No counterpart in the reference, whose annealing
// benchmark names it beside parallel tempering as the next solver
// (benchmarks/annealing/performance.md:52-59). Between two inverse
// temperatures the population is resampled systematically (fixed size) in
// proportion to exp(-dbeta E); every replica then sweeps with the sparse
// annealing kernel.
// ---------------------------------------------------------------------------

constexpr int RESAMPLE_BLOCKS = 1024;  // blocks of the cumulative sums (part of the definition)
constexpr int RESAMPLE_CTA = 32;       // threads per CTA of the resampling kernels (one block each)

struct ResampleArgs {
  const double *e;     // [R] energies of the current population
  int R;
  double dbeta;
  int step;
  uint32_t seed_lo, seed_hi;
  double *cum;         // [R] scratch: running sums inside each block
  double *tot;         // [RESAMPLE_BLOCKS] scratch: block totals
  double *emin;        // [1] scratch: minimum energy
  int *parent;         // [R] out: parent of each slot
  double *logq;        // out: ln Q of the step
};

// Resampling, part 0: the population's minimum energy (one CTA).
__global__ void __launch_bounds__(1024) pa_min_kernel(const __grid_constant__ ResampleArgs a) {
  __shared__ double s_min[32];
  double m = INFINITY;
  for (int i = threadIdx.x; i < a.R; i += blockDim.x) m = fmin(m, a.e[i]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = s_min[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmin(r, s_min[w]);
    *a.emin = r;
  }
}

// Resampling, part 1: block b (thread b of the grid) covers replicas
// [b L, min((b+1) L, R)), L = ceil(R / 1024); its weights
// exp(-dbeta (E_i - E_min)) are summed in order into cum (running sums) and
// tot[b] (the block total). The work is spread over 32 CTAs because FP64
// exp is slow on one SM.
__global__ void __launch_bounds__(RESAMPLE_CTA) pa_weights_kernel(const __grid_constant__ ResampleArgs a) {
  const double emin = *a.emin;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = (a.R + RESAMPLE_BLOCKS - 1) / RESAMPLE_BLOCKS;
  const int b0 = b * L, b1 = min(a.R, b0 + L);
  double run = 0.0;
  for (int i = b0; i < b1; ++i) {
    run += exp(-a.dbeta * (a.e[i] - emin));
    a.cum[i] = run;
  }
  a.tot[b] = run;
}

// Slots j with (u + j) * stride < c: a prefix of 0 .. R (the targets grow
// with j), found from an estimate and corrected with the same comparisons a
// search over the targets would make.
__device__ __forceinline__ int slots_below(double c, double u, double stride, double inv_stride, int R) {
  const double q = c * inv_stride - u;
  int j = q <= 0.0 ? 0 : (q >= (double)R ? R : (int)ceil(q));
  while (j > 0 && (u + (j - 1)) * stride >= c) --j;
  while (j < R && (u + j) * stride < c) ++j;
  return j;
}

// Resampling, part 2. Offsets: the 1,024 block totals form 32 groups of 32;
// lane g of the first warp sums group g's totals in order (its exclusive
// prefixes are the in-group offsets), lane 0 sums the 32 group totals in order
// (the group offsets); offset = group offset + in-group offset and W = the
// sum of the group totals. Every CTA forms them (64 dependent adds) instead of
// waiting for another launch. Then replica i of block b, with cumulative sum
// C_i = offset_b + cum[i], owns the slots [slots_below(C_{i-1}),
// slots_below(C_i)) (the last replica also every slot above): the slot takes
// the first replica whose cumulative sum exceeds its target (u + j) W / R.
__global__ void __launch_bounds__(RESAMPLE_CTA) pa_assign_kernel(const __grid_constant__ ResampleArgs a) {
  __shared__ double s_pre[RESAMPLE_BLOCKS];
  __shared__ double s_goff[32];
  __shared__ double s_w;
  const int t = threadIdx.x;
  for (int k = t; k < RESAMPLE_BLOCKS; k += blockDim.x) s_pre[k] = a.tot[k];
  __syncthreads();
  if (t < 32) {
    double g = 0.0;
    for (int k = 0; k < 32; ++k) {
      const double v = s_pre[32 * t + k];
      s_pre[32 * t + k] = g;
      g += v;
    }
    s_goff[t] = g;
    __syncwarp();
    if (t == 0) {
      double acc = 0.0;
      for (int k = 0; k < 32; ++k) {
        const double v = s_goff[k];
        s_goff[k] = acc;
        acc += v;
      }
      s_w = acc;
    }
  }
  __syncthreads();
  const double W = s_w;
  if (blockIdx.x == 0 && t == 0) {
    const double emin_term = __dmul_rn(-a.dbeta, *a.emin);
    *a.logq = __dadd_rn(emin_term, log(W / a.R));
  }
  const int b = blockIdx.x * blockDim.x + t;
  const int L = (a.R + RESAMPLE_BLOCKS - 1) / RESAMPLE_BLOCKS;
  const int b0 = b * L, b1 = min(a.R, b0 + L);
  if (b0 >= b1) return;
  const Philox4 p = philox4x32_10((uint32_t)a.step, 0u, 0u, kStreamResample, a.seed_lo, a.seed_hi);
  const double u = u01_open64(p.x);
  const double stride = W / a.R, inv = a.R / W;
  const double off = s_goff[b >> 5] + s_pre[b];
  // The previous block's last cumulative sum is its offset plus its total
  // (its last running sum).
  int j = b == 0 ? 0 : slots_below(s_goff[(b - 1) >> 5] + s_pre[b - 1] + a.tot[b - 1], u, stride, inv, a.R);
  for (int i = b0; i < b1; ++i) {
    const int j1 = i == a.R - 1 ? a.R : slots_below(off + a.cum[i], u, stride, inv, a.R);
    for (; j < j1; ++j) a.parent[j] = i;
  }
}

static void launch_resample(const ResampleArgs &ra, cudaStream_t s) {
  const unsigned grid = RESAMPLE_BLOCKS / RESAMPLE_CTA;
  pa_min_kernel<<<1, 1024, 0, s>>>(ra);
  OS_CUDA(cudaGetLastError());
  pa_weights_kernel<<<grid, RESAMPLE_CTA, 0, s>>>(ra);
  OS_CUDA(cudaGetLastError());
  pa_assign_kernel<<<grid, RESAMPLE_CTA, 0, s>>>(ra);
  OS_CUDA(cudaGetLastError());
}

__global__ void iota_kernel(int *v, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) v[i] = i;
}

static void check_pa_params(const os_pa_params *prm) {
  OS_REQUIRE(prm != nullptr, "null parameters");
  OS_REQUIRE(prm->beta != nullptr && prm->num_steps >= 1, "empty beta schedule");
  for (int k = 0; k < prm->num_steps; ++k)
    OS_REQUIRE(std::isfinite(prm->beta[k]) && prm->beta[k] >= 0.0, "beta[%d] must be finite and >= 0", k);
  OS_REQUIRE(prm->sweeps_per_beta >= 1, "sweeps_per_beta must be positive");
  OS_REQUIRE(prm->population >= 1 && prm->population <= 65535, "population must be in 1 .. 65535");
  OS_REQUIRE(prm->resync_every >= 0, "resync_every must be >= 0");
  const long long steps = (long long)prm->num_steps * prm->sweeps_per_beta;
  OS_REQUIRE(steps < (1ll << 31), "too many sweeps (%lld)", steps);
}

struct PaRun {
  os_sa_plan p;                // sparse buffers of the current population; beta = the schedule
  int K = 0, spb = 0, resync = 0;
  std::vector<double> beta;    // host copy of the schedule
  os::DevBuf<float> h2;        // the other population (copy target)
  os::DevBuf<uint8_t> x2, xbest2;
  os::DevBuf<double> e2, ebest2, cum, tot, emin, logq, efinal;
  os::DevBuf<int> parent, anc, anc2;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~PaRun() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
};

template <class T> static void swap_buf(os::DevBuf<T> &a, os::DevBuf<T> &b) {
  std::swap(a.ptr, b.ptr);
  std::swap(a.count, b.count);
}

static void pa_create(PaRun &pr, os_ctx *ctx, const os_qubo_csr *q, const os_pa_params *prm) {
  OS_REQUIRE(q != nullptr, "null QUBO");
  check_pa_params(prm);
  os_sa_params sp{};
  sp.beta = prm->beta;
  sp.num_iter = prm->num_steps;
  sp.sweeps_per_beta = prm->sweeps_per_beta;
  sp.num_tries = prm->population;
  sp.seed = prm->seed;
  sp.acceptance = OS_ACCEPT_PHYSICAL;
  sp.site_order = OS_SITES_SEQUENTIAL;
  sp.resync_every = 0;
  sp.init_prob = nullptr;
  pr.p.kind = 1;
  os_sa_plan_common(&pr.p, ctx, &sp, q->n);
  plan_create_sparse(&pr.p, q);
  pr.K = prm->num_steps;
  pr.spb = prm->sweeps_per_beta;
  pr.resync = prm->resync_every;
  pr.beta.assign(prm->beta, prm->beta + prm->num_steps);
  const size_t R = prm->population, n = (size_t)q->n;
  pr.h2.alloc(R * n);
  pr.x2.alloc(R * n);
  pr.xbest2.alloc(R * n);
  pr.e2.alloc(R);
  pr.ebest2.alloc(R);
  pr.cum.alloc(R);
  pr.tot.alloc(RESAMPLE_BLOCKS);
  pr.emin.alloc(1);
  pr.logq.alloc(pr.K);
  pr.efinal.alloc(R);
  pr.parent.alloc(R);
  pr.anc.alloc(R);
  pr.anc2.alloc(R);
  for (auto &e : pr.ev) OS_CUDA(cudaEventCreate(&e));
}

static void pa_execute(PaRun &pr) {
  os_sa_plan *p = &pr.p;
  cudaStream_t s = p->ctx->stream;
  p->launches = 0;
  const int n = p->n, R = p->T;
  iota_kernel<<<(R + 127) / 128, 128, 0, s>>>(pr.anc.get(), R);
  OS_CUDA(cudaGetLastError());
  SparseResyncArgs r = start_sparse(p);
  p->launches += 1;
  ResampleArgs ra{};
  ra.R = R;
  ra.seed_lo = r.seed_lo;
  ra.seed_hi = r.seed_hi;
  ra.cum = pr.cum.get();
  ra.tot = pr.tot.get();
  ra.emin = pr.emin.get();
  ra.parent = pr.parent.get();
  const int cta_traj = p->traj_per_cta;
  const int threads = p->warps * 32;
  const size_t smem = (size_t)n * 5 * cta_traj;
  const int grid = (R + cta_traj - 1) / cta_traj;
  OS_CUDA(cudaEventRecord(pr.ev[0], s));
  for (int k = 0; k < pr.K; ++k) {
    ra.e = p->se.get();
    ra.dbeta = pr.beta[k] - (k ? pr.beta[k - 1] : 0.0);
    ra.step = k;
    ra.logq = pr.logq.get() + k;
    launch_resample(ra, s);
    // The sweep reads each slot's parent from the current buffers and
    // writes the new population into the other ones, which then swap.
    SparseArgs a = sweep_args(p, r);
    a.parent = pr.parent.get();
    a.h_in = p->sh.get();
    a.x_in = p->sx.get();
    a.xbest_in = p->sxbest.get();
    a.e_in = p->se.get();
    a.ebest_in = p->sebest.get();
    a.anc_in = pr.anc.get();
    a.h = pr.h2.get();
    a.x = pr.x2.get();
    a.xbest = pr.xbest2.get();
    a.e = pr.e2.get();
    a.ebest = pr.ebest2.get();
    a.anc = pr.anc2.get();
    a.step_begin = k * pr.spb;
    a.step_end = a.step_begin + pr.spb;
    sa_sparse_kernel<kPopulation><<<grid, threads, smem, s>>>(a);
    OS_CUDA(cudaGetLastError());
    swap_buf(p->sh, pr.h2);
    swap_buf(p->sx, pr.x2);
    swap_buf(p->sxbest, pr.xbest2);
    swap_buf(p->se, pr.e2);
    swap_buf(p->sebest, pr.ebest2);
    swap_buf(pr.anc, pr.anc2);
    r.h = p->sh.get();
    r.x = p->sx.get();
    r.xbest = p->sxbest.get();
    r.e = p->se.get();
    r.ebest = p->sebest.get();
    p->launches += 4;
    if ((pr.resync > 0 && (k + 1) % pr.resync == 0) || k + 1 == pr.K) {
      sa_sparse_resync_kernel<<<R, 256, 0, s>>>(r);
      OS_CUDA(cudaGetLastError());
      ++p->launches;
    }
  }
  OS_CUDA(cudaEventRecord(pr.ev[1], s));
  finish_sparse(p);
  sa_sparse_rescore_kernel<<<rescore_blocks(R), 256, 0, s>>>(p->row_ptr.get(), p->col.get(), p->val64.get(),
                                                           p->diag64.get(), n, R, p->sx.get(), pr.efinal.get());
  OS_CUDA(cudaGetLastError());
  ++p->launches;
}

static void pa_result(PaRun &pr, os_pa_result *res) {
  OS_REQUIRE(res != nullptr, "null result");
  os_sa_plan *p = &pr.p;
  OS_CUDA(cudaStreamSynchronize(p->ctx->stream));
  const int R = p->T, n = p->n;
  std::vector<double> e(R);
  OS_CUDA(cudaMemcpy(e.data(), p->e64.get(), sizeof(double) * R, cudaMemcpyDeviceToHost));
  std::vector<unsigned long long> acc(R);
  OS_CUDA(cudaMemcpy(acc.data(), p->accepted.get(), sizeof(unsigned long long) * R, cudaMemcpyDeviceToHost));
  unsigned long long drift_bits = 0;
  OS_CUDA(cudaMemcpy(&drift_bits, p->drift.get(), sizeof drift_bits, cudaMemcpyDeviceToHost));
  std::vector<int> anc(R);
  OS_CUDA(cudaMemcpy(anc.data(), pr.anc.get(), sizeof(int) * R, cudaMemcpyDeviceToHost));
  const int best = argmin_first(e);
  if (res->state) OS_CUDA(cudaMemcpy(res->state, p->states.get() + (size_t)best * n, n, cudaMemcpyDeviceToHost));
  res->energy = e[best];
  if (res->log_z) {
    std::vector<double> lq(pr.K);
    OS_CUDA(cudaMemcpy(lq.data(), pr.logq.get(), sizeof(double) * pr.K, cudaMemcpyDeviceToHost));
    double z = n * std::log(2.0);
    for (int k = 0; k < pr.K; ++k) res->log_z[k] = (z += lq[k]);
  }
  if (res->final_energies)
    OS_CUDA(cudaMemcpy(res->final_energies, pr.efinal.get(), sizeof(double) * R, cudaMemcpyDeviceToHost));
  if (res->final_states) OS_CUDA(cudaMemcpy(res->final_states, p->sx.get(), (size_t)R * n, cudaMemcpyDeviceToHost));
  std::sort(anc.begin(), anc.end());
  res->families = (uint32_t)(std::unique(anc.begin(), anc.end()) - anc.begin());
  double drift;
  std::memcpy(&drift, &drift_bits, sizeof drift);
  res->max_field_drift = drift;
  res->attempts = (unsigned long long)p->steps * (unsigned long long)n * (unsigned long long)R;
  unsigned long long total = 0;
  for (auto v : acc) total += v;
  res->accepted = total;
  float ms = 0.f;
  OS_CUDA(cudaEventElapsedTime(&ms, pr.ev[0], pr.ev[1]));
  res->device_ms = ms;
}

}  // namespace sa
}  // namespace os

using namespace os;
using namespace os::sa;

extern "C" {

os_status os_sa_plan_create_sparse(os_ctx *ctx, const os_qubo_csr *qubo, const os_sa_params *params,
                                   os_sa_plan **out) {
  return guard([&] {
    OS_REQUIRE(out != nullptr, "null output");
    check_schedule(params);
    OS_REQUIRE(params->resync_every >= 0, "resync_every = -1 (no resync) is for dense plans only");
    OS_REQUIRE(qubo != nullptr, "null QUBO");
    OS_REQUIRE(params->site_order == OS_SITES_SEQUENTIAL,
               "sparse annealing sweeps all sites per step (site_order must be SEQUENTIAL)");
    activate(ctx);
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


os_status os_pt_run_sparse(os_ctx *ctx, const os_qubo_csr *qubo, const os_pt_params *params,
                           os_pt_result *result) {
  return guard([&] {
    check_pt_params(qubo, params);
    OS_REQUIRE(result != nullptr, "null result");
    activate(ctx);
    PtRun pr;
    pt_create(pr, ctx, qubo, params);
    pt_execute(pr);
    pt_result(pr, result);
  });
}

os_status os_pt_exchange_replay(os_ctx *ctx, uint32_t num_chains, int32_t num_temps, const double *beta,
                                const double *energies, uint64_t seed, int32_t round0, int32_t num_rounds,
                                int32_t *temps, uint64_t *swaps_accepted) {
  return guard([&] {
    check_ladder(beta, num_temps);
    OS_REQUIRE(num_chains >= 1, "num_chains must be positive");
    OS_REQUIRE(round0 >= 0 && num_rounds >= 0, "rounds must be >= 0");
    OS_REQUIRE(energies != nullptr && temps != nullptr, "null argument");
    const size_t total = (size_t)num_chains * (size_t)num_temps;
    OS_REQUIRE(total <= (1u << 30), "too many replicas");
    std::vector<int> at(total, -1);
    for (size_t c = 0; c < num_chains; ++c)
      for (int r = 0; r < num_temps; ++r) {
        const int k = temps[c * num_temps + r];
        OS_REQUIRE(k >= 0 && k < num_temps && at[c * num_temps + k] < 0,
                   "temps of chain %zu is not a permutation", c);
        at[c * num_temps + k] = (int)(c * num_temps + r);
      }
    activate(ctx);
    cudaStream_t s = ctx->stream;
    DevBuf<double> b, e;
    DevBuf<int> t, ta;
    DevBuf<unsigned long long> sw;
    b.alloc(num_temps);
    e.alloc(total);
    t.alloc(total);
    ta.alloc(total);
    sw.alloc(std::max(num_temps - 1, 1));
    OS_CUDA(cudaMemcpyAsync(b.get(), beta, sizeof(double) * num_temps, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemcpyAsync(e.get(), energies, sizeof(double) * total, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemcpyAsync(t.get(), temps, sizeof(int) * total, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemcpyAsync(ta.get(), at.data(), sizeof(int) * total, cudaMemcpyHostToDevice, s));
    OS_CUDA(cudaMemsetAsync(sw.get(), 0, sizeof(unsigned long long) * sw.count, s));
    ExchangeArgs x{};
    x.beta = b.get();
    x.e = e.get();
    x.temp = t.get();
    x.traj_at = ta.get();
    x.swaps = sw.get();
    x.chains = (int)num_chains;
    x.nt = num_temps;
    x.round0 = round0;
    x.rounds = num_rounds;
    x.seed_lo = (uint32_t)seed;
    x.seed_hi = (uint32_t)(seed >> 32);
    if (num_rounds > 0) {
      pt_exchange_kernel<<<exchange_blocks(num_chains), 128, 0, s>>>(x);
      OS_CUDA(cudaGetLastError());
    }
    OS_CUDA(cudaMemcpyAsync(temps, t.get(), sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    if (swaps_accepted && num_temps > 1)
      OS_CUDA(cudaMemcpyAsync(swaps_accepted, sw.get(), sizeof(unsigned long long) * (num_temps - 1),
                              cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
  });
}


os_status os_pa_run_sparse(os_ctx *ctx, const os_qubo_csr *qubo, const os_pa_params *params,
                           os_pa_result *result) {
  return guard([&] {
    OS_REQUIRE(qubo != nullptr, "null QUBO");
    check_pa_params(params);
    OS_REQUIRE(result != nullptr, "null result");
    activate(ctx);
    PaRun pr;
    pa_create(pr, ctx, qubo, params);
    pa_execute(pr);
    pa_result(pr, result);
  });
}

os_status os_pa_resample_replay(os_ctx *ctx, uint32_t population, const double *energies, double dbeta,
                                uint64_t seed, int32_t step, int32_t *parents, double *log_q) {
  return guard([&] {
    OS_REQUIRE(energies && parents && log_q, "null argument");
    OS_REQUIRE(population >= 1 && population <= (1u << 24), "population must be in 1 .. 2^24");
    OS_REQUIRE(std::isfinite(dbeta), "dbeta must be finite");
    OS_REQUIRE(step >= 0, "step must be >= 0");
    for (uint32_t i = 0; i < population; ++i) OS_REQUIRE(std::isfinite(energies[i]), "energies[%u] not finite", i);
    activate(ctx);
    cudaStream_t s = ctx->stream;
    DevBuf<double> e, cum, tot, emin, lq;
    DevBuf<int> par;
    e.alloc(population);
    cum.alloc(population);
    tot.alloc(RESAMPLE_BLOCKS);
    emin.alloc(1);
    lq.alloc(1);
    par.alloc(population);
    OS_CUDA(cudaMemcpyAsync(e.get(), energies, sizeof(double) * population, cudaMemcpyHostToDevice, s));
    ResampleArgs ra{};
    ra.e = e.get();
    ra.R = (int)population;
    ra.dbeta = dbeta;
    ra.step = step;
    ra.seed_lo = (uint32_t)seed;
    ra.seed_hi = (uint32_t)(seed >> 32);
    ra.cum = cum.get();
    ra.tot = tot.get();
    ra.emin = emin.get();
    ra.parent = par.get();
    ra.logq = lq.get();
    launch_resample(ra, s);
    OS_CUDA(cudaMemcpyAsync(parents, par.get(), sizeof(int) * population, cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaMemcpyAsync(log_q, lq.get(), sizeof(double), cudaMemcpyDeviceToHost, s));
    OS_CUDA(cudaStreamSynchronize(s));
  });
}

}  // extern "C"
