/* onesolver.h -- C ABI of the GB300 (sm_103a) oneSolver backend.
 *
 * This is the drop-in boundary for oneSolver's two hot paths. The reference
 * (quantumz-io/oneSolver) has no FFI layer; its boundary is the C++ template
 * API plus two CLIs. Each entry point below names the reference function it
 * replaces (paths relative to the reference project root). The C++ mirror of
 * the reference API (include/onesolver/*.hpp: qubo::QUBOModel, sa::anneal,
 * exhaustive::solve, devices::construct_device_selector) is written on top of
 * these functions, and so are the CLIs.
 *
 * Conventions
 *   - Every function returns an os_status; no C++ exception crosses the ABI.
 *     On failure os_last_error() (thread-local) holds a human-readable reason.
 *   - The caller owns every host buffer. Device memory lives inside an
 *     os_ctx (or a plan created from one) and is freed with it.
 *   - Calls are synchronous unless the name says "execute" (those only
 *     enqueue work on the given stream).
 *   - A dense QUBO is the reference's flattened matrix
 *     (helpers::flatten_qubo, include/helpers/qubo_helpers.hpp:26-44):
 *     n*n doubles, row-major, diagonal = linear terms. Only the upper
 *     triangle (i <= j) is read, exactly as both reference energy functions
 *     read it (annealing.hpp:31-40, exhaustive.hpp:44-61), so a symmetric or
 *     an upper-triangular matrix gives the same result.
 *   - Exhaustive states are uint64 with bit i = variable i
 *     (helpers::ulong_to_vec, include/helpers/ulong_to_vec.hpp:23-32).
 */
#ifndef ONESOLVER_H_
#define ONESOLVER_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OS_ABI_VERSION 1

typedef enum os_status {
  OS_OK = 0,
  OS_INVALID_ARG = 1,          /* bad argument; reference: std::invalid_argument */
  OS_CUDA_ERROR = 2,           /* CUDA runtime error; reference: sycl::exception */
  OS_TIMEOUT = 3,              /* a bounded device wait ran out */
  OS_OVERFLOW_MINIMISERS = 4,  /* more minimisers than the caller's buffer holds */
  OS_NO_DEVICE = 5,            /* no CUDA device of the requested index */
  OS_PARSE_ERROR = 6,          /* .qubo text rejected (qubo.hpp:313-314,355-373,413-415) */
  OS_UNSUPPORTED = 7           /* e.g. --device-type host/cpu: this library has no CPU backend */
} os_status;

/* ------------------------------------------------------------------------ */
/* Library, errors, devices                                                 */
/* ------------------------------------------------------------------------ */

/* ABI version of the loaded library (OS_ABI_VERSION). No reference counterpart. */
int32_t os_abi_version(void);

/* Detail of the last failure on this thread. Reference: the what() string of
 * the exception thrown (annealing.hpp:128-132, qubo.hpp:313-415). */
const char *os_last_error(void);

/* Short name of a status code. */
const char *os_status_string(os_status status);

/* Device selection by the reference's --device-type string. Replaces
 * devices::construct_device_selector (include/helpers/devices.hpp:27-42):
 * "gpu" -> CUDA device 0; "cpu" and "host" -> OS_UNSUPPORTED (this library
 * has no CPU backend and never falls back to one); anything else ->
 * OS_INVALID_ARG with "Unknown device type: <s>". */
os_status os_select_device(const char *device_type, int32_t *device_out);

/* Device name for the CLIs' "Using device:" line
 * (app/one-solver-anneal.cpp:149-151). */
os_status os_device_name(int32_t device, char *buf, size_t cap);

/* Execution context: one CUDA device, one stream, cached device buffers.
 * Replaces the sycl::queue the reference passes to its solvers
 * (app/one-solver-anneal.cpp:139-147).
 * Every plan and network made on a context must be destroyed before the
 * context: their device buffers come from the context's stream-ordered
 * memory pool and are returned on its stream. os_ctx_destroy waits for the
 * context's stream before it releases the stream and the pool. */
typedef struct os_ctx os_ctx;
os_status os_ctx_create(int32_t device, os_ctx **out);
os_status os_ctx_destroy(os_ctx *ctx);
/* Use a caller-owned cudaStream_t (passed as void*) instead of the
 * context's own stream; NULL restores the context's stream. A plan's
 * destroy waits for the stream current at that moment and returns the
 * plan's buffers on the stream it was created on: a caller that executed a
 * plan on another stream waits for that stream (or makes it current again)
 * before destroying the plan. */
os_status os_ctx_set_stream(os_ctx *ctx, void *stream);

/* ------------------------------------------------------------------------ */
/* Model and file IO (host only; no GPU needed)                             */
/* ------------------------------------------------------------------------ */

/* Parsed QUBO model. Replaces qubo::QUBOModel<int,double> as produced by
 * QUBOModel::load (include/model/qubo.hpp:425-430) through parse_qubo
 * (qubo.hpp:392-417) and QUBOBuilder (qubo.hpp:282-379). */
typedef struct os_model os_model;

/* Parse .qubo text with the reference grammar and validation. Errors are
 * OS_PARSE_ERROR with the reference's message in os_last_error(). */
os_status os_model_parse(const char *text, size_t len, os_model **out);
os_status os_model_load_file(const char *path, os_model **out);
void os_model_free(os_model *model);

/* QUBOModel::get_nodes (qubo.hpp:177-180): max used index + 1. */
int64_t os_model_nodes(const os_model *model);
/* Number of stored linear / quadratic coefficients. */
int64_t os_model_num_linear(const os_model *model);
int64_t os_model_num_quadratic(const os_model *model);
/* QUBOModel::get_variable / get_connection (qubo.hpp:216-240): a missing
 * key reads as 0. */
double os_model_get_variable(const os_model *model, int32_t i);
double os_model_get_connection(const os_model *model, int32_t i, int32_t j);
/* helpers::flatten_qubo (qubo_helpers.hpp:26-44) into out[n*n]. */
os_status os_model_flatten(const os_model *model, double *out, size_t cap);
/* QUBOModel::str (qubo.hpp:182-202). Writes a NUL-terminated string;
 * *len_out gets the full length (excluding NUL). */
os_status os_model_str(const os_model *model, char *out, size_t cap, size_t *len_out);

/* Ising model in COO text ("i j bias" lines, 1-based variables, i == j a
 * linear bias, '#' comments) -> QUBO text in the format the reference's
 * converter writes (benchmarks/annealing/scripts/convert_qbsolv_to_coo.py:
 * "p qubo 0 N N C", then every (i, j) with i <= j sorted, 0-based):
 * Q_ii = 2 h_i - 2 sum_j J_ij, Q_ij = 4 J_ij, and *offset = sum J - sum h, so
 * that E_ising(s) = E_qubo(x) + offset with s = 2x - 1. Call with out = NULL
 * to learn the length (*len_out). */
os_status os_ising_to_qubo_text(const char *ising_text, size_t len, char *out, size_t cap, size_t *len_out,
                                double *offset);

/* qubo::Solution::save (include/model/solution.hpp:58-67): the two-line CSV
 * with the energy at 6 significant digits. */
os_status os_solution_csv(const char *state, int32_t n, double energy,
                          char *out, size_t cap, size_t *len_out);

/* ------------------------------------------------------------------------ */
/* Exhaustive search                                                        */
/* ------------------------------------------------------------------------ */

typedef struct os_qubo_dense {
  int32_t n;         /* number of variables */
  const double *f;   /* n*n flattened matrix (host), upper triangle read */
} os_qubo_dense;

typedef enum os_coef_kind {
  OS_COEF_AUTO = 0,     /* int32 if every coefficient is an integer and the
                           energy range fits, else int64, else fixed64 */
  OS_COEF_INT32 = 1,    /* exact int32 Gray-code enumeration */
  OS_COEF_INT64 = 2,    /* exact int64 Gray-code enumeration */
  OS_COEF_FIXED64 = 3   /* non-integer coefficients: int64 fixed-point
                           enumeration, then a candidate window re-scored in
                           FP64 in the reference's summation order */
} os_coef_kind;

typedef struct os_exh_params {
  int32_t coef_kind;        /* os_coef_kind */
  int32_t fixed_high_bits;  /* 0 = whole space; k > 0 fixes the top k bits */
  uint64_t prefix;          /* value of the fixed top bits (shard index) */
  uint64_t max_minimisers;  /* capacity of os_exh_result.states */
  int32_t inner_bits;       /* 0 = default (10); 9 or 10 sets how many low
                               bits the unrolled inner loop walks (tuning) */
  int32_t variant;          /* 0 = default (3 where it applies, else 2);
                               1 = three-input add + min per state;
                               2 = multiply-add + fused add-min;
                               3 = two states per three-input add in 16-bit
                               halves and a per-half minimum, for int32
                               coefficients whose magnitudes (upper
                               triangle) sum to at most 8,000 and
                               n - fixed_high_bits > inner_bits
                               (int32 only; every variant is exact) */
} os_exh_params;

typedef struct os_exh_result {
  double energy;              /* ground energy under the reference's FP64
                                 energy function (exhaustive.hpp:112-129) */
  uint64_t state;             /* smallest minimising state: the one the
                                 reference returns (exhaustive.hpp:130-133,158-166) */
  uint64_t count;             /* total number of degenerate minimisers */
  uint64_t *states;           /* caller buffer; min(count, max_minimisers)
                                 minimisers in ascending order (may be NULL
                                 when max_minimisers is 0) */
  uint64_t states_enumerated; /* 2^(n - fixed_high_bits) */
  int32_t coef_kind_used;     /* os_coef_kind actually run */
  int32_t collect_passes;     /* 1, or 2 when the degenerate set needed a
                                 second collection pass */
} os_exh_result;

/* Replaces exhaustive::solve (include/exhaustive/exhaustive.hpp:29-167).
 * Host buffers in and out; the call uploads the QUBO, enumerates all states
 * on the GPU, and returns the ground energy, the reference's minimiser and
 * the full degenerate set. n may be 1..50 (the reference's own limit is 30,
 * exhaustive.hpp:67 and ulong_to_vec.hpp:24-26). Returns
 * OS_OVERFLOW_MINIMISERS (with count and the first max_minimisers states
 * filled in) when the degenerate set is larger than the caller's buffer. */
os_status os_exhaustive_run(os_ctx *ctx, const os_qubo_dense *qubo,
                            const os_exh_params *params, os_exh_result *result);

/* The same search split into device-resident steps, for callers that keep
 * the problem on the GPU across calls (and for timing the kernels alone):
 * create uploads and prepares the problem, execute only enqueues the
 * enumeration kernels on the context's stream, result synchronises, runs a
 * second collection pass if the first overflowed, and copies the answer
 * back. No reference counterpart (the reference's solve is one call). */
typedef struct os_exh_plan os_exh_plan;
os_status os_exhaustive_plan_create(os_ctx *ctx, const os_qubo_dense *qubo,
                                    const os_exh_params *params,
                                    os_exh_plan **out);
os_status os_exhaustive_plan_execute(os_exh_plan *plan);
os_status os_exhaustive_plan_result(os_exh_plan *plan, os_exh_result *result);
/* Kernel launches made by the last execute (for launch accounting). */
int32_t os_exhaustive_plan_launches(const os_exh_plan *plan);
/* The instruction variant the plan's enumeration runs (os_exh_params.variant
 * after defaults: 1, 2 or 3; int64 and fixed-point searches report 1); 0
 * when the space is small enough for one thread per state. */
int32_t os_exhaustive_plan_variant(const os_exh_plan *plan);
/* Device time of the last execute's enumeration kernel, from CUDA events
 * recorded on the context's stream around it (waits for it to finish). */
os_status os_exhaustive_plan_kernel_ms(os_exh_plan *plan, float *ms);
void os_exhaustive_plan_destroy(os_exh_plan *plan);

/* Exhaustive search that allocates no device memory. No counterpart in the
 * reference. For callers that cannot call cudaMalloc: a process that reserves
 * the whole device memory for its own pool at start-up, or a latency-critical
 * path where cudaMalloc / cudaFree would synchronise the device and stall
 * other streams. All device scratch lives in one file-scope array of
 * OS_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until
 * the process exits; inputs and outputs are the caller's host buffers, as in
 * os_exhaustive_run, and the work runs on `stream` (a cudaStream_t, NULL =
 * the legacy default stream) of the current device.
 *   - Integer coefficients only (int32 or int64 enumeration); non-integer
 *     instances return OS_INVALID_ARG (use os_exhaustive_run).
 *   - n <= 50 and max_minimisers <= OS_NOALLOC_MAX_MINIMISERS; larger
 *     requests return OS_INVALID_ARG. inner_bits and variant are checked and
 *     honoured as os_exhaustive_run does.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) and keeps it for later calls.
 *   - Every call copies the answer back into the caller's host buffers and
 *     waits on `stream` for that before it returns.
 *   - Every call reuses the same array, so calls whose work overlaps on the
 *     GPU (other host threads, other streams) race; serialise them. */
#define OS_NOALLOC_SCRATCH_BYTES (3u << 20)
#define OS_NOALLOC_MAX_MINIMISERS 65536
os_status os_exhaustive_run_noalloc(const os_qubo_dense *qubo, const os_exh_params *params,
                                    os_exh_result *result, void *stream);

/* ------------------------------------------------------------------------ */
/* Simulated annealing                                                      */
/* ------------------------------------------------------------------------ */

typedef enum os_acceptance {
  OS_ACCEPT_REFERENCE = 0,  /* exp((E_cur - E_new) / beta) > u, as the
                               reference does (annealing.hpp:106-108) */
  OS_ACCEPT_PHYSICAL = 1    /* exp(-beta * (E_new - E_cur)) > u */
} os_acceptance;

typedef enum os_site_order {
  OS_SITES_RANDOM = 0,      /* one step = one attempt at a uniformly random
                               site (the reference, annealing.hpp:97-101) */
  OS_SITES_SEQUENTIAL = 1   /* one step = one sweep: an attempt at every
                               site in a fixed order (n attempts) */
} os_site_order;

typedef struct os_sa_params {
  const double *beta;       /* num_iter values (host); the schedule */
  int32_t num_iter;         /* schedule length (annealing.hpp:56-57) */
  int32_t sweeps_per_beta;  /* steps per beta value (annealing.hpp:58) */
  uint32_t num_tries;       /* independent trajectories (annealing.hpp:57) */
  uint64_t seed;            /* Philox key; replaces the fixed 1234 of
                               annealing.hpp:87 */
  int32_t acceptance;       /* os_acceptance */
  int32_t site_order;       /* os_site_order */
  int32_t resync_every;     /* steps between FP64 local-field resyncs
                               (0 = only one check at the end; -1 = none,
                               dense plans only: the drift is not measured
                               and max_field_drift reads -1) */
  const float *init_prob;   /* optional n values: P(x_i = 1) at start (warm
                               start); NULL = fair coin per spin as the
                               reference's bit() (annealing.hpp:91-93) */
} os_sa_params;

typedef struct os_sa_result {
  char *state;              /* [n] best state over all trajectories */
  double energy;            /* its energy, re-scored in FP64 with the
                               reference's energy function */
  double *traj_energies;    /* optional [num_tries]: FP64 re-scored best
                               energy of each trajectory */
  char *traj_states;        /* optional [num_tries * n] best states */
  double max_field_drift;   /* max |h_fp32 - h_fp64| over resyncs */
  uint64_t attempts;        /* spin-flip attempts performed */
  uint64_t accepted;        /* accepted flips */
} os_sa_result;

/* Replaces sa::anneal (include/simulated_annealing/annealing.hpp:55-140).
 * Dense QUBO, host buffers in and out. Trajectories run on the GPU with
 * FP32 local fields (FP64 resync), counter-based Philox randoms per
 * (trajectory, step, site), and the host-side argmin of annealing.hpp:134-139
 * (first minimum of the re-scored energies). */
os_status os_sa_run(os_ctx *ctx, const os_qubo_dense *qubo,
                    const os_sa_params *params, os_sa_result *result);

/* Sparse QUBO in CSR form: the off-diagonal couplings of row i are
 * col[row_ptr[i] .. row_ptr[i+1]) with values val (both triangles present,
 * i.e. the symmetric flattened matrix without its zeros), diag[i] = linear
 * term. */
typedef struct os_qubo_csr {
  int32_t n;
  const int32_t *row_ptr;   /* n+1 */
  const int32_t *col;       /* nnz */
  const double *val;        /* nnz */
  const double *diag;       /* n */
} os_qubo_csr;

/* sa::anneal on a sparse QUBO (e.g. Chimera droplet instances,
 * benchmarks/annealing/chimera_droplets_qbsolv): sites are coloured so that
 * no two sites of a colour are coupled, and one sweep updates the colours in
 * order, every site of a colour in parallel. This is the sequential sweep in
 * colour-sorted site order. Requires site_order = OS_SITES_SEQUENTIAL. */
os_status os_sa_run_sparse(os_ctx *ctx, const os_qubo_csr *qubo,
                           const os_sa_params *params, os_sa_result *result);

/* Many independent dense instances (uneven n <= 1792) annealed with one
 * shared schedule: every chunk of resync_every steps is one persistent
 * work-queue launch over (instance, block of trajectories) items, largest
 * instances first; the whole step sequence is captured once as a CUDA graph
 * and replayed; the number of trajectories per CTA is picked by timing probe
 * launches on the batch. num_tries trajectories per instance, sequential
 * sweeps only, random initial spins. results[k] receives instance k's
 * answer. No reference counterpart (the reference anneals one instance per
 * sa::anneal call, annealing.hpp:55-140). */
os_status os_sa_run_batched(os_ctx *ctx, int32_t num_instances,
                            const os_qubo_dense *instances,
                            const os_sa_params *params, os_sa_result *results);

/* The reference's kernel body (annealing.hpp:87-125) with caller-given
 * randoms, one GPU thread per trajectory with FP64 local fields: init[t*n+i]
 * replaces bit(), site[t*S+a] replaces bit_index() and u[t*S+a] replaces
 * uniform() for attempt a of trajectory t, S = num_iter * sweeps_per_beta.
 * One (site, u) pair is consumed per attempt whether or not u is needed.
 * For integer-valued coefficients the energies equal the reference's
 * per-attempt full recomputation exactly. This is a separate scalar kernel,
 * not the sweep kernels of os_sa_run; those are verified by the plans'
 * replay mode (os_sa_plan_set_replay). Outputs per trajectory: best state
 * and energy, final state and energy, accepted-flip count (any output
 * pointer may be NULL). */
os_status os_sa_verify(os_ctx *ctx, const os_qubo_dense *qubo,
                       const double *beta, int32_t num_iter,
                       int32_t sweeps_per_beta, uint32_t num_tries,
                       int32_t acceptance, const char *init,
                       const int32_t *site, const double *u,
                       char *best_states, double *best_energies,
                       char *final_states, double *final_energies,
                       int64_t *accept_count);

/* FP64 energies of m states under the reference's energy function
 * (annealing.hpp:31-40), computed on the GPU in the same summation order.
 * states is m*n chars (host), energies m doubles (host). */
os_status os_energy_batch(os_ctx *ctx, const os_qubo_dense *qubo,
                          const char *states, int32_t m, double *energies);

/* Device-resident SA plan (dense or sparse): create uploads the instance and
 * schedule, execute enqueues one whole anneal (all trajectories, all
 * steps) on the context's stream, result synchronises and copies the answer
 * back. No reference counterpart. */
typedef struct os_sa_plan os_sa_plan;
os_status os_sa_plan_create_dense(os_ctx *ctx, const os_qubo_dense *qubo,
                                  const os_sa_params *params, os_sa_plan **out);
os_status os_sa_plan_create_sparse(os_ctx *ctx, const os_qubo_csr *qubo,
                                   const os_sa_params *params, os_sa_plan **out);
/* Batched plan (see os_sa_run_batched); its answers come back through
 * os_sa_plan_result_batched, one os_sa_result per instance. */
os_status os_sa_plan_create_batched(os_ctx *ctx, int32_t num_instances,
                                    const os_qubo_dense *instances,
                                    const os_sa_params *params, os_sa_plan **out);
os_status os_sa_plan_result_batched(os_sa_plan *plan, os_sa_result *results);
/* Trajectories per CTA chosen by the batched plan's autotuner. */
int32_t os_sa_plan_tuned_warps(const os_sa_plan *plan);
os_status os_sa_plan_execute(os_sa_plan *plan);
os_status os_sa_plan_result(os_sa_plan *plan, os_sa_result *result);
int32_t os_sa_plan_launches(const os_sa_plan *plan);
/* Device time of the last execute's sweep kernels (sum over launches), from
 * CUDA events recorded on the context's stream around each of them. */
os_status os_sa_plan_kernel_ms(os_sa_plan *plan, float *ms);
void os_sa_plan_destroy(os_sa_plan *plan);

/* Replay (deterministic verification) mode of a dense, sparse or batched
 * plan. The reference draws its randoms from oneMKL's philox4x32x10
 * (annealing.hpp:87,91-93,101,108), which cannot be reproduced; in replay
 * mode the plan's next executes take them from the caller instead and run
 * everything else unchanged: the same sweep kernels (their replay
 * instantiation), visit order, field updates, energy and best-state
 * bookkeeping and FP64 resyncs. Replaces the randoms of annealing.hpp:
 *   init       initial spins, 0 / nonzero per variable (bit(), :91-93):
 *              [T][n]; batched plans: instance after instance, [T][n_k] each
 *   threshold  attempt at site k in step s of trajectory t accepts when
 *              dE < threshold (uniform() and the test of :106-108 in
 *              threshold form: -beta ln u for the reference rule,
 *              -ln(u) / beta for the physical rule). Sequential sweeps:
 *              [T][steps][n] indexed by site (batched: per instance, as init);
 *              random sites: [T][steps]
 *   site       random sites only: [T][steps], the site of each attempt
 *              (bit_index(), :101); NULL for sequential sweeps
 * steps = num_iter * sweeps_per_beta. NULL `replay` returns the plan to
 * Philox draws. */
typedef struct os_sa_replay {
  const char *init;
  const float *threshold;
  const int32_t *site;
} os_sa_replay;
os_status os_sa_plan_set_replay(os_sa_plan *plan, const os_sa_replay *replay);

/* Per-trajectory state after the last execute, for checking a replay (any
 * pointer may be NULL): final and best spins (bytes, [T][n]; batched:
 * instance after instance), the tracked energy of the final state and the
 * best tracked energy (the kernels' running energies, FP32 for dense and
 * batched plans, FP64 sums of FP32 differences for sparse plans, reset by
 * every FP64 resync), and the accepted flips. Best states are checked after
 * every accepted flip by the dense and batched kernels (annealing.hpp:
 * 115-121) and at the end of every sweep by the sparse kernel. */
os_status os_sa_plan_trajectories(os_sa_plan *plan, char *final_states, char *best_states,
                                  double *energies, double *best_energies, uint64_t *accepted);

/* The site order of one sequential sweep of the plan (n entries; batched:
 * each instance's n_k entries, instance after instance). Dense kernels visit
 * slot by slot (slot s = the 32 sites 128 (s / 4) + 4 l + s mod 4, lanes l
 * in order); the sparse kernel visits the colour classes in order, every
 * class in the listed order. OS_INVALID_ARG for random-site plans. */
os_status os_sa_plan_sweep_order(const os_sa_plan *plan, int32_t *order);

/* ------------------------------------------------------------------------ */
/* Parallel tempering (replica exchange)                                    */
/* ------------------------------------------------------------------------ */

/* No reference counterpart: the reference's annealing benchmark recommends
 * parallel tempering as the next solver after plain annealing
 * (benchmarks/annealing/performance.md:52-59), whose Chimera runs never reach
 * the tensor-network ground states (benchmarks/annealing/README:20-21).
 *
 * num_chains independent chains of num_temps replicas each. Replica
 * t = chain * num_temps + r starts at temperature index r from fair-coin
 * spins and keeps its spins; only temperature labels move. A round is
 * sweeps_per_round colour-parallel sweeps of every replica at its own
 * inverse temperature (physical rule exp(-beta dE) > u, FP32 local fields),
 * then one exchange attempt for every adjacent pair (k, k+1) with
 * k = round mod 2, k + 2, ... in every chain, accepted when
 * ln u < (beta[k+1] - beta[k]) * (E_cold - E_hot) with E_hot / E_cold the
 * tracked energies of the replicas at k / k+1 and u a Philox draw per
 * (pair, round, chain). */
typedef struct os_pt_params {
  const double *beta;        /* num_temps inverse temperatures (host),
                                finite, >= 0, non-decreasing */
  int32_t num_temps;         /* replicas per chain, >= 1 */
  uint32_t num_chains;       /* independent chains, >= 1 */
  int32_t num_rounds;        /* exchange rounds, >= 1 */
  int32_t sweeps_per_round;  /* sweeps of every replica per round, >= 1 */
  uint64_t seed;             /* Philox key (sweeps, initial spins, exchanges) */
  int32_t resync_every;      /* rounds between FP64 local-field resyncs
                                (0 = one check at the end) */
} os_pt_params;

typedef struct os_pt_result {
  char *state;               /* [n] best state any replica visited */
  double energy;             /* its FP64 energy (reference energy function) */
  double *chain_energies;    /* optional [num_chains]: best FP64 energy of
                                each chain */
  int32_t *final_temps;      /* optional [num_chains * num_temps]:
                                temperature index of each replica at the end */
  double *final_energies;    /* optional [num_chains * num_temps]: FP64
                                energy of each replica's final state */
  char *final_states;        /* optional [num_chains * num_temps * n] */
  uint64_t *swaps_accepted;  /* optional [num_temps - 1]: accepted exchanges
                                of each adjacent pair, summed over chains */
  uint64_t *swaps_attempted; /* optional [num_temps - 1] */
  double max_field_drift;    /* max |h_fp32 - h_fp64| over resyncs */
  uint64_t attempts;         /* spin-flip attempts performed */
  uint64_t accepted;         /* accepted flips */
  double device_ms;          /* device time of the rounds (sweeps, exchanges,
                                resyncs), CUDA events on the context's stream */
} os_pt_result;

/* Parallel tempering on a sparse QUBO (CSR as for os_sa_run_sparse), with
 * the sparse annealing kernel as the sweep; host buffers in and out. At most
 * 65535 replicas (num_chains * num_temps). */
os_status os_pt_run_sparse(os_ctx *ctx, const os_qubo_csr *qubo,
                           const os_pt_params *params, os_pt_result *result);

/* Exchange-only replay for verification: runs the exchange step of
 * os_pt_run_sparse on the GPU for rounds round0 .. round0 + num_rounds - 1
 * with every replica's energy held at energies[t] (no sweeps). temps
 * (num_chains * num_temps, in/out) gives each replica's temperature index
 * and must be a permutation of 0..num_temps-1 within every chain;
 * swaps_accepted (optional, num_temps - 1) receives the accepted exchanges
 * per pair. The same Philox draws as os_pt_run_sparse with that seed. */
os_status os_pt_exchange_replay(os_ctx *ctx, uint32_t num_chains, int32_t num_temps,
                                const double *beta, const double *energies,
                                uint64_t seed, int32_t round0, int32_t num_rounds,
                                int32_t *temps, uint64_t *swaps_accepted);

/* ------------------------------------------------------------------------ */
/* Population annealing                                                     */
/* ------------------------------------------------------------------------ */

/* No reference counterpart (benchmarks/annealing/performance.md:52-59 names
 * population annealing beside parallel tempering as the next solver).
 *
 * A population of `population` replicas starts from fair-coin spins (the
 * equilibrium at beta = 0). Step k (k = 0 .. num_steps-1) resamples the
 * population from beta[k-1] to beta[k] (beta[-1] = 0), then runs
 * sweeps_per_beta colour-parallel sweeps of every replica at beta[k]
 * (physical rule). Resampling is systematic: with weights
 * w_i = exp(-(beta[k] - beta[k-1]) (E_i - E_min)) and cumulative sums
 * C_i = w_0 + ... + w_i, slot j takes the replica i with C_{i-1} <= (u + j) W / R
 * < C_i (W = C_{R-1}, R = population, u one Philox draw per step), so the
 * population size is fixed. The cumulative sums are formed in 1024 blocks
 * of ceil(R / 1024) consecutive replicas: a running sum inside each block,
 * plus the block's offset (the block totals in 32 groups of 32, each group
 * summed in order, then the group totals in order). log_z[k] estimates
 * ln Z(beta[k]) = n ln 2 + sum_{m <= k} ln Q_m with
 * ln Q_m = -(beta[m] - beta[m-1]) E_min + ln(W / R) (Machta, PRE 82 (2010)). */
typedef struct os_pa_params {
  const double *beta;        /* num_steps inverse temperatures (host),
                                finite and >= 0 */
  int32_t num_steps;         /* >= 1 */
  int32_t sweeps_per_beta;   /* sweeps of every replica per step, >= 1 */
  uint32_t population;       /* replicas, 1 .. 65535 */
  uint64_t seed;             /* Philox key */
  int32_t resync_every;      /* steps between FP64 local-field resyncs
                                (0 = one check at the end) */
} os_pa_params;

typedef struct os_pa_result {
  char *state;               /* [n] best state any replica visited */
  double energy;             /* its FP64 energy (reference energy function) */
  double *log_z;             /* optional [num_steps]: ln Z estimates */
  double *final_energies;    /* optional [population]: FP64 energies of the
                                final population */
  char *final_states;        /* optional [population * n] */
  uint32_t families;         /* distinct initial replicas that still have
                                descendants at the end */
  double max_field_drift;    /* max |h_fp32 - h_fp64| over resyncs */
  uint64_t attempts;         /* spin-flip attempts performed */
  uint64_t accepted;         /* accepted flips */
  double device_ms;          /* device time of the steps (resampling,
                                copies, sweeps, resyncs), CUDA events */
} os_pa_result;

/* Population annealing on a sparse QUBO (CSR as for os_sa_run_sparse), with
 * the sparse annealing kernel as the sweep; host buffers in and out. */
os_status os_pa_run_sparse(os_ctx *ctx, const os_qubo_csr *qubo,
                           const os_pa_params *params, os_pa_result *result);

/* Resampling-only replay for verification: the resampling step of
 * os_pa_run_sparse for step `step` on caller-given energies[population]
 * with inverse-temperature increment dbeta. parents[population] receives
 * each slot's parent replica and *log_q the step's ln Q. Same Philox draw as
 * os_pa_run_sparse with that seed. */
os_status os_pa_resample_replay(os_ctx *ctx, uint32_t population, const double *energies,
                                double dbeta, uint64_t seed, int32_t step,
                                int32_t *parents, double *log_q);

/* Philox4x32-10 of the device generator, evaluated on the GPU for `count`
 * consecutive counters starting at ctr (ctr[0] incremented); out receives
 * 4*count words. For checking the generator against its published
 * definition. No reference counterpart. */
os_status os_philox_sample(os_ctx *ctx, const uint32_t ctr[4],
                           const uint32_t key[2], int32_t count,
                           uint32_t *out);

/* ------------------------------------------------------------------------ */
/* Learned warm start (no reference counterpart)                            */
/* ------------------------------------------------------------------------ */

/* A message-passing network over the coupling matrix that predicts per-spin
 * probabilities P(x_i = 1) for os_sa_params.init_prob. The reference always
 * starts from fair coins (annealing.hpp:91-93); plain random-init annealing
 * stays the fallback. Hidden width 64 (the kernels are built for it), 1..8
 * layers; BF16 products on the 5th-generation tensor cores (tcgen05.mma, FP32
 * accumulator in tensor memory) for the coupling-matrix messages, FP32
 * elsewhere; Adam on the GPU. With
 * orient = 1 labels are oriented so that spin 0 is 1 and predictions come
 * in that orientation (for field-free Ising QUBOs, which are symmetric under
 * the global flip); orient = 0 keeps labels as given. */
typedef struct os_mpnn os_mpnn;
os_status os_mpnn_create(os_ctx *ctx, int32_t hidden, int32_t layers, int32_t orient, uint64_t seed,
                         os_mpnn **out);
void os_mpnn_destroy(os_mpnn *model);
int64_t os_mpnn_num_params(const os_mpnn *model);
os_status os_mpnn_get_params(os_mpnn *model, float *out, size_t cap);
os_status os_mpnn_set_params(os_mpnn *model, const float *in, size_t count);
/* Stage an instance (and optionally its label state, n chars) on the GPU. */
os_status os_mpnn_add_instance(os_mpnn *model, const os_qubo_dense *qubo, const char *label, int32_t *index);
os_status os_mpnn_clear_instances(os_mpnn *model);
/* Mean BCE loss and its gradient (os_mpnn_num_params floats) for one stored
 * labelled instance at the current parameters. */
os_status os_mpnn_loss_grad(os_mpnn *model, int32_t index, float *loss, float *grads, size_t cap);
/* `epochs` passes of Adam (one step per labelled instance, shuffled). */
os_status os_mpnn_train(os_mpnn *model, int32_t epochs, float lr, uint64_t shuffle_seed, float *epoch_loss);
/* Per-spin P(x_i = 1) (n floats) for a new instance. */
os_status os_mpnn_predict(os_mpnn *model, const os_qubo_dense *qubo, float *prob);
/* The same prediction for a dense annealing plan's own instance, from the
 * matrix the plan already holds on the device, written straight into the
 * plan's initial-spin probabilities (as if os_sa_params.init_prob had been
 * given): no host copy either way and no synchronisation; it only enqueues
 * on the shared context's stream, before the plan's next execute. The plan
 * and the network must share a context. */
os_status os_sa_plan_warm_start(os_sa_plan *plan, os_mpnn *model);

/* Measured roofline denominators for the integer/FP32/shared-memory-bound
 * paths (the pool-wide measured peaks cover HBM copy bandwidth and bf16
 * GEMMs only): the INT32 issue rate of the enumeration's per-state instruction pair
 * (three-input add, integer min), in Gop/s; the FP32 FMA rate, in GFLOP/s;
 * and the shared-memory read rate of the annealing field update (128-bit
 * shared loads feeding paired FP32 FMAs), in GB/s. No reference counterpart. */
os_status os_probe_int32_peak(os_ctx *ctx, double *gops);
/* States per second of exhaustive variant `variant`'s own inner block walk
 * (1: three-input add + min; 2: multiply-add + fused add-min; 3: packed
 * 16-bit halves, a three-input add per two states and a three-input per-half
 * minimum per four), the enumeration kernel's instruction sequence run block
 * after block at full occupancy, with couplings that change between blocks as
 * they do in the enumeration: the ceiling of the enumeration's inner loop
 * without its per-item bookkeeping. */
os_status os_probe_exhaustive_pair(os_ctx *ctx, int32_t variant, double *states_per_s);
os_status os_probe_fp32_fma_peak(os_ctx *ctx, double *gflops);
os_status os_probe_smem_row_peak(os_ctx *ctx, double *gbs);

#ifdef __cplusplus
}
#endif

#endif /* ONESOLVER_H_ */
