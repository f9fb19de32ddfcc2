/*
 * gpuropolis.h -- C ABI of the GB300 Metropolis-Hastings sampler over
 * arithmetic expressions (libgpuropolis.so).
 *
 * The reference has no library interface: its sampling loop lives in main()
 * (main.cu:1011-1257) and talks to one CUDA kernel,
 *     MH_simple_kernel(int N, op* P, data_t* C, datum* D, int ndata, int steps,
 *                      bayes_t* prior, bayes_t* likelihood, int random_seed)
 * (main.cu:679), launched once per block of steps (main.cu:1160), with
 * synchronous copies of the chain state either side (main.cu:1143-1147,
 * 1163-1167, 1233-1234).  Each entry point below replaces one of those steps;
 * the comment on each names the reference lines.  Plain pointers and sizes
 * only; every call returns a status code (GPR_OK == 0) and never exits the
 * process; gpr_last_error() describes the last failure of a handle.
 *
 * State layout (unchanged from the reference, main.cu:387-389):
 *   P[i*N + chain]  int32   op code of heap node i (0-based) of a chain
 *   C[i*N + chain]  float   constant of heap node i
 *   prior[chain], likelihood[chain]  double
 * Op codes use the reference numbering (main.cu:53): ONE=0, CONST=1, INV=2,
 * A=3, B=4, PLUS=5, MINUS=6, RMINUS=7, CPLUS=8, TIMES=9, CTIMES=10, DIV=11,
 * RDIV=12, LOG=13, EXP=14, POW=15, CPOW=16, RPOW=17, CRPOW=18, SQRT=19,
 * SIN=20, ASIN=21, COS=22, ACOS=23, TAN=24, ATAN=25, ABS=26.
 *
 * A handle is not thread-safe; all of its work runs on one CUDA stream.
 */
#ifndef GPUROPOLIS_H
#define GPUROPOLIS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GPR_OK = 0,
    GPR_ERR_ARG = 1,       /* invalid argument (size, pointer, option)       */
    GPR_ERR_CUDA = 2,      /* a CUDA call failed; see gpr_last_error         */
    GPR_ERR_STATE = 3,     /* call out of order (e.g. no data set)           */
    GPR_ERR_DEVICE = 4,    /* the kernel reported an error flag              */
    GPR_ERR_NOMEM = 5
};

enum { GPR_RNG_LCG = 0, GPR_RNG_PHILOX = 1 };
enum { GPR_CONST_REFERENCE = 0, GPR_CONST_RANDOM_WALK = 1, GPR_CONST_HMC = 2 };
/* Op codes beyond the reference's 27: the input variables of multivariate
 * data, printed X, Y, Z in op-code strings. */
enum { GPR_OP_X1 = 27, GPR_OP_X2 = 28, GPR_OP_X3 = 29 };

#define GPR_MAX_PROGRAM_LENGTH 255
#define GPR_MAX_OPS 32

typedef struct gpr_config {
    int program_length;      /* heap nodes per program (PROGRAM_LENGTH, main.cu:26); odd, 1..255 */
    int n_ops;               /* size of the op set drawn by proposals                         */
    int ops[GPR_MAX_OPS];    /* op codes of the set, in draw order (reference: 0..NOPS-1)     */
    int rng;                 /* GPR_RNG_LCG (main.cu:213-216) or GPR_RNG_PHILOX               */
    int const_proposal;      /* GPR_CONST_REFERENCE (main.cu:746-785), GPR_CONST_RANDOM_WALK or GPR_CONST_HMC */
    float rw_sd;             /* random-walk sd for GPR_CONST_RANDOM_WALK                      */
    int device;              /* CUDA device ordinal (--gpu, main.cu:104)                      */
    void* stream;            /* cudaStream_t to run on, or NULL to let the handle create one  */
    int n_vars;              /* input variables: 1 (the reference) or 3 (x1, x2, x3; 0 reads as 1) */
    int reserved[7];
} gpr_config;

typedef struct gpr_handle gpr_handle;

/* Fill *cfg with the reference's defaults: PROGRAM_LENGTH 31, the 27-op set
 * in enum order, LCG, independence constant proposals (main.cu:21-53). */
void gpr_default_config(gpr_config* cfg);

/* Create a sampler for n_chains chains (N, main.cu:97).  Allocates the device
 * state (replaces the DEVARRAY allocations, main.cu:1143-1147). */
int gpr_create(const gpr_config* cfg, int n_chains, gpr_handle** out);

/* Release everything the handle owns (main.cu:1251-1254). */
int gpr_destroy(gpr_handle* h);

/* Upload the dataset: n points of (x, y, sd), host arrays (the datum array D,
 * main.cu:48,1143).  sd must be > 0 (main.cu:332). */
int gpr_set_data(gpr_handle* h, const float* x, const float* y, const float* sd, int n);

/* Multivariate data (no reference counterpart): n points of (x1, x2, x3, y,
 * sd) for a handle created with n_vars = 3, whose op set may hold the leaf
 * ops GPR_OP_X1..GPR_OP_X3; a child beyond the heap reads x1. */
int gpr_set_data3(gpr_handle* h, const float* x1, const float* x2, const float* x3, const float* y,
                  const float* sd, int n);

/* Batched data (no reference counterpart; the reference runs one dataset per
 * process, main.cu:1143): n_datasets datasets in one launch, dataset d of
 * sizes[d] points, the points concatenated in dataset order in x1 (and x2,
 * x3 for three variables), y and sd.  The handle's chains split evenly:
 * chain c fits dataset c / (n_chains / n_datasets), so n_chains must be a
 * multiple of n_datasets.  Each chain's prior, likelihood and moves are
 * exactly those of a handle holding its dataset alone (gpr_set_data).
 * gpr_set_data / gpr_set_data3 return the handle to a single dataset. */
int gpr_set_batched_data(gpr_handle* h, int n_datasets, const int* sizes, const float* x1, const float* x2,
                         const float* x3, const float* y, const float* sd);

/* Captured block sequence (no reference counterpart; it replaces the host
 * loop's launches, main.cu:1156-1239): records n_blocks MH blocks of `steps`
 * steps each, with the handle's current data, layout and moves, as one CUDA
 * graph.  gpr_run_captured(h, seeds) enqueues a replay with seeds[0..n_blocks)
 * as the blocks' random seeds (set in the graph's kernel parameters before the
 * launch, so replays may be queued back to back), with the chains identical
 * to n_blocks gpr_run_block calls with those seeds.  Changing the data,
 * layout or moves drops the capture (GPR_ERR_STATE on replay). */
int gpr_capture_blocks(gpr_handle* h, int n_blocks, int steps);
int gpr_run_captured(gpr_handle* h, const int* seeds);

/* Upload chain state in the reference layout (main.cu:1144-1145, 1233-1234).
 * P holds program_length*N ints, C program_length*N floats (host memory). */
int gpr_set_state(gpr_handle* h, const int32_t* P, const float* C);

/* Upload prior and likelihood per chain (host arrays of N doubles; the
 * reference copies them to the device too, main.cu:1146-1147).  The MH kernel
 * recomputes both, so this matters only to the selection calls below on a
 * state the device has not scored. */
int gpr_set_scores(gpr_handle* h, const double* prior, const double* likelihood);

/* Download chain state (main.cu:1163-1166).  Any pointer may be NULL. */
int gpr_get_state(gpr_handle* h, int32_t* P, float* C, double* prior, double* likelihood);

/* Run `steps` Metropolis-Hastings steps on every chain, the block the
 * reference launches at main.cu:1160 with random_seed = host rand().  Queued on
 * the handle's stream; returns once queued (gpr_sync waits). */
int gpr_run_block(gpr_handle* h, int steps, int random_seed);

/* Recompute prior and likelihood of the current state without stepping
 * (compute_prior / compute_likelihood, main.cu:529-544, 454-468); results land
 * in the handle's device prior/likelihood arrays. */
int gpr_evaluate(gpr_handle* h);

/* Wait for the handle's stream; reports device-side error flags. */
int gpr_sync(gpr_handle* h);

/* Device pointers of the handle's state (for callers that keep data on the
 * GPU); valid until gpr_destroy. */
int gpr_device_state(gpr_handle* h, int32_t** P, float** C, double** prior, double** likelihood);

/* Kernel launches issued by this handle since creation (evidence counter). */
int64_t gpr_launch_count(gpr_handle* h);

/* Human-readable description of the last error on h (or, when h is NULL, of
 * the calling thread's last failed gpr_create or gpr_run_block_noalloc). */
const char* gpr_last_error(gpr_handle* h);

/* Library version string. */
const char* gpr_version(void);

/* ---- diagnostics (no reference counterpart; used by the parity tests) ---- */

/* Evaluate every chain's current program at nx points xs (host array) with
 * the device evaluator: out[chain*nx + i] = f_chain(xs[i]) (the reference's
 * call(), main.cu:446-448), plus the description length (main.cu:532) and
 * node count (main.cu:604-608) of each program. */
int gpr_debug_eval_values(gpr_handle* h, const float* xs, int nx, float* out, float* length,
                          int* count);

/* The evaluator's exp (op 0), log (op 1) and pow (op 2, second operand b)
 * applied elementwise to n host values (for accuracy tests against FP64). */
int gpr_debug_math(gpr_handle* h, int op, const float* a, const float* b, float* out, int n);

/* Run one block of `steps` MH steps (as gpr_run_block, same results) with the
 * phase-timed build of the handle's current layout, and copy min(n, 17)
 * counters to out: [0..14] clock64 cycles spent per phase, summed over the
 * warps (claim, load, step barrier, structure proposal, constant proposal,
 * compile, Cauchy prior, evaluation program, first barrier, ranking,
 * evaluation, second barrier, combine, accept, store), [15] evaluation
 * passes, [16] program instructions interpreted.  Only single-dataset,
 * one-variable, LCG handles whose layout has heavy ops unrolled are
 * instrumented; others return GPR_ERR_ARG. */
int gpr_debug_phase_profile(gpr_handle* h, int steps, int random_seed, uint64_t* out, int n);

/* The issue cost of FP64 against FP32 arithmetic on `device`: the times (ms)
 * of the same independent adds as FP64 on every lane, as FP64 on one lane per
 * warp, and as FP32 on every lane (8 CTAs of 256 threads per SM, iters x 4
 * adds per thread).  It is why the kernels keep FP64 out of their step loops. */
int gpr_debug_fp_issue(int device, int iters, float* ms_dadd32, float* ms_dadd1, float* ms_fadd32);

/* How many times the kernels poll the barrier of the bulk copy that stages
 * the dataset into a CTA's shared memory before giving up (default 2^22).  A
 * CTA that gives up sets error flag 1, waits (bounded) for its own copy to
 * land, and leaves: gpr_sync then returns GPR_ERR_DEVICE and the handle stays
 * usable.  0 makes every staged launch give up at once -- for testing that
 * path without a faulty GPU. */
int gpr_debug_stage_wait(gpr_handle* h, int polls);

/* Layout autotuner (no reference counterpart): times one block of `steps`
 * MH steps under each valid evaluation layout -- the pipelined kernel (two
 * chains per warp) or the lockstep one (one chain per warp), K = 4 or 8
 * points per lane, data held in registers (one pass), read from shared
 * memory in passes or streamed from device memory, transcendental/division
 * ops unrolled or (lockstep kernel) through a compact loop -- then, for the
 * best of those, the CTA size (8 or 4 warps) and, for the lockstep kernel,
 * the CTA barrier period (1, 5 steps, none), on the handle's current state and
 * data; keeps the fastest and restores the state, scores and counters.  Every
 * layout gives the same chains bit for bit, so the choice changes speed only.
 * Call after gpr_set_data/gpr_set_state. */
int gpr_autotune(gpr_handle* h, int steps, int seed, int* K, int* onepass, int* rolled, float* best_ms);

/* Select an evaluation layout explicitly (K 4 or 8; onepass needs n <= 32K)
 * on the lockstep kernel.  gpr_set_layout2 also sets the CTA barrier period
 * in MH steps (0 = none) and the warps (chains) per CTA (1, 2, 4 or 8);
 * gpr_set_layout3 also selects the pipelined kernel (pipe = 1: two chains per
 * warp, heavy ops unrolled, the barrier period unused). */
int gpr_set_layout(gpr_handle* h, int K, int onepass, int rolled);
int gpr_set_layout2(gpr_handle* h, int K, int onepass, int rolled, int lockstep, int warps_per_cta);
int gpr_set_layout3(gpr_handle* h, int K, int onepass, int rolled, int lockstep, int warps_per_cta, int pipe);

/* Read the dataset from device memory in every pass (always = 1) instead of
 * staging it into each CTA's shared memory; 0 (default) streams only when
 * staging does not fit, as for datasets of tens of thousands of points.
 * Results are identical either way.  gpr_layout_streamed reports the mode
 * of the current layout. */
int gpr_set_streaming(gpr_handle* h, int always);
int gpr_layout_streamed(gpr_handle* h);

/* Layout of a GPR_CONST_HMC handle's kernel: warps (chains) per CTA (1, 2, 4
 * or 8) and at most ctas_per_sm resident CTAs per SM (0: as many as fit).
 * Fewer CTAs leave more of each SM's L1 to the gradient tapes; gpr_autotune
 * times a set of these for GPR_CONST_HMC handles. */
int gpr_set_hmc_layout(gpr_handle* h, int warps_per_cta, int ctas_per_sm);

/* Launch geometry chosen for the current dataset: points per lane K, whether
 * the data stay in registers (onepass), warps per CTA, CTAs, shared bytes. */
int gpr_launch_geometry(gpr_handle* h, int* K, int* onepass, int* warps_per_cta, int* ctas,
                        int64_t* smem_bytes);

/* The cudaStream_t the handle runs on. */
void* gpr_stream(gpr_handle* h);

/* 1 when the current layout runs heavy ops through the compact loop; the
 * current CTA barrier period. */
int gpr_layout_rolled(gpr_handle* h);
int gpr_layout_lockstep(gpr_handle* h);
/* 1 when the current layout runs the pipelined kernel: two chains per warp,
 * the chains of a CTA in two groups taking turns (one group draws and
 * compiles its proposals while every warp evaluates the other group's), one
 * CTA barrier per half-step, the evaluation of a chain split over all warps. */
int gpr_layout_pipelined(gpr_handle* h);

/* Counters accumulated by the MH kernel since the last reset (no reference
 * counterpart): [0] likelihood evaluations, [1] sum of evaluated node counts,
 * [2] data points evaluated, [3] sum of (node count + 4) * points (the
 * algorithmic FP32 work), [4]/[5] structure moves proposed/accepted,
 * [6]/[7] constant moves proposed/accepted.  Copies min(n, 8) values. */
int gpr_get_stats(gpr_handle* h, uint64_t* out, int n);
int gpr_reset_stats(gpr_handle* h);

/* ---- gradients and Hamiltonian constant moves (no reference counterpart) ---- */

/* Move schedule: a structure move every struct_every steps (the reference:
 * 5, main.cu:699; 0: never, i.e. constants only) and, for GPR_CONST_HMC
 * handles, the leapfrog step hmc_eps and step count hmc_steps (1 = MALA) of
 * the Hamiltonian constant moves that take the place of the reference's
 * constant proposals.  Defaults: 5, 0.01, 8. */
int gpr_set_moves(gpr_handle* h, int struct_every, float hmc_eps, int hmc_steps);

/* Trajectory jitter of the Hamiltonian constant moves: each move draws its
 * leapfrog step as (the chain's) step x U(1 - eps_frac, 1 + eps_frac) and its
 * leapfrog count uniformly from the integers in [L(1 - len_frac), L(1 +
 * len_frac)] (rounded; at least 1), from a counter-based stream keyed by
 * (seed, chain, step).  Randomising the trajectory keeps detailed balance
 * and breaks the periodic orbits a fixed step x count can fall into on
 * strongly correlated posteriors.  Defaults: 0, 0 (fixed trajectories). */
int gpr_set_hmc_jitter(gpr_handle* h, float eps_frac, float len_frac);

/* Per-chain proposal scales: with target_accept in (0, 1), the following
 * blocks adapt each chain's own random-walk sd (GPR_CONST_RANDOM_WALK:
 * Robbins-Monro on log sd) or leapfrog step (GPR_CONST_HMC: dual averaging,
 * Hoffman and Gelman 2014) toward that acceptance rate of its constant moves;
 * 0 stops adapting and keeps the scales reached.  The first call gives every
 * chain the configured scale.  gpr_chain_scales copies the N scales out. */
int gpr_adapt_scales(gpr_handle* h, float target_accept);
int gpr_chain_scales(gpr_handle* h, float* out);

/* d log-likelihood / d C for every chain's current state (the likelihood of
 * main.cu:454-468 differentiated in each constant), by a reverse-mode
 * adjoint of the device evaluator (FP32 sums at the likelihood's 2^-64 scale,
 * so gradients beyond the FP32 range survive): grad[i*N + chain] (host,
 * program_length*N doubles; 0 for constants the program does not read) and,
 * when non-NULL, likelihood[chain].  Where an intermediate of the FP32 sweep
 * leaves the FP32 range, that chain's gradient comes out non-finite. */
int gpr_loglik_grad(gpr_handle* h, double* grad, double* likelihood);

/* gpr_run_block that also records, after every step, the first trace_n
 * constants of every chain: trace[(chain*steps + step)*trace_n + i] (host,
 * N*steps*trace_n floats).  For mixing measurements. */
int gpr_run_block_traced(gpr_handle* h, int steps, int random_seed, int trace_n, float* trace);

/* The same, recording only chains 0..n_chains-1 (all chains still step):
 * trace[(chain*steps + step)*trace_n + i], n_chains*steps*trace_n floats. */
int gpr_run_block_traced_first(gpr_handle* h, int steps, int random_seed, int trace_n, int n_chains,
                               float* trace);

/* ---- selection over the chains' posteriors, on the device ---- */

/* Resampling of the reference's outer loop (main.cu:1215-1231) without the
 * two full-state copies around it.  The cutoff is the posterior (prior +
 * likelihood of the last block) at ascending rank (int)(N * param) in the
 * order of the reference's comparator, NaN lowest (main.cu:987-995, 1219;
 * mode GPR_RESAMPLE_QUANTILE = 0, param 0.5 in the reference), or the largest
 * posterior minus param (mode GPR_RESAMPLE_MAP_DELTA = 1).  Every chain
 * strictly below it is re-drawn from the initial distribution, all ops then
 * all constants as main.cu:1224-1228 does: op = ops[random_int(n_ops - 1)],
 * constant = 10^(random_int(8) - 4) * random_normal().  The draws come from
 * the Philox stream keyed by (seed, chain | 2^31), not from the host's rand(),
 * so this is the device counterpart of gpr_host_resample, not a bit-exact
 * replacement.  Queued on the handle's stream; when n_redrawn or cutoff is
 * non-NULL the call waits and reports them.  Needs n_ops >= 2. */
int gpr_resample(gpr_handle* h, int mode, double param, uint32_t seed, int* n_redrawn, double* cutoff);

/* gpr_resample per dataset (batched data, gpr_set_batched_data): each
 * dataset's chains are resampled against the cutoff of their own posteriors,
 * the rank rule applied to the N / n_datasets chains of the dataset;
 * cutoffs (optional) receives one cutoff per dataset.  On a handle with one
 * dataset it is gpr_resample.  gpr_resample on batched data does the same
 * and reports a NaN cutoff.  gpr_top_chains and gpr_map_chain select over
 * all chains of the handle. */
int gpr_resample_datasets(gpr_handle* h, int mode, double param, uint32_t seed, int* n_redrawn,
                          double* cutoffs);

/* The re-draw of gpr_resample against a cutoff the caller supplies: every
 * chain whose posterior is strictly below `cutoff` is re-drawn, chain c from
 * the stream keyed by (seed, chain_offset + c).  For one population of chains
 * spread over several handles or GPUs: the cutoff is computed over the whole
 * population (the largest posterior minus delta, or the posterior at the
 * quantile's rank, reference comparator order), and each handle passes the
 * index of its first chain, so that the handles together re-draw exactly what
 * one handle holding every chain would (gpr_resample with that cutoff).  Waits
 * for the re-draw; *n_redrawn (optional) receives the count. */
int gpr_resample_below(gpr_handle* h, double cutoff, uint32_t seed, int chain_offset, int* n_redrawn);

/* Candidates for the k best chains: every chain whose posterior is >= the
 * k-th largest posterior minus margin (NaN never; all non-NaN chains when
 * fewer than k are non-NaN).  Up to `capacity` chain indices are written to
 * chains in ascending order, *n receives how many qualify (possibly more than
 * k, or than capacity) and *threshold the k-th largest posterior.  With a
 * margin above the rounding of the printed score this yields every line that
 * `sort -g -k3 samples.txt | tail -n k` (run-all.sh:45, tops.txt) can select
 * from one block. */
int gpr_top_chains(gpr_handle* h, int k, double margin, int* chains, int capacity, int* n, double* threshold);

/* The MAP chain: the smallest chain index with the largest posterior, and
 * that posterior (chain -1 when every posterior is NaN). */
int gpr_map_chain(gpr_handle* h, int* chain, double* posterior);

/* ---- running without allocating (no counterpart in the reference) ---- */

/* Largest dataset gpr_run_block_noalloc takes: its fixed device scratch holds
 * x, y and a weight for this many points (48 KB, plus 1.5 KB of tables). */
#define GPR_NOALLOC_MAX_POINTS 4096

/* Run `steps` MH steps (as gpr_run_block) on chains whose state the caller
 * keeps in its own device memory, allocating nothing: no handle, no device
 * memory, no host buffers.  It is for callers that must not allocate: a
 * process whose device memory belongs to another allocator's pool (a library
 * cudaMalloc beside that pool can fail, or fragment and shrink it), or a
 * loop that cannot pay for cudaMalloc/cudaFree, which may synchronise the
 * whole device.
 *
 * P, C (program_length * n_chains, the reference layout P[i*N + chain]; P must
 * hold valid op codes), prior and likelihood (n_chains doubles) are DEVICE
 * pointers, read and updated in place like the reference kernel's arguments
 * (main.cu:1160).  x, y, sd are HOST arrays of ndata points, sd > 0.  A
 * dataset of more than GPR_NOALLOC_MAX_POINTS points is rejected with
 * GPR_ERR_ARG before any device work; use gpr_create + gpr_set_data for it.
 * The results are those of gpr_create + gpr_set_data + gpr_set_state +
 * gpr_run_block with the default layout and the same seed.
 *
 * The dataset, the Hastings-term table and two counters (next chain, error
 * flags: both must be 0 when the kernel starts) live in one fixed scratch
 * array per device.  Each call writes all of them on its stream before its
 * launch, so the caller zeroes nothing.  Two calls that overlap on one device
 * (from other threads, or on other streams) share that array and race:
 * serialise them.  Runs on cfg->stream (NULL: the default stream), waits for
 * that stream to finish the block before returning, and reports kernel error
 * flags as gpr_sync does.  Every call looks up the scratch array's device
 * address with cudaGetSymbolAddress (which allocates nothing), so a context
 * reset between calls is harmless.  Because every call synchronises its
 * stream, no call can be made while a stream is being captured into a graph.
 * cfg->n_vars must be 0 or 1 (one input variable).  Failures are
 * described by gpr_last_error(NULL), per host thread. */
int gpr_run_block_noalloc(const gpr_config* cfg, int n_chains, int32_t* P, float* C,
                          double* prior, double* likelihood, const float* x, const float* y,
                          const float* sd, int ndata, int steps, int random_seed);

#ifdef __cplusplus
}
#endif

#endif /* GPUROPOLIS_H */
