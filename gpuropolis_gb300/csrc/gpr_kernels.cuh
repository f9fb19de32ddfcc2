/*
 * gpr_kernels.cuh -- launch parameters shared by the kernels (gpr_kernels.cu)
 * and the host library (gpr_capi.cu).
 */
#ifndef GPR_KERNELS_CUH
#define GPR_KERNELS_CUH

#include <stdint.h>
#include <cuda_runtime.h>

namespace gpr {

/* Exact 31-bit division by a run-time constant: x / d == (x * m) >> s for
 * every 0 <= x < 2^31 (Granlund-Montgomery, m = ceil(2^(31+l)/d), s = 31+l,
 * l = ceil(log2 d)). */
struct Magic {
    uint32_t m;
    uint32_t s;
};

/* Everything one launch of the MH block kernel needs.  Passed by value. */
struct KParams {
    /* chain state, reference layout (main.cu:387-389) */
    int32_t* P;
    float* C;
    double* prior;
    double* lik;
    int N;            /* chains                                              */
    int PL;           /* heap nodes per program (= NCONSTANTS)               */
    int steps;        /* MH steps this block (0 = evaluate only)             */
    uint32_t seed;    /* random_seed argument of MH_simple_kernel            */

    /* dataset, staged per CTA into shared memory; arrays padded to 4 floats */
    const float* dx;
    const float* dy;
    const float* dw;   /* 2^-64 / (2 sd^2) as float: weights at the bookkeeping scale */
    const float* dx2;  /* multivariate data: the second and third input variables */
    const float* dx3;
    int nv;            /* input variables: 1, or 3 for x1, x2, x3 (0 reads as 1) */
    /* batched data (nds > 0): dataset d is points [ds_off[d], ds_off[d] + ds_n[d])
     * of the arrays (offsets multiples of 4), with normalising sum ds_ns[2d],
     * ds_ns[2d+1] (2^-64 scale, double-float); chain c belongs to dataset
     * c / chains_per_ds; chain groups are claimed dataset by dataset in the
     * order ds_order (largest first); nd / nd_pad then give the largest */
    int nds;
    int chains_per_ds;
    const int* ds_off;
    const int* ds_n;
    const float* ds_ns;
    const int* ds_order;
    int nd;
    int nd_pad;        /* multiple of 4                                       */
    float normsum_hi, normsum_lo;  /* 2^-64 * sum_d 0.5*(logf(2 PIf) + 2 logf(sd_d)), double-float
                                    * (the Hamiltonian kernel's bookkeeping)  */
    /* The weights dw are 2^-e / (2 sd^2), e chosen per handle so that every
     * weight is at most 2^-32: the sum S of a chain's terms (f - y)^2 w then
     * cannot overflow FP32, chunk by chunk or in total.  The MH kernels keep
     * S as a double-float at that scale; the likelihood is -S 2^e - the
     * normalising sum, formed in FP64 only when a block's scores are written. */
    double lik_unscale;     /* 2^e                                            */
    int lik_e;              /* e                                              */
    float unscale1, unscale2;   /* 2^e as a product of two floats             */
    float w_to_df;          /* 2^(e-64): dw * w_to_df is the Hamiltonian kernel's 2^-64-scaled weight */
    double normsum64;       /* sum_d 0.5*(logf(2 PIf) + 2 logf(sd_d))          */
    const double* ds_ns64;  /* batched: the same per dataset                   */
    float ln1u_hi, ln1u_lo; /* log((double)NOPS + 1) as a double-float (main.cu:536) */
    float cauchy_c_hi, cauchy_c_lo;   /* PL * logf(PIf), the constant part of the
                                       * Cauchy prior (main.cu:304, 537-540), double-float */
    float* part;            /* chunk sums of the pipelined kernel when a dataset has more
                             * chunks than its shared-memory board holds      */
    int part_stride;        /* floats per (CTA, group, warp) in part          */

    /* proposals */
    int rng_mode;      /* 0 LCG, 1 Philox                                     */
    int const_mode;    /* 0 reference independence proposal, 1 random walk    */
    float rw_sd;
    int nops;
    int8_t opmap[32];  /* draw index -> op code                               */
    Magic mag_pl, mag_nops, mag_1e6;   /* divisors of random_int(n) (main.cu:220) */
    float ln1_hi, ln1_lo;  /* 2^-64 * log((double)NOPS + 1) (main.cu:536), double-float */

    /* float constants the reference computes with libm on the host side of
     * the oracle; the host library computes them the same way once */
    float lpi_f;       /* logf(PIf)                        lcauchypdf, main.cu:304 */
    float lnorm1_f;    /* 0.5*(logf(2 PIf) + 2 logf(1.0f)) lnormalpdf(.,1), main.cu:300 */
    float logf_r;      /* logf(PROPOSE_GEOM_R) as a float   lgeometricpdf, main.cu:308 */
    float log1mr_f;    /* log(1.0 - (double)PROPOSE_GEOM_R)                     */
    float log2_f;      /* log(2.0)                                              */
    float logpi_f;     /* log(PROPOSE_INT), float overload (logf)               */
    float log1mpi_f;   /* log(1.0 - (double)PROPOSE_INT)                        */
    float geom_logr;   /* gpr_rng_logf(PROPOSE_GEOM_R), random_geometric        */
    const float* logcount;  /* logf((float)k), k = 0..PL: Hastings term, main.cu:702,723 */

    /* work distribution and error reporting */
    int* next_chain;   /* dynamic chain counter (zeroed before launch)          */
    int* err;          /* device error flags                                    */
    unsigned long long* stats;  /* GPR_STAT_* counters, accumulated per launch  */
    int lockstep;      /* >0: the warps of a CTA realign every `lockstep` steps  */
    int stage_wait_iters;  /* polls of the dataset staging barrier before the kernel
                            * gives up with error flag 1 (default 2^22)          */
    int levels;        /* value-stack slots per lane                            */
    int max_instr;     /* instruction buffer length per program                 */

    /* move schedule and Hamiltonian constant moves */
    int struct_every;  /* a structure move every this many steps (main.cu:699: 5); 0 = never */
    float hmc_eps;     /* leapfrog step of the gradient constant moves          */
    int hmc_L;         /* leapfrog steps (1 = MALA)                             */
    float hmc_jit_eps; /* each move's step: hmc step x U(1 - j, 1 + j); 0 = fixed */
    float hmc_jit_len; /* each move's leapfrog count: uniform integer in
                        * [L(1 - j), L(1 + j)] (rounded, >= 1); 0 = fixed     */
    float* trace;      /* optional: C[0..trace_n) of each chain after each step,
                        * trace[(chain * steps + step) * trace_n + i]             */
    int trace_n;       /* <= 32 */
    int trace_chains;  /* only chains below this are traced                     */
    float* chain_scale;   /* optional: per-chain random-walk sd (const_mode 1) or
                           * leapfrog step (Hamiltonian moves), else rw_sd / hmc_eps */
    float adapt_target;   /* > 0: adapt chain_scale toward this acceptance rate
                           * during the block and write it back at its end */
    unsigned long long* phase;   /* instrumented kernels only: GPR_PH_SLOTS sums */

    /* the reference LCG (main.cu:215) advanced 2^b steps is the affine map
     * x -> lcgA[b]*x + lcgC[b] (mod 2^32, then masked to 31 bits) */
    uint32_t lcgA[20];
    uint32_t lcgC[20];
};

/* Fill p.lcgA / p.lcgC. */
void fill_lcg_jump_table(KParams& p);

/* Kernel entry points of the translation units gpr_mh_k*.cu. */
const void* mh_kernel_k4(int rng, int rolled);
const void* mh_kernel_k4m(int rng, int rolled);
const void* mh_kernel_k8(int rng, int rolled);
const void* mh_kernel_k8m(int rng, int rolled);
const void* mh_kernel_k4s(int rng, int rolled);   /* dataset streamed from device memory */
const void* mh_kernel_k4v(int rng, int rolled, int stream);   /* three input variables */
const void* mh_kernel_k4b(int rng, int rolled, int stream);    /* batched data */
const void* mh_kernel_k4bv(int rng, int rolled, int stream);   /* batched, three input variables */

/* Launch geometry picked by the host (persistent grid). */
struct LaunchCfg {
    int K;             /* points per lane per pass: 1, 2, 4 or 8                */
    int onepass;       /* nd <= 32*K: data kept in registers                    */
    int rolled;        /* heavy ops through the non-unrolled loop                */
    int lockstep;      /* CTA barrier period in MH steps (0: warps run freely)   */
    int warps_per_cta;
    int ctas;
    int pipe;          /* the pipelined kernel: two chains per warp, one barrier per half-step */
    size_t smem_bytes;
    int carveout;      /* shared-memory share of L1 in percent, 0 = the driver's choice */
    int stream;        /* dataset read from device memory, not staged per CTA   */
};

size_t mh_smem_bytes(const KParams& p, int K, int warps_per_cta, int stream = 0);
size_t pipe_smem_bytes(const KParams& p, int K, int warps_per_cta, int stream = 0);
/* Chunk-sum floats the pipelined kernel needs in p.part for nd points (0:
 * its shared-memory board suffices), per (CTA, group, warp). */
int pipe_part_stride(int nd);
const void* pipe_kernel_k4(int rng, int rolled, int onepass, int stream);
const void* pipe_kernel_k8(int rng, int rolled, int onepass);
const void* pipe_kernel_k4v(int rng, int rolled, int stream);
const void* pipe_kernel_k4b(int rng, int rolled, int stream, int nv);
cudaError_t launch_mh_block(const KParams& p, const LaunchCfg& lc, cudaStream_t st);
/* The phase-timed instantiation of the same layout (gpr_mh_prof.cu); p.phase
 * must point at GPR_PH_SLOTS zeroed counters.  Single dataset, one input
 * variable, LCG or Philox, heavy ops unrolled; other layouts are refused. */
cudaError_t launch_mh_block_prof(const KParams& p, const LaunchCfg& lc, cudaStream_t st);
const void* mh_kernel_prof(int K, int onepass, int rng, int stream);
const void* prof_kernel(const LaunchCfg& lc);   /* the LCG phase-timed build of lc, or nullptr */
cudaError_t mh_occupancy(const KParams& p, const LaunchCfg& lc, int* ctas_per_sm);

/* Diagnostics: evaluate every chain's program at nx points, and report the
 * compiled length / node count (used by the parity tests). */
cudaError_t launch_eval_values(const KParams& p, const float* xs, int nx, float* out,
                               float* length, int* count, cudaStream_t st);

cudaError_t launch_math(int op, const float* a, const float* b, float* out, int n, cudaStream_t st);
/* Times (ms) of the same adds on the current device: FP64 on all lanes, FP64
 * on one lane per warp, FP32 on all lanes. */
cudaError_t time_fp_adds(int iters, float* ms_d32, float* ms_d1, float* ms_f32);

/* Gradient of the log-likelihood and the MH kernel with Hamiltonian constant
 * moves (gpr_hmc.cu).  grad_smem_bytes: dynamic shared memory of either for
 * a CTA of warps_per_cta chains. */
size_t grad_smem_bytes(const KParams& p, int warps_per_cta, int stream = 0);
bool grad_supported(const KParams& p);   /* PROGRAM_LENGTH <= 127 */
cudaError_t launch_loglik_grad(const KParams& p, double* grad, double* lik, int stream, cudaStream_t st);
cudaError_t hmc_occupancy(const KParams& p, int warps_per_cta, size_t smem, int carveout, int stream,
                          int* ctas_per_sm);
cudaError_t launch_hmc_block(const KParams& p, const LaunchCfg& lc, cudaStream_t st);

/* Selection over the chains' posteriors (gpr_resample.cu).  launch_select
 * writes one order-preserving key per chain (gpr_select.h) into keys and,
 * for each of `segments` equal runs of chains, the key of ascending rank
 * `rank` within the run into out[segment].  launch_redraw re-draws every
 * chain whose posterior is below the cutoff -- the value of sel_key[chain /
 * seg_len] (seg_len 0: sel_key[0]), minus delta when map_delta -- from the
 * initial distribution, counting them in *n_redrawn.  launch_collect appends the chains with key >= kmin to out and
 * counts them; launch_first_index writes the smallest chain with key == k. */
cudaError_t launch_select(const KParams& p, int rank, unsigned long long* keys, unsigned long long* out,
                          cudaStream_t st, int segments = 1);
cudaError_t launch_redraw(const KParams& p, const unsigned long long* sel_key, int seg_len, int map_delta,
                          double delta, uint32_t seed, Magic mag_ops1, Magic mag_order, int* n_redrawn,
                          cudaStream_t st, uint32_t chain_offset = 0);
cudaError_t launch_collect(const unsigned long long* keys, int N, unsigned long long kmin, int* out, int cap,
                           int* count, cudaStream_t st);
cudaError_t launch_first_index(const unsigned long long* keys, int N, const unsigned long long* k, int* out,
                               cudaStream_t st);

}  // namespace gpr

#endif /* GPR_KERNELS_CUH */
