/*
 * gpr_capi.cu -- the C ABI of include/gpuropolis.h: handle lifetime, device
 * state, dataset upload, launch geometry, error reporting.
 *
 * It owns what the reference's main() does around its kernel launch: the
 * device allocations and copies of P, C, D, prior, likelihood
 * (main.cu:1123-1147, 1163-1167, 1233-1234) and the launch itself
 * (main.cu:1160).  Nothing here calls exit(); every failure becomes a status
 * code and a message (the reference prints and continues, main.cu:162-168).
 */
#include <cuda_runtime.h>
#include <math.h>
#include <cmath>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <limits>
#include <new>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gpuropolis.h"
#include "gpr_common.h"
#include "gpr_kernels.cuh"
#include "gpr_rngmath.h"
#include "gpr_select.h"

#define GPR_VERSION_STRING "gpuropolis-gb300 0.1 (sm_103a)"

struct gpr_handle {
    gpr_config cfg;
    int N = 0;
    int PL = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;

    int32_t* dP = nullptr;
    float* dC = nullptr;
    double* dprior = nullptr;
    double* dlik = nullptr;
    float* dlogcount = nullptr;
    int* dcounter = nullptr;   /* [0] next chain, [1] error flags */
    unsigned long long* dstats = nullptr;
    float* ddata = nullptr;    /* x | y | w | sd, each nd_pad floats */
    /* selection scratch, allocated by the first gpr_resample/gpr_top_chains/gpr_map_chain */
    float* dscale = nullptr;               /* per-chain proposal scales          */
    float* dpart = nullptr;                /* chunk sums of the pipelined kernel for large datasets */
    size_t dpart_floats = 0;
    double* dds_ns64 = nullptr;            /* batched data: unscaled normalising sums */
    int stream_data = 0;                   /* 1: always stream the dataset       */
    int* dds = nullptr;                    /* batched data: off | n | order      */
    float* dds_ns = nullptr;               /* batched data: normalising sums     */
    /* a captured block sequence (gpr_capture_blocks): the graph, and per block
     * its kernel node with the node's launch parameters (the seed is set per
     * replay) */
    cudaGraph_t graph_src = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<cudaGraphNode_t> graph_nodes;
    std::vector<cudaKernelNodeParams> graph_params;
    std::vector<gpr::KParams> graph_kp;
    int graph_blocks = 0;
    unsigned long long* dkeys = nullptr;   /* N posterior keys                   */
    unsigned long long* dsel = nullptr;    /* [0] selected key (per dataset)     */
    int dsel_cap = 0;
    int* dseli = nullptr;                  /* [0] count, [1] first index         */
    int* dtop = nullptr;                   /* candidate chains, dtop_cap entries */
    int dtop_cap = 0;
    int nd = -1;
    int nd_pad = 0;
    double normsum = 0.0;

    gpr::KParams kp;
    gpr::LaunchCfg lc;
    int64_t launches = 0;
    std::string err;
};

/* An NVTX range over a C-ABI call, so that blocks, resampling and state
 * transfers show as named spans in Nsight timelines (almost free when no
 * tool is attached). */
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

/* Failures with no handle to hold them (gpr_create, gpr_run_block_noalloc):
 * one message per host thread, so that calls failing at once on different
 * threads do not race on it. */
static thread_local std::string g_create_error;

static int fail(gpr_handle* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h) h->err = buf; else g_create_error = buf;
    return code;
}

#define CUDA_TRY(h, call)                                                                     \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail((h), GPR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));  \
    } while (0)

static gpr::Magic magic_for(uint32_t d) {
    int l = 0;
    while ((1ull << l) < (unsigned long long)d) ++l;
    unsigned long long m = ((1ull << (31 + l)) + d - 1) / d;
    gpr::Magic r;
    r.m = (uint32_t)m;
    r.s = (uint32_t)(31 + l);
    return r;
}

/* Polls of the dataset staging barrier before a kernel reports a timeout. */
#define GPR_STAGE_WAIT_DEFAULT (1 << 22)

/* divisor of random_int(n), main.cu:220 */
static uint32_t divisor_for(int n) { return (uint32_t)(2147483647 / (n + 1)); }

/* The exponent e of the likelihood weights 2^-e / (2 sd^2): the largest is
 * at most 2^-32, so a term (at most FLT_MAX times its weight) is at most
 * 2^96 and the FP32 sum of up to 2^31 terms cannot overflow.  e is clamped to
 * [-100, 250] (2^e is then a product of two normal floats): datasets with an
 * sd below 1e-33 could overflow at the clamp.  The Hamiltonian kernel, which
 * keeps its own 2^-64 scale, holds weights up to sd of about 5e-30 only, as
 * it always has. */
static int weight_exponent(const float* sd, size_t n) {
    double maxw = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double s = (double)sd[i];
        const double w = 1.0 / (2.0 * s * s);
        if (w > maxw) maxw = w;
    }
    if (!(maxw > 0.0) || !std::isfinite(maxw)) return 0;
    int x = 0;
    frexp(maxw, &x);                    /* maxw <= 2^x */
    return std::min(250, std::max(-100, x + 32));
}

/* The per-point weight of a point with standard deviation sd. */
static float point_weight(float sd, int e) {
    const double s = (double)sd;
    return (float)(ldexp(1.0, -e) / (2.0 * s * s));
}

/* The scale fields of the kernel parameters for weight exponent e. */
static void set_weight_scale(gpr::KParams& kp, int e) {
    kp.lik_unscale = ldexp(1.0, e);
    kp.lik_e = e;
    const int e1 = std::min(127, std::max(-126, e));
    kp.unscale1 = (float)ldexp(1.0, e1);
    kp.unscale2 = (float)ldexp(1.0, e - e1);
    kp.w_to_df = (float)ldexp(1.0, e - 64);
}

/* The prior's constants as double-floats: log(NOPS + 1) (main.cu:536) and
 * PL logf(PIf), the constant part of the Cauchy sum (main.cu:304, 537-540). */
static void set_prior_constants(gpr::KParams& kp, int n_ops, int PL) {
    const double PIf = 3.141592653589;                             /* main.cu:194 */
    const double ln1 = log((double)n_ops + 1);
    kp.ln1u_hi = (float)ln1;
    kp.ln1u_lo = (float)(ln1 - (double)kp.ln1u_hi);
    const double cc = (double)PL * (double)logf((float)PIf);
    kp.cauchy_c_hi = (float)cc;
    kp.cauchy_c_lo = (float)(cc - (double)kp.cauchy_c_hi);
}

extern "C" {

void gpr_default_config(gpr_config* cfg) {
    if (!cfg) return;
    memset(cfg, 0, sizeof *cfg);
    cfg->program_length = 31;           /* PROGRAM_LENGTH, main.cu:26 */
    cfg->n_ops = OP_NREF;               /* NOPS, main.cu:53 */
    for (int i = 0; i < OP_NREF; ++i) cfg->ops[i] = i;
    cfg->rng = GPR_RNG_LCG;
    cfg->const_proposal = GPR_CONST_REFERENCE;
    cfg->rw_sd = 0.1f;
    cfg->n_vars = 1;
    cfg->device = 0;
    cfg->stream = nullptr;
}

const char* gpr_version(void) { return GPR_VERSION_STRING; }

const char* gpr_last_error(gpr_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int64_t gpr_launch_count(gpr_handle* h) { return h ? h->launches : 0; }

static void free_all(gpr_handle* h) {
    cudaFree(h->dP); cudaFree(h->dC); cudaFree(h->dprior); cudaFree(h->dlik);
    cudaFree(h->dlogcount); cudaFree(h->dcounter); cudaFree(h->ddata); cudaFree(h->dstats);
    cudaFree(h->dkeys); cudaFree(h->dsel); cudaFree(h->dseli); cudaFree(h->dtop); cudaFree(h->dscale);
    cudaFree(h->dds); cudaFree(h->dds_ns); cudaFree(h->dds_ns64); cudaFree(h->dpart);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->graph_src) cudaGraphDestroy(h->graph_src);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

int gpr_create(const gpr_config* cfg, int n_chains, gpr_handle** out) {
    if (!out) return fail(nullptr, GPR_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!cfg) return fail(nullptr, GPR_ERR_ARG, "cfg is NULL");
    if (n_chains <= 0) return fail(nullptr, GPR_ERR_ARG, "n_chains must be > 0 (got %d)", n_chains);
    const int PL = cfg->program_length;
    if (PL < 1 || PL > GPR_MAX_PROGRAM_LENGTH || (PL % 2) == 0)
        return fail(nullptr, GPR_ERR_ARG, "program_length must be odd and in [1, %d] (got %d)",
                    GPR_MAX_PROGRAM_LENGTH, PL);
    if (cfg->n_ops < 1 || cfg->n_ops > GPR_MAX_OPS)
        return fail(nullptr, GPR_ERR_ARG, "n_ops must be in [1, %d] (got %d)", GPR_MAX_OPS, cfg->n_ops);
    const int nv = cfg->n_vars == 0 ? 1 : cfg->n_vars;
    if (nv != 1 && nv != 3) return fail(nullptr, GPR_ERR_ARG, "n_vars must be 1 or 3 (got %d)", cfg->n_vars);
    for (int i = 0; i < cfg->n_ops; ++i) {
        const int o = cfg->ops[i];
        if (o < 0 || o >= OP_NALL)
            return fail(nullptr, GPR_ERR_ARG, "ops[%d] = %d is not an op code", i, o);
        if ((o == OP_X2 || o == OP_X3) && nv != 3)
            return fail(nullptr, GPR_ERR_ARG, "ops[%d] = %d reads x2/x3, which needs n_vars = 3", i, o);
    }
    if (cfg->rng != GPR_RNG_LCG && cfg->rng != GPR_RNG_PHILOX)
        return fail(nullptr, GPR_ERR_ARG, "unknown rng mode %d", cfg->rng);
    if (cfg->const_proposal != GPR_CONST_REFERENCE && cfg->const_proposal != GPR_CONST_RANDOM_WALK &&
        cfg->const_proposal != GPR_CONST_HMC)
        return fail(nullptr, GPR_ERR_ARG, "unknown constant proposal %d", cfg->const_proposal);
    if ((long long)n_chains * PL > (1ll << 31) - 1)
        return fail(nullptr, GPR_ERR_ARG, "n_chains * program_length exceeds 2^31-1");

    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return fail(nullptr, GPR_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
    if (cfg->device < 0 || cfg->device >= ndev)
        return fail(nullptr, GPR_ERR_ARG, "invalid GPU device %d (%d present)", cfg->device, ndev);

    gpr_handle* h = new gpr_handle();
    h->cfg = *cfg;
    h->N = n_chains;
    h->PL = PL;
    h->device = cfg->device;
    auto bail = [&](int code) { free_all(h); std::string m = h->err; delete h; g_create_error = m; return code; };
#define CREATE_TRY(call)                                                                       \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            fail(h, GPR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));            \
            return bail(GPR_ERR_CUDA);                                                         \
        }                                                                                      \
    } while (0)
    CREATE_TRY(cudaSetDevice(h->device));
    CREATE_TRY(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
    if (cfg->stream) {
        h->stream = (cudaStream_t)cfg->stream;
    } else {
        CREATE_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    const size_t n = (size_t)n_chains;
    CREATE_TRY(cudaMalloc(&h->dP, n * PL * sizeof(int32_t)));
    CREATE_TRY(cudaMalloc(&h->dC, n * PL * sizeof(float)));
    CREATE_TRY(cudaMalloc(&h->dprior, n * sizeof(double)));
    CREATE_TRY(cudaMalloc(&h->dlik, n * sizeof(double)));
    CREATE_TRY(cudaMalloc(&h->dlogcount, (PL + 2) * sizeof(float)));
    CREATE_TRY(cudaMalloc(&h->dcounter, 2 * sizeof(int)));
    CREATE_TRY(cudaMalloc(&h->dstats, GPR_NSTATS * sizeof(unsigned long long)));
    CREATE_TRY(cudaMemsetAsync(h->dstats, 0, GPR_NSTATS * sizeof(unsigned long long), h->stream));
    CREATE_TRY(cudaMemsetAsync(h->dP, 0, n * PL * sizeof(int32_t), h->stream));
    CREATE_TRY(cudaMemsetAsync(h->dC, 0, n * PL * sizeof(float), h->stream));
    CREATE_TRY(cudaMemsetAsync(h->dprior, 0, n * sizeof(double), h->stream));
    CREATE_TRY(cudaMemsetAsync(h->dlik, 0, n * sizeof(double), h->stream));
    CREATE_TRY(cudaMemsetAsync(h->dcounter, 0, 2 * sizeof(int), h->stream));

    /* Hastings term table: logf((float)k) (main.cu:702,723) */
    std::vector<float> lc(PL + 2);
    for (int k = 0; k < PL + 2; ++k) lc[k] = logf((float)k);
    CREATE_TRY(cudaMemcpyAsync(h->dlogcount, lc.data(), lc.size() * sizeof(float),
                               cudaMemcpyHostToDevice, h->stream));
    CREATE_TRY(cudaStreamSynchronize(h->stream));

    gpr::KParams& kp = h->kp;
    memset(&kp, 0, sizeof kp);
    kp.P = h->dP; kp.C = h->dC; kp.prior = h->dprior; kp.lik = h->dlik;
    kp.N = n_chains; kp.PL = PL;
    kp.nv = nv;
    kp.rng_mode = cfg->rng;
    kp.const_mode = cfg->const_proposal;
    kp.rw_sd = cfg->rw_sd;
    kp.nops = cfg->n_ops;
    for (int i = 0; i < cfg->n_ops; ++i) kp.opmap[i] = (int8_t)cfg->ops[i];
    kp.mag_pl = magic_for(divisor_for(PL));
    kp.mag_nops = magic_for(divisor_for(cfg->n_ops));
    kp.mag_1e6 = magic_for(divisor_for(1000000));
    {
        const double ln1 = log((double)cfg->n_ops + 1) * 0x1p-64;   /* main.cu:536, scaled */
        kp.ln1_hi = (float)ln1;
        kp.ln1_lo = (float)(ln1 - (double)kp.ln1_hi);
    }
    const double PIf = 3.141592653589;                             /* main.cu:194 */
    kp.lpi_f = logf((float)PIf);                                   /* main.cu:304 */
    kp.lnorm1_f = (float)(0.5 * ((double)logf((float)(2.0 * PIf)) + 2.0 * (double)logf(1.0f)));
    const float R = 0.1f, PI_INT = 0.15f;                          /* main.cu:32,34 */
    kp.logf_r = logf(R);
    kp.log1mr_f = (float)log(1.0 - (double)R);
    kp.log2_f = (float)log(2.0);
    kp.logpi_f = logf(PI_INT);                 /* log(PROPOSE_INT) binds to the float overload */
    kp.log1mpi_f = (float)log(1.0 - (double)PI_INT);
    kp.geom_logr = gpr_rng_logf(R);
    set_prior_constants(kp, cfg->n_ops, PL);
    set_weight_scale(kp, 0);
    kp.logcount = h->dlogcount;
    kp.next_chain = h->dcounter;
    kp.err = h->dcounter + 1;
    kp.stats = h->dstats;
    kp.lockstep = 1;
    kp.stage_wait_iters = GPR_STAGE_WAIT_DEFAULT;
    kp.struct_every = 5;                                           /* main.cu:699 */
    kp.hmc_eps = 0.01f;
    kp.hmc_L = 8;
    kp.hmc_jit_eps = 0.0f;
    kp.hmc_jit_len = 0.0f;
    kp.max_instr = GPR_MAX_INSTR(PL);
    /* Value-stack depth: a push happens at a binary node whose children are
     * both subtrees, so at a node j <= PL/2; pending pushes lie on one
     * root-to-node path, at most floor(log2(PL/2)) + 1 of them. */
    int lev = 1;
    while ((1 << lev) <= PL / 2) ++lev;
    kp.levels = lev;
    gpr::fill_lcg_jump_table(kp);
    *out = h;
    return GPR_OK;
#undef CREATE_TRY
}

int gpr_destroy(gpr_handle* h) {
    if (!h) return GPR_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return GPR_OK;
}

/* The handle has no dataset until a new one is fully uploaded: a failure
 * while replacing the data leaves no pointer to freed device memory behind
 * (gpr_run_block then reports that no data were set). */
static void forget_data(gpr_handle* h) {
    h->nd = -1;
    h->nd_pad = 0;
    gpr::KParams& kp = h->kp;
    kp.nd = 0; kp.nd_pad = 0; kp.nds = 0;
    kp.dx = kp.dy = kp.dw = kp.dx2 = kp.dx3 = nullptr;
    kp.ds_off = kp.ds_n = kp.ds_order = nullptr;
    kp.ds_ns = nullptr;
    kp.ds_ns64 = nullptr;
}

/* A captured block sequence bakes the launch parameters in: any change of
 * data, layout or moves drops it. */
static void drop_graph(gpr_handle* h) {
    if (h->graph) { cudaStreamSynchronize(h->stream); cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    if (h->graph_src) { cudaGraphDestroy(h->graph_src); h->graph_src = nullptr; }
    h->graph_nodes.clear(); h->graph_params.clear(); h->graph_kp.clear();
    h->graph_blocks = 0;
}

/* Largest CTA size (warps) whose chain group (one chain per warp, two for
 * the pipelined kernel) divides the chains of one dataset, so that a group
 * never straddles two datasets. */
static int batched_wpc(const gpr::KParams& kp, int wpc, int pipe = 0) {
    if (kp.nds <= 0) return wpc;
    const int per = pipe ? 2 : 1;
    while (wpc > 1 && kp.chains_per_ds % (per * wpc)) wpc /= 2;
    return wpc;
}

/* The MH kernel with Hamiltonian constant moves: one chain per warp,
 * wpc0 warps per CTA, four points per lane per pass, a persistent grid of at
 * most ctas_per_sm CTAs per SM (0: as many as fit).  Capping the CTAs also
 * caps the shared-memory carveout, which leaves the rest of the SM's L1 to
 * the thread-local gradient tapes. */
static int configure_hmc(gpr_handle* h, int wpc0 = 4, int ctas_per_sm = 0, int stream_mode = -1) {
    if (wpc0 < 1 || wpc0 > 8) wpc0 = 4;
    drop_graph(h);
    gpr::KParams& kp = h->kp;
    if (!gpr::grad_supported(kp))
        return fail(h, GPR_ERR_ARG, "gradient moves support program_length <= 127 (got %d)", kp.PL);
    gpr::LaunchCfg lc;
    lc.K = 4; lc.onepass = 0; lc.rolled = 0; lc.lockstep = 0; lc.carveout = 0;
    /* Streamed when asked, for batched data (each warp reads its own chain's
     * dataset from device memory), when staging does not fit, and when the
     * staged copy would take over a quarter of the CTA's shared memory: the
     * memory it frees goes to L1, which holds the gradient tapes (on the
     * 1024-point rational model streaming measured 23% faster). */
    const size_t staged = gpr::grad_smem_bytes(kp, wpc0, 0), streamed = gpr::grad_smem_bytes(kp, wpc0, 1);
    lc.stream = h->stream_data || kp.nds > 0 || staged > 227 * 1024 ||
                (stream_mode < 0 ? 4 * (staged - streamed) > staged : stream_mode > 0);
    int wpc = wpc0;
    size_t smem = gpr::grad_smem_bytes(kp, wpc, lc.stream);
    while (smem > 227 * 1024 && wpc > 1) smem = gpr::grad_smem_bytes(kp, wpc /= 2, lc.stream);
    if (smem > 227 * 1024)
        return fail(h, GPR_ERR_ARG, "programs of length %d do not fit in shared memory", kp.PL);
    if (ctas_per_sm > 0) {
        int sm_smem = 0;
        CUDA_TRY(h, cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device));
        const double need = (double)ctas_per_sm * (double)(smem + 1024);   /* + the per-CTA reserve */
        lc.carveout = (int)std::min(100.0, std::ceil(100.0 * need / (double)sm_smem));
    }
    int per_sm = 0;
    CUDA_TRY(h, gpr::hmc_occupancy(kp, wpc, smem, lc.carveout, lc.stream, &per_sm));
    if (per_sm < 1) return fail(h, GPR_ERR_ARG, "kernel cannot be resident (smem %zu)", smem);
    if (ctas_per_sm > 0 && per_sm > ctas_per_sm) per_sm = ctas_per_sm;
    long long ctas = (long long)h->num_sms * per_sm;
    const long long need = (h->N + wpc - 1) / wpc;
    if (ctas > need) ctas = need;
    lc.warps_per_cta = wpc;
    lc.smem_bytes = smem;
    lc.ctas = (int)ctas;
    h->lc = lc;
    return GPR_OK;
}

/* A dataset is streamed from device memory when the caller asks for it, or
 * when staging it beside a full CTA of warps would not fit in shared memory;
 * streaming uses K = 4 points per lane in passes.  pipe: the pipelined kernel
 * (two chains per warp, one barrier per half-step; lockstep is then unused);
 * it needs heavy ops unrolled, and for batched data chain groups of
 * 2 x warps_per_cta chains within one dataset. */
static int configure_launch(gpr_handle* h, int K, int onepass, int rolled, int lockstep = 1, int wpc0 = 8,
                            int pipe = 1) {
    gpr::KParams& kp = h->kp;
    if (kp.const_mode == GPR_CONST_HMC) return configure_hmc(h);
    drop_graph(h);
    gpr::LaunchCfg lc;
    lc.carveout = 0;
    if (pipe && rolled) return fail(h, GPR_ERR_ARG, "the pipelined kernel runs heavy ops unrolled only");
    if (pipe && kp.nds > 0 && kp.chains_per_ds % 2)
        pipe = 0;   /* an odd number of chains per dataset cannot pair up within one dataset */
    if (kp.nds > 0) {   /* batched: CTA groups within one dataset, staged per group; K = 4 in passes */
        K = 4;
        onepass = 0;
        if (lockstep < 1) lockstep = 1;
        wpc0 = batched_wpc(kp, wpc0, pipe);
    }
    auto smem_of = [&](int k, int w, int st) {
        return pipe ? gpr::pipe_smem_bytes(kp, k, w, st) : gpr::mh_smem_bytes(kp, k, w, st);
    };
    lc.stream = h->stream_data || smem_of(K, wpc0, 0) > 227 * 1024;
    if (lc.stream) { K = 4; onepass = 0; }
    lc.K = K;
    lc.onepass = onepass;
    lc.rolled = rolled;
    lc.lockstep = lockstep;
    lc.pipe = pipe;
    int wpc = wpc0;
    size_t smem = smem_of(lc.K, wpc, lc.stream);
    while (smem > 227 * 1024 && wpc > 1) {
        wpc /= 2;
        smem = smem_of(lc.K, wpc, lc.stream);
    }
    if (kp.nds > 0) wpc = batched_wpc(kp, wpc, pipe);
    if (smem > 227 * 1024)
        return fail(h, GPR_ERR_ARG, "programs of length %d do not fit in shared memory", kp.PL);
    lc.warps_per_cta = wpc;
    lc.smem_bytes = smem;
    int per_sm = 0;
    CUDA_TRY(h, gpr::mh_occupancy(kp, lc, &per_sm));
    if (per_sm < 1) return fail(h, GPR_ERR_ARG, "kernel cannot be resident (smem %zu)", smem);
    long long ctas = (long long)h->num_sms * per_sm;
    const int per_cta = pipe ? 2 * wpc : wpc;
    long long need = (h->N + per_cta - 1) / per_cta;
    if (ctas > need) ctas = need;
    lc.ctas = (int)ctas;
    /* chunk sums beyond the pipelined kernel's shared-memory board: one row
     * per (CTA, group, warp) in device memory */
    kp.part_stride = 0;
    const int stride = pipe ? gpr::pipe_part_stride(kp.nd) : 0;
    if (stride > 0) {
        const size_t need_f = (size_t)lc.ctas * 16 * (size_t)stride;
        if (h->dpart_floats < need_f) {
            CUDA_TRY(h, cudaStreamSynchronize(h->stream));
            cudaFree(h->dpart);
            h->dpart = nullptr;
            h->dpart_floats = 0;
            CUDA_TRY(h, cudaMalloc(&h->dpart, need_f * sizeof(float)));
            h->dpart_floats = need_f;
        }
        kp.part = h->dpart;
        kp.part_stride = stride;
    }
    h->lc = lc;
    return GPR_OK;
}

/* Default layout before any autotuning: K = 4 points per lane, one pass when
 * the data fit, heavy ops unrolled; the lockstep kernel while a CTA can
 * balance its chains' passes over its warps (up to GPR_MAX_PASSES passes: on
 * the 250-point workload it measured 10% faster), the pipelined kernel beyond
 * (which splits any number of passes over the warps: 20% faster on the
 * 65,536-point workload than free-running warps).  Three input variables and
 * batched data take K = 4 in passes (gpr_autotune re-checks per dataset). */
static int choose_launch(gpr_handle* h) {
    const int pipe = (h->kp.nd + 127) / 128 > GPR_MAX_PASSES ? 1 : 0;
    return configure_launch(h, 4, (h->kp.nd <= 128 && h->kp.nv != 3 && h->kp.nds == 0) ? 1 : 0, 0, 1, 8, pipe);
}

/* Device layout of a dataset: x1 | y | w | sd | x2 | x3, nd_pad floats each
 * (x2, x3 only for three input variables). */
static int set_data_body(gpr_handle* h, const float* x, const float* x2, const float* x3, const float* y,
                         const float* sd, int n);

/* The host staging copies of a dataset can exceed host memory; no C++
 * exception may leave a C entry point, so allocation failures become error
 * codes. */
static int set_data_impl(gpr_handle* h, const float* x, const float* x2, const float* x3, const float* y,
                         const float* sd, int n) {
    try {
        return set_data_body(h, x, x2, x3, y, sd, n);
    } catch (const std::bad_alloc&) {
        return fail(h, GPR_ERR_ARG, "not enough host memory to stage %d points", n);
    }
}

static int set_data_body(gpr_handle* h, const float* x, const float* x2, const float* x3, const float* y,
                         const float* sd, int n) {
    if (n < 0) return fail(h, GPR_ERR_ARG, "n must be >= 0");
    if (n > 0 && (!x || !y || !sd)) return fail(h, GPR_ERR_ARG, "x, y, sd must be non-NULL");
    const bool three = h->kp.nv == 3;
    if (n > 0 && three && (!x2 || !x3)) return fail(h, GPR_ERR_ARG, "x2, x3 must be non-NULL");
    for (int i = 0; i < n; ++i)
        if (!(sd[i] > 0.0f)) return fail(h, GPR_ERR_ARG, "sd[%d] = %g is not > 0", i, (double)sd[i]);
    CUDA_TRY(h, cudaSetDevice(h->device));
    const int nd_pad = (n + 3) & ~3;
    std::vector<float> host((size_t)(three ? 6 : 4) * nd_pad, 0.0f);
    if (three)
        for (int i = 0; i < n; ++i) {
            host[4 * (size_t)nd_pad + i] = x2[i];
            host[5 * (size_t)nd_pad + i] = x3[i];
        }
    double normsum = 0.0;
    const double PIf = 3.141592653589;
    const int we = weight_exponent(sd, (size_t)n);
    for (int i = 0; i < n; ++i) {
        host[i] = x[i];
        host[nd_pad + i] = y[i];
        host[2 * (size_t)nd_pad + i] = point_weight(sd[i], we);
        host[3 * (size_t)nd_pad + i] = sd[i];
        /* the constant part of lnormalpdf (main.cu:300), per point */
        normsum += 0.5 * ((double)logf((float)(2.0 * PIf)) + 2.0 * (double)logf(sd[i]));
    }
    drop_graph(h);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    forget_data(h);
    if (h->ddata) { cudaFree(h->ddata); h->ddata = nullptr; }
    if (nd_pad > 0) {
        CUDA_TRY(h, cudaMalloc(&h->ddata, host.size() * sizeof(float)));
        CUDA_TRY(h, cudaMemcpyAsync(h->ddata, host.data(), host.size() * sizeof(float),
                                    cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    }
    h->nd = n;
    h->nd_pad = nd_pad;
    h->normsum = normsum;
    gpr::KParams& kp = h->kp;
    kp.nd = n; kp.nd_pad = nd_pad;
    {
        const double ns = normsum * 0x1p-64;
        kp.normsum_hi = (float)ns;
        kp.normsum_lo = (float)(ns - (double)kp.normsum_hi);
    }
    kp.normsum64 = normsum;
    set_weight_scale(kp, we);
    kp.dx = h->ddata;
    kp.dy = h->ddata ? h->ddata + nd_pad : nullptr;
    kp.dw = h->ddata ? h->ddata + 2 * (size_t)nd_pad : nullptr;
    kp.dx2 = (h->ddata && three) ? h->ddata + 4 * (size_t)nd_pad : nullptr;
    kp.dx3 = (h->ddata && three) ? h->ddata + 5 * (size_t)nd_pad : nullptr;
    return choose_launch(h);
}

int gpr_set_data(gpr_handle* h, const float* x, const float* y, const float* sd, int n) {
    if (!h) return GPR_ERR_ARG;
    if (h->kp.nv == 3) return fail(h, GPR_ERR_ARG, "a handle with three input variables takes gpr_set_data3");
    return set_data_impl(h, x, nullptr, nullptr, y, sd, n);
}

static int set_batched_body(gpr_handle* h, int n_datasets, const int* sizes, const float* x1, const float* x2,
                            const float* x3, const float* y, const float* sd);

int gpr_set_batched_data(gpr_handle* h, int n_datasets, const int* sizes, const float* x1, const float* x2,
                         const float* x3, const float* y, const float* sd) {
    if (!h) return GPR_ERR_ARG;
    try {
        return set_batched_body(h, n_datasets, sizes, x1, x2, x3, y, sd);
    } catch (const std::bad_alloc&) {
        return fail(h, GPR_ERR_ARG, "not enough host memory to stage %d datasets", n_datasets);
    }
}

static int set_batched_body(gpr_handle* h, int n_datasets, const int* sizes, const float* x1, const float* x2,
                            const float* x3, const float* y, const float* sd) {
    if (n_datasets < 1 || !sizes) return fail(h, GPR_ERR_ARG, "n_datasets must be >= 1 with sizes");
    if (h->N % n_datasets) return fail(h, GPR_ERR_ARG, "%d chains do not split evenly into %d datasets",
                                       h->N, n_datasets);
    const int cpd = h->N / n_datasets;
    const bool three = h->kp.nv == 3;
    long long total = 0, maxn = 0, npad = 0;
    for (int d = 0; d < n_datasets; ++d) {
        if (sizes[d] < 0) return fail(h, GPR_ERR_ARG, "sizes[%d] = %d is negative", d, sizes[d]);
        total += sizes[d];
        npad += (sizes[d] + 3) & ~3;
        if (sizes[d] > maxn) maxn = sizes[d];
    }
    if (npad > (1ll << 30)) return fail(h, GPR_ERR_ARG, "batched data too large");
    if (total > 0 && (!x1 || !y || !sd || (three && (!x2 || !x3))))
        return fail(h, GPR_ERR_ARG, "point arrays must be non-NULL (x2, x3 for three variables)");
    for (long long i = 0; i < total; ++i)
        if (!(sd[i] > 0.0f)) return fail(h, GPR_ERR_ARG, "sd[%lld] = %g is not > 0", i, (double)sd[i]);
    CUDA_TRY(h, cudaSetDevice(h->device));
    drop_graph(h);
    const size_t T = (size_t)npad;
    std::vector<float> host((three ? 6 : 4) * T + 4, 0.0f);
    std::vector<int> meta(3 * (size_t)n_datasets);
    std::vector<float> ns(2 * (size_t)n_datasets);
    std::vector<double> ns64((size_t)n_datasets);
    const double PIf = 3.141592653589;
    const int we = weight_exponent(sd, (size_t)total);
    size_t off = 0, src = 0;
    for (int d = 0; d < n_datasets; ++d) {
        meta[d] = (int)off;
        meta[n_datasets + d] = sizes[d];
        double normsum = 0.0;
        for (int i = 0; i < sizes[d]; ++i, ++src) {
            host[off + i] = x1[src];
            host[T + off + i] = y[src];
            host[2 * T + off + i] = point_weight(sd[src], we);
            host[3 * T + off + i] = sd[src];
            if (three) { host[4 * T + off + i] = x2[src]; host[5 * T + off + i] = x3[src]; }
            normsum += 0.5 * ((double)logf((float)(2.0 * PIf)) + 2.0 * (double)logf(sd[src]));   /* main.cu:300 */
        }
        ns64[d] = normsum;
        const double nsd = normsum * 0x1p-64;
        ns[2 * d] = (float)nsd;
        ns[2 * d + 1] = (float)(nsd - (double)ns[2 * d]);
        off += (sizes[d] + 3) & ~3;
    }
    /* datasets claimed largest first, so that uneven sizes balance across the grid */
    std::vector<int> order(n_datasets);
    for (int d = 0; d < n_datasets; ++d) order[d] = d;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sizes[a] > sizes[b]; });
    for (int d = 0; d < n_datasets; ++d) meta[2 * n_datasets + d] = order[d];
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    forget_data(h);
    if (h->ddata) { cudaFree(h->ddata); h->ddata = nullptr; }
    cudaFree(h->dds); cudaFree(h->dds_ns); cudaFree(h->dds_ns64);
    h->dds = nullptr; h->dds_ns = nullptr; h->dds_ns64 = nullptr;
    CUDA_TRY(h, cudaMalloc(&h->ddata, host.size() * sizeof(float)));
    CUDA_TRY(h, cudaMalloc(&h->dds, meta.size() * sizeof(int)));
    CUDA_TRY(h, cudaMalloc(&h->dds_ns, ns.size() * sizeof(float)));
    CUDA_TRY(h, cudaMalloc(&h->dds_ns64, ns64.size() * sizeof(double)));
    CUDA_TRY(h, cudaMemcpyAsync(h->ddata, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->dds, meta.data(), meta.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->dds_ns, ns.data(), ns.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->dds_ns64, ns64.data(), ns64.size() * sizeof(double), cudaMemcpyHostToDevice,
                                h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    gpr::KParams& kp = h->kp;
    h->nd = (int)maxn;
    h->nd_pad = (int)((maxn + 3) & ~3);
    kp.nd = h->nd; kp.nd_pad = h->nd_pad;
    kp.normsum_hi = kp.normsum_lo = 0.0f;
    kp.normsum64 = 0.0;
    set_weight_scale(kp, we);
    kp.dx = h->ddata; kp.dy = h->ddata + T; kp.dw = h->ddata + 2 * T;
    kp.dx2 = three ? h->ddata + 4 * T : nullptr;
    kp.dx3 = three ? h->ddata + 5 * T : nullptr;
    kp.nds = n_datasets;
    kp.chains_per_ds = cpd;
    kp.ds_off = h->dds;
    kp.ds_n = h->dds + n_datasets;
    kp.ds_order = h->dds + 2 * n_datasets;
    kp.ds_ns = h->dds_ns;
    kp.ds_ns64 = h->dds_ns64;
    return choose_launch(h);
}

static int run(gpr_handle* h, int steps, int seed);

int gpr_capture_blocks(gpr_handle* h, int n_blocks, int steps) {
    if (!h) return GPR_ERR_ARG;
    if (n_blocks < 1 || steps < 0) return fail(h, GPR_ERR_ARG, "n_blocks must be >= 1 and steps >= 0");
    if (h->nd < 0) return fail(h, GPR_ERR_STATE, "gpr_set_data has not been called");
    CUDA_TRY(h, cudaSetDevice(h->device));
    drop_graph(h);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    /* one counter reset and one kernel node per block; after each block the
     * capture's single frontier node is that block's kernel */
    std::vector<cudaGraphNode_t> nodes;
    CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = GPR_OK;
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < n_blocks && rc == GPR_OK && e == cudaSuccess; ++b) {
        rc = run(h, steps, 0);
        if (rc != GPR_OK) break;
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        e = cudaStreamGetCaptureInfo(h->stream, &cs, nullptr, nullptr, &deps, nullptr, &ndeps);
        if (e == cudaSuccess && ndeps != 1) e = cudaErrorStreamCaptureUnmatched;
        if (e == cudaSuccess) nodes.push_back(deps[0]);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
    if (e == cudaSuccess) e = e2;
    std::vector<cudaKernelNodeParams> params(nodes.size());
    std::vector<gpr::KParams> kps(nodes.size());
    for (size_t b = 0; b < nodes.size() && e == cudaSuccess && rc == GPR_OK; ++b) {
        cudaGraphNodeType t;
        e = cudaGraphNodeGetType(nodes[b], &t);
        if (e == cudaSuccess && t != cudaGraphNodeTypeKernel) e = cudaErrorStreamCaptureUnmatched;
        if (e == cudaSuccess) e = cudaGraphKernelNodeGetParams(nodes[b], &params[b]);
        if (e == cudaSuccess) {   /* the kernels take one argument, the KParams */
            kps[b] = *(const gpr::KParams*)params[b].kernelParams[0];
            params[b].extra = nullptr;
        }
    }
    cudaGraphExec_t ex = nullptr;
    if (e == cudaSuccess && rc == GPR_OK) e = cudaGraphInstantiate(&ex, g, 0);
    if (rc != GPR_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (rc != GPR_OK) return rc;
        return fail(h, GPR_ERR_CUDA, "gpr_capture_blocks: %s", cudaGetErrorString(e));
    }
    h->graph_src = g;
    h->graph = ex;
    h->graph_nodes = std::move(nodes);
    h->graph_params = std::move(params);
    h->graph_kp = std::move(kps);
    h->graph_blocks = n_blocks;
    return GPR_OK;
}

int gpr_run_captured(gpr_handle* h, const int* seeds) {
    if (!h || !seeds) return GPR_ERR_ARG;
    NvtxRange r("gpr_run_captured: MH blocks");
    if (!h->graph) return fail(h, GPR_ERR_STATE, "no captured block sequence (gpr_capture_blocks)");
    CUDA_TRY(h, cudaSetDevice(h->device));
    /* the seeds go into the kernel nodes' parameters: the update applies to
     * launches after it, not to a replay already enqueued */
    for (int b = 0; b < h->graph_blocks; ++b) {
        gpr::KParams kp = h->graph_kp[b];
        kp.seed = (uint32_t)seeds[b];
        cudaKernelNodeParams np = h->graph_params[b];
        void* args[] = {(void*)&kp};
        np.kernelParams = args;
        CUDA_TRY(h, cudaGraphExecKernelNodeSetParams(h->graph, h->graph_nodes[b], &np));
    }
    CUDA_TRY(h, cudaGraphLaunch(h->graph, h->stream));
    h->launches += h->graph_blocks;
    return GPR_OK;
}

int gpr_set_data3(gpr_handle* h, const float* x1, const float* x2, const float* x3, const float* y,
                  const float* sd, int n) {
    if (!h) return GPR_ERR_ARG;
    if (h->kp.nv != 3) return fail(h, GPR_ERR_ARG, "gpr_set_data3 needs a handle created with n_vars = 3");
    return set_data_impl(h, x1, x2, x3, y, sd, n);
}

int gpr_set_state(gpr_handle* h, const int32_t* P, const float* C) {
    if (!h) return GPR_ERR_ARG;
    NvtxRange r("gpr_set_state: state in");
    if (!P || !C) return fail(h, GPR_ERR_ARG, "P and C must be non-NULL");
    const size_t cnt = (size_t)h->N * h->PL;
    for (size_t i = 0; i < cnt; ++i) {
        if (P[i] < 0 || P[i] >= OP_NALL)
            return fail(h, GPR_ERR_ARG, "P[%zu] = %d is not an op code", i, P[i]);
        if ((P[i] == OP_X2 || P[i] == OP_X3) && h->kp.nv != 3)
            return fail(h, GPR_ERR_ARG, "P[%zu] = %d reads x2/x3, which needs n_vars = 3", i, P[i]);
    }
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, cudaMemcpyAsync(h->dP, P, cnt * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->dC, C, cnt * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GPR_OK;
}

int gpr_set_scores(gpr_handle* h, const double* prior, const double* likelihood) {
    if (!h) return GPR_ERR_ARG;
    if (!prior || !likelihood) return fail(h, GPR_ERR_ARG, "prior and likelihood must be non-NULL");
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, cudaMemcpyAsync(h->dprior, prior, h->N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->dlik, likelihood, h->N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GPR_OK;
}

int gpr_get_state(gpr_handle* h, int32_t* P, float* C, double* prior, double* likelihood) {
    if (!h) return GPR_ERR_ARG;
    NvtxRange r("gpr_get_state: state out");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t cnt = (size_t)h->N * h->PL;
    if (P) CUDA_TRY(h, cudaMemcpyAsync(P, h->dP, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    if (C) CUDA_TRY(h, cudaMemcpyAsync(C, h->dC, cnt * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    if (prior) CUDA_TRY(h, cudaMemcpyAsync(prior, h->dprior, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (likelihood)
        CUDA_TRY(h, cudaMemcpyAsync(likelihood, h->dlik, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return gpr_sync(h);
}

static int run(gpr_handle* h, int steps, int seed) {
    if (h->nd < 0) return fail(h, GPR_ERR_STATE, "gpr_set_data has not been called");
    CUDA_TRY(h, cudaSetDevice(h->device));
    h->kp.steps = steps;
    h->kp.seed = (uint32_t)seed;
    CUDA_TRY(h, cudaMemsetAsync(h->dcounter, 0, sizeof(int), h->stream));
    if (h->kp.const_mode == GPR_CONST_HMC) CUDA_TRY(h, gpr::launch_hmc_block(h->kp, h->lc, h->stream));
    else CUDA_TRY(h, gpr::launch_mh_block(h->kp, h->lc, h->stream));
    h->launches++;
    return GPR_OK;
}

int gpr_run_block(gpr_handle* h, int steps, int random_seed) {
    if (!h) return GPR_ERR_ARG;
    NvtxRange r("gpr_run_block: MH block");
    if (steps < 0) return fail(h, GPR_ERR_ARG, "steps must be >= 0 (got %d)", steps);
    return run(h, steps, random_seed);
}

int gpr_evaluate(gpr_handle* h) {
    if (!h) return GPR_ERR_ARG;
    return run(h, 0, 0);
}

int gpr_sync(gpr_handle* h) {
    if (!h) return GPR_ERR_ARG;
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    int flags = 0;
    CUDA_TRY(h, cudaMemcpy(&flags, h->dcounter + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (flags) {
        cudaMemset(h->dcounter + 1, 0, sizeof(int));
        return fail(h, GPR_ERR_DEVICE, "kernel error flags 0x%x (1: dataset staging timed out, "
                    "2: constant-proposal offsets did not converge, 4: a consistency check of the phase-timed build "
                    "failed)", flags);
    }
    return GPR_OK;
}

int gpr_device_state(gpr_handle* h, int32_t** P, float** C, double** prior, double** likelihood) {
    if (!h) return GPR_ERR_ARG;
    if (P) *P = h->dP;
    if (C) *C = h->dC;
    if (prior) *prior = h->dprior;
    if (likelihood) *likelihood = h->dlik;
    return GPR_OK;
}

int gpr_debug_eval_values(gpr_handle* h, const float* xs, int nx, float* out, float* length,
                          int* count) {
    if (!h) return GPR_ERR_ARG;
    if (nx < 0 || (nx > 0 && (!xs || !out)) || !length || !count)
        return fail(h, GPR_ERR_ARG, "bad arguments");
    CUDA_TRY(h, cudaSetDevice(h->device));
    float *dxs = nullptr, *dout = nullptr, *dlen = nullptr;
    int* dcnt = nullptr;
    const size_t no = (size_t)h->N * (size_t)nx;
    const size_t nvx = h->kp.nv == 3 ? 3 : 1;   /* xs holds x1 | x2 | x3 for three variables */
    int rc = GPR_OK;
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc(&dxs, (nvx * (size_t)nx + 1) * sizeof(float))) != cudaSuccess) goto done;
    if ((e = cudaMalloc(&dout, (no + 1) * sizeof(float))) != cudaSuccess) goto done;
    if ((e = cudaMalloc(&dlen, h->N * sizeof(float))) != cudaSuccess) goto done;
    if ((e = cudaMalloc(&dcnt, h->N * sizeof(int))) != cudaSuccess) goto done;
    if (nx > 0 && (e = cudaMemcpyAsync(dxs, xs, nvx * (size_t)nx * sizeof(float), cudaMemcpyHostToDevice, h->stream)) != cudaSuccess) goto done;
    if ((e = gpr::launch_eval_values(h->kp, dxs, nx, dout, dlen, dcnt, h->stream)) != cudaSuccess) goto done;
    h->launches++;
    if (nx > 0 && (e = cudaMemcpyAsync(out, dout, no * sizeof(float), cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess) goto done;
    if ((e = cudaMemcpyAsync(length, dlen, h->N * sizeof(float), cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess) goto done;
    if ((e = cudaMemcpyAsync(count, dcnt, h->N * sizeof(int), cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess) goto done;
    e = cudaStreamSynchronize(h->stream);
done:
    if (e != cudaSuccess) rc = fail(h, GPR_ERR_CUDA, "gpr_debug_eval_values: %s", cudaGetErrorString(e));
    cudaFree(dxs); cudaFree(dout); cudaFree(dlen); cudaFree(dcnt);
    return rc;
}

int gpr_debug_math(gpr_handle* h, int op, const float* a, const float* b, float* out, int n) {
    if (!h || n < 0 || op < 0 || op > 2 || (n > 0 && (!a || !out || (op == 2 && !b))))
        return fail(h, GPR_ERR_ARG, "bad arguments");
    CUDA_TRY(h, cudaSetDevice(h->device));
    float* d = nullptr;
    const size_t bytes = (size_t)(n + 1) * sizeof(float);
    CUDA_TRY(h, cudaMalloc(&d, 3 * bytes));
    float *da = d, *db = d + (n + 1), *dout = d + 2 * (size_t)(n + 1);
    cudaError_t e = cudaMemcpyAsync(da, a, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && op == 2)
        e = cudaMemcpyAsync(db, b, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = gpr::launch_math(op, da, db, dout, n, h->stream);
    if (e == cudaSuccess) { h->launches++; e = cudaMemcpyAsync(out, dout, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, h->stream); }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(h, GPR_ERR_CUDA, "gpr_debug_math: %s", cudaGetErrorString(e));
    return GPR_OK;
}

int gpr_debug_fp_issue(int device, int iters, float* ms_dadd32, float* ms_dadd1, float* ms_fadd32) {
    if (iters < 1 || !ms_dadd32 || !ms_dadd1 || !ms_fadd32) return fail(nullptr, GPR_ERR_ARG, "bad arguments");
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = gpr::time_fp_adds(iters, ms_dadd32, ms_dadd1, ms_fadd32);
    if (e != cudaSuccess) return fail(nullptr, GPR_ERR_CUDA, "gpr_debug_fp_issue: %s", cudaGetErrorString(e));
    return GPR_OK;
}

int gpr_debug_stage_wait(gpr_handle* h, int polls) {
    if (!h) return GPR_ERR_ARG;
    if (polls < 0) return fail(h, GPR_ERR_ARG, "polls must be >= 0 (got %d)", polls);
    drop_graph(h);
    h->kp.stage_wait_iters = polls;
    return GPR_OK;
}

int gpr_debug_phase_profile(gpr_handle* h, int steps, int random_seed, uint64_t* out, int n) {
    if (!h) return GPR_ERR_ARG;
    if (steps < 0 || n < 0 || (n > 0 && !out)) return fail(h, GPR_ERR_ARG, "bad arguments");
    if (h->nd < 0) return fail(h, GPR_ERR_STATE, "gpr_set_data has not been called");
    if (h->kp.const_mode == GPR_CONST_HMC || h->kp.nv == 3 || h->kp.nds > 0 || h->lc.rolled ||
        h->kp.rng_mode != GPR_RNG_LCG || !gpr::prof_kernel(h->lc))
        return fail(h, GPR_ERR_ARG, "no phase-timed build of this layout");
    CUDA_TRY(h, cudaSetDevice(h->device));
    unsigned long long* d = nullptr;
    CUDA_TRY(h, cudaMalloc(&d, GPR_PH_SLOTS * sizeof(unsigned long long)));
    unsigned long long tmp[GPR_PH_SLOTS] = {};
    gpr::KParams kp = h->kp;
    kp.steps = steps;
    kp.seed = (uint32_t)random_seed;
    kp.phase = d;
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof tmp, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->dcounter, 0, sizeof(int), h->stream);
    if (e == cudaSuccess) e = gpr::launch_mh_block_prof(kp, h->lc, h->stream);
    if (e == cudaSuccess) {
        h->launches++;
        e = cudaMemcpyAsync(tmp, d, sizeof tmp, cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(h, GPR_ERR_CUDA, "gpr_debug_phase_profile: %s", cudaGetErrorString(e));
    for (int i = 0; i < n && i < GPR_PH_SLOTS; ++i) out[i] = tmp[i];
    return gpr_sync(h);
}

int gpr_autotune(gpr_handle* h, int steps, int seed, int* K, int* onepass, int* rolled, float* best_ms) {
    if (!h || steps <= 0) return fail(h, GPR_ERR_ARG, "bad arguments");
    if (h->nd < 0) return fail(h, GPR_ERR_STATE, "gpr_set_data has not been called");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const bool hmc = h->kp.const_mode == GPR_CONST_HMC;
    const size_t cnt = (size_t)h->N * h->PL;
    int32_t* sP = nullptr; float* sC = nullptr; double* sPr = nullptr; double* sLi = nullptr;
    unsigned long long* sSt = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GPR_OK;
    /* staged layouts, then (unless the handle always streams) the streamed one,
     * which reads the data from device memory / L2 and leaves shared memory to
     * the warps; batched data and three variables take multi-pass layouts only;
     * each with the pipelined kernel (heavy ops unrolled) and the lockstep one */
    struct Cand { int K, onepass, rolled, stream, pipe; } cands[24];
    int nc = 0;
    const int saved_stream = h->stream_data;
    const bool multi_only = h->kp.nds > 0 || h->kp.nv == 3;
    for (int pi = 1; pi >= 0; --pi)
        for (int Kc : {4, 8})
            for (int op = 1; op >= 0; --op)
                for (int ro = 0; ro <= (pi ? 0 : 1); ++ro)
                    if ((!op || (h->nd <= 32 * Kc && !multi_only)) && !(multi_only && Kc != 4))
                        cands[nc++] = {Kc, op, ro, saved_stream, pi};
    if (!saved_stream)
        for (int pi = 1; pi >= 0; --pi)
            for (int ro = 0; ro <= (pi ? 0 : 1); ++ro) cands[nc++] = {4, 0, ro, 1, pi};
    const gpr::LaunchCfg orig = h->lc;
    float best = 1e30f;
    gpr::LaunchCfg bestlc = orig;
    cudaError_t e;
    /* trial blocks leave the per-chain scales alone */
    const float saved_target = h->kp.adapt_target;
    h->kp.adapt_target = 0.0f;
#define AT_TRY(call) do { if ((e = (call)) != cudaSuccess) { rc = fail(h, GPR_ERR_CUDA, "gpr_autotune: %s: %s", #call, cudaGetErrorString(e)); goto done; } } while (0)
    AT_TRY(cudaMalloc(&sP, cnt * sizeof(int32_t)));
    AT_TRY(cudaMalloc(&sC, cnt * sizeof(float)));
    AT_TRY(cudaMalloc(&sPr, h->N * sizeof(double)));
    AT_TRY(cudaMalloc(&sLi, h->N * sizeof(double)));
    AT_TRY(cudaMalloc(&sSt, GPR_NSTATS * sizeof(unsigned long long)));
    AT_TRY(cudaMemcpyAsync(sP, h->dP, cnt * sizeof(int32_t), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(sC, h->dC, cnt * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(sPr, h->dprior, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(sLi, h->dlik, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(sSt, h->dstats, GPR_NSTATS * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaEventCreate(&e0));
    AT_TRY(cudaEventCreate(&e1));
    /* the Hamiltonian kernel: CTA size and resident CTAs per SM, i.e. occupancy
     * against L1 left for the gradient tapes */
    if (hmc) {
        /* CTA size and residency cap, each with the data staged (unless the
         * handle always streams) and streamed */
        const int shapes[8][2] = {{4, 0}, {4, 7}, {4, 5}, {4, 4}, {2, 0}, {1, 0}, {8, 0}, {8, 3}};
        for (int i = 0; i < 16; ++i) {
            const int want_stream = i >= 8;
            if (configure_hmc(h, shapes[i % 8][0], shapes[i % 8][1], want_stream) != GPR_OK) continue;
            if (h->lc.stream != want_stream) continue;   /* forced one way: tried once */
            for (int rep = 0; rep < 2; ++rep) {
                AT_TRY(cudaMemcpyAsync(h->dP, sP, cnt * sizeof(int32_t), cudaMemcpyDeviceToDevice, h->stream));
                AT_TRY(cudaMemcpyAsync(h->dC, sC, cnt * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
                AT_TRY(cudaEventRecord(e0, h->stream));
                if ((rc = run(h, steps, seed)) != GPR_OK) goto done;
                AT_TRY(cudaEventRecord(e1, h->stream));
                AT_TRY(cudaEventSynchronize(e1));
            }
            float ms = 0.0f;
            AT_TRY(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) { best = ms; bestlc = h->lc; }
        }
        nc = 0;
    }
    for (int i = 0; i < nc; ++i) {
        h->stream_data = cands[i].stream;
        const int crc = configure_launch(h, cands[i].K, cands[i].onepass, cands[i].rolled, 1, 8, cands[i].pipe);
        h->stream_data = saved_stream;
        if (crc != GPR_OK || (cands[i].stream && !h->lc.stream) || h->lc.pipe != cands[i].pipe) continue;
        for (int rep = 0; rep < 2; ++rep) {   /* first run warms up, second is timed */
            AT_TRY(cudaMemcpyAsync(h->dP, sP, cnt * sizeof(int32_t), cudaMemcpyDeviceToDevice, h->stream));
            AT_TRY(cudaMemcpyAsync(h->dC, sC, cnt * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
            AT_TRY(cudaEventRecord(e0, h->stream));
            if ((rc = run(h, steps, seed)) != GPR_OK) goto done;
            AT_TRY(cudaEventRecord(e1, h->stream));
            AT_TRY(cudaEventSynchronize(e1));
        }
        float ms = 0.0f;
        AT_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) { best = ms; bestlc = h->lc; }
    }
    /* second stage: barrier period (lockstep kernel) and CTA size for the best layout */
    if (!hmc) {
        const gpr::LaunchCfg base = bestlc;
        const int periods[3] = {1, 5, 0};
        const int wpcs[2] = {8, 4};
        for (int pi = 0; pi < (base.pipe ? 1 : 3); ++pi)
            for (int wi = 0; wi < 2; ++wi) {
                if (periods[pi] == base.lockstep && wpcs[wi] == base.warps_per_cta) continue;
                h->stream_data = base.stream ? 1 : saved_stream;
                const int crc = configure_launch(h, base.K, base.onepass, base.rolled, periods[pi], wpcs[wi],
                                                 base.pipe);
                h->stream_data = saved_stream;
                if (crc != GPR_OK) continue;
                for (int rep = 0; rep < 2; ++rep) {
                    AT_TRY(cudaMemcpyAsync(h->dP, sP, cnt * sizeof(int32_t), cudaMemcpyDeviceToDevice, h->stream));
                    AT_TRY(cudaMemcpyAsync(h->dC, sC, cnt * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
                    AT_TRY(cudaEventRecord(e0, h->stream));
                    if ((rc = run(h, steps, seed)) != GPR_OK) goto done;
                    AT_TRY(cudaEventRecord(e1, h->stream));
                    AT_TRY(cudaEventSynchronize(e1));
                }
                float ms = 0.0f;
                AT_TRY(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) { best = ms; bestlc = h->lc; }
            }
    }
    if (!hmc) {
        /* re-derive the chosen layout (and its scratch) rather than copying it */
        h->stream_data = bestlc.stream ? 1 : saved_stream;
        rc = configure_launch(h, bestlc.K, bestlc.onepass, bestlc.rolled, bestlc.lockstep, bestlc.warps_per_cta,
                              bestlc.pipe);
        h->stream_data = saved_stream;
        if (rc != GPR_OK) goto done;
    } else {
        h->lc = bestlc;
    }
    AT_TRY(cudaMemcpyAsync(h->dP, sP, cnt * sizeof(int32_t), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(h->dC, sC, cnt * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(h->dprior, sPr, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(h->dlik, sLi, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaMemcpyAsync(h->dstats, sSt, GPR_NSTATS * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, h->stream));
    AT_TRY(cudaStreamSynchronize(h->stream));
    if (K) *K = h->lc.K;
    if (onepass) *onepass = h->lc.onepass;
    if (rolled) *rolled = h->lc.rolled;
    if (best_ms) *best_ms = best;
#undef AT_TRY
done:
    h->kp.adapt_target = saved_target;
    if (rc != GPR_OK) h->lc = orig;
    cudaFree(sP); cudaFree(sC); cudaFree(sPr); cudaFree(sLi); cudaFree(sSt);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}

int gpr_set_hmc_layout(gpr_handle* h, int warps_per_cta, int ctas_per_sm) {
    if (!h) return GPR_ERR_ARG;
    if (h->kp.const_mode != GPR_CONST_HMC) return fail(h, GPR_ERR_ARG, "not a GPR_CONST_HMC handle");
    if ((warps_per_cta != 1 && warps_per_cta != 2 && warps_per_cta != 4 && warps_per_cta != 8) || ctas_per_sm < 0)
        return fail(h, GPR_ERR_ARG, "invalid layout: %d warps per CTA, %d CTAs per SM", warps_per_cta, ctas_per_sm);
    CUDA_TRY(h, cudaSetDevice(h->device));
    return configure_hmc(h, warps_per_cta, ctas_per_sm);
}

int gpr_set_streaming(gpr_handle* h, int always) {
    if (!h) return GPR_ERR_ARG;
    h->stream_data = always ? 1 : 0;
    if (h->nd < 0) return GPR_OK;
    CUDA_TRY(h, cudaSetDevice(h->device));
    return choose_launch(h);
}

int gpr_layout_streamed(gpr_handle* h) { return h ? h->lc.stream : 0; }

int gpr_set_layout(gpr_handle* h, int K, int onepass, int rolled) {
    return gpr_set_layout2(h, K, onepass, rolled, 1, 8);
}

int gpr_set_layout2(gpr_handle* h, int K, int onepass, int rolled, int lockstep, int warps_per_cta) {
    return gpr_set_layout3(h, K, onepass, rolled, lockstep, warps_per_cta, 0);
}

int gpr_set_layout3(gpr_handle* h, int K, int onepass, int rolled, int lockstep, int warps_per_cta, int pipe) {
    if (!h) return GPR_ERR_ARG;
    if (pipe && rolled) return fail(h, GPR_ERR_ARG, "the pipelined kernel runs heavy ops unrolled only");
    if (h->kp.const_mode == GPR_CONST_HMC) return fail(h, GPR_ERR_ARG, "the HMC kernel has a single layout");
    if ((K != 4 && K != 8) || (onepass && h->kp.nd > 32 * K) || lockstep < 0 ||
        (warps_per_cta != 1 && warps_per_cta != 2 && warps_per_cta != 4 && warps_per_cta != 8))
        return fail(h, GPR_ERR_ARG, "invalid layout K=%d onepass=%d lockstep=%d warps=%d for %d points", K,
                    onepass, lockstep, warps_per_cta, h->kp.nd);
    if ((h->kp.nv == 3 || h->kp.nds > 0) && (K != 4 || onepass))
        return fail(h, GPR_ERR_ARG, "%s take K=4 in passes (got K=%d onepass=%d)",
                    h->kp.nds > 0 ? "batched datasets" : "three input variables", K, onepass);
    CUDA_TRY(h, cudaSetDevice(h->device));
    return configure_launch(h, K, onepass ? 1 : 0, rolled ? 1 : 0, lockstep, warps_per_cta, pipe ? 1 : 0);
}

int gpr_launch_geometry(gpr_handle* h, int* K, int* onepass, int* warps_per_cta, int* ctas, int64_t* smem) {
    if (!h) return GPR_ERR_ARG;
    if (K) *K = h->lc.K;
    if (onepass) *onepass = h->lc.onepass;
    if (warps_per_cta) *warps_per_cta = h->lc.warps_per_cta;
    if (ctas) *ctas = h->lc.ctas;
    if (smem) *smem = (int64_t)h->lc.smem_bytes;
    return GPR_OK;
}

void* gpr_stream(gpr_handle* h) { return h ? (void*)h->stream : nullptr; }

int gpr_layout_rolled(gpr_handle* h) { return h ? h->lc.rolled : 0; }
int gpr_layout_lockstep(gpr_handle* h) { return h ? h->lc.lockstep : 0; }
int gpr_layout_pipelined(gpr_handle* h) { return h ? h->lc.pipe : 0; }

int gpr_get_stats(gpr_handle* h, uint64_t* out, int n) {
    if (!h || !out || n < 0) return GPR_ERR_ARG;
    unsigned long long tmp[GPR_NSTATS];
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, cudaMemcpyAsync(tmp, h->dstats, sizeof tmp, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    for (int i = 0; i < n && i < GPR_NSTATS; ++i) out[i] = tmp[i];
    return GPR_OK;
}

int gpr_reset_stats(gpr_handle* h) {
    if (!h) return GPR_ERR_ARG;
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, cudaMemsetAsync(h->dstats, 0, GPR_NSTATS * sizeof(unsigned long long), h->stream));
    return GPR_OK;
}

/* ---- move schedule, Hamiltonian moves, gradients, adaptation ---- */

int gpr_set_moves(gpr_handle* h, int struct_every, float hmc_eps, int hmc_steps) {
    if (!h) return GPR_ERR_ARG;
    if (struct_every < 0) return fail(h, GPR_ERR_ARG, "struct_every must be >= 0 (got %d)", struct_every);
    if (!(hmc_eps > 0.0f) || !(hmc_eps < 1e30f)) return fail(h, GPR_ERR_ARG, "hmc_eps must be > 0");
    if (hmc_steps < 1 || hmc_steps > 1024) return fail(h, GPR_ERR_ARG, "hmc_steps must be in [1, 1024]");
    drop_graph(h);
    h->kp.struct_every = struct_every;
    h->kp.hmc_eps = hmc_eps;
    h->kp.hmc_L = hmc_steps;
    return GPR_OK;
}

int gpr_set_hmc_jitter(gpr_handle* h, float eps_frac, float len_frac) {
    if (!h) return GPR_ERR_ARG;
    if (!(eps_frac >= 0.0f && eps_frac < 1.0f))
        return fail(h, GPR_ERR_ARG, "eps_frac must be in [0, 1) (got %g)", (double)eps_frac);
    if (!(len_frac >= 0.0f && len_frac <= 1.0f))
        return fail(h, GPR_ERR_ARG, "len_frac must be in [0, 1] (got %g)", (double)len_frac);
    drop_graph(h);
    h->kp.hmc_jit_eps = eps_frac;
    h->kp.hmc_jit_len = len_frac;
    return GPR_OK;
}

int gpr_adapt_scales(gpr_handle* h, float target_accept) {
    if (!h) return GPR_ERR_ARG;
    if (!(target_accept >= 0.0f && target_accept < 1.0f))
        return fail(h, GPR_ERR_ARG, "target acceptance %g is not in [0, 1)", (double)target_accept);
    if (h->kp.const_mode == GPR_CONST_REFERENCE)
        return fail(h, GPR_ERR_ARG, "the reference's constant proposals have no scale to adapt");
    CUDA_TRY(h, cudaSetDevice(h->device));
    if (!h->dscale) {
        /* the scales become the handle's only once they hold the start value */
        float* d = nullptr;
        CUDA_TRY(h, cudaMalloc(&d, (size_t)h->N * sizeof(float)));
        const float s0 = h->kp.const_mode == GPR_CONST_HMC ? h->kp.hmc_eps : h->kp.rw_sd;
        std::vector<float> init;
        try {
            init.assign((size_t)h->N, s0);
        } catch (const std::bad_alloc&) {
            cudaFree(d);
            return fail(h, GPR_ERR_ARG, "not enough host memory for %d chain scales", h->N);
        }
        cudaError_t e = cudaMemcpyAsync(d, init.data(), init.size() * sizeof(float), cudaMemcpyHostToDevice,
                                        h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) {
            cudaFree(d);
            return fail(h, GPR_ERR_CUDA, "gpr_adapt_scales: %s", cudaGetErrorString(e));
        }
        h->dscale = d;
        h->kp.chain_scale = d;
    }
    drop_graph(h);
    h->kp.adapt_target = target_accept;
    return GPR_OK;
}

int gpr_chain_scales(gpr_handle* h, float* out) {
    if (!h || !out) return GPR_ERR_ARG;
    if (!h->dscale) return fail(h, GPR_ERR_STATE, "no per-chain scales (gpr_adapt_scales has not been called)");
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, cudaMemcpyAsync(out, h->dscale, (size_t)h->N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GPR_OK;
}

int gpr_loglik_grad(gpr_handle* h, double* grad, double* likelihood) {
    if (!h) return GPR_ERR_ARG;
    if (!grad) return fail(h, GPR_ERR_ARG, "grad is NULL");
    if (h->nd < 0) return fail(h, GPR_ERR_STATE, "gpr_set_data has not been called");
    if (!gpr::grad_supported(h->kp))
        return fail(h, GPR_ERR_ARG, "gradients support program_length <= 127 (got %d)", h->PL);

    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t cnt = (size_t)h->N * h->PL;
    double* dg = nullptr;
    double* dl = nullptr;
    cudaError_t e = cudaMalloc(&dg, cnt * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dl, (size_t)h->N * sizeof(double));
    /* batched data: every warp reads its chain's dataset from device memory */
    const bool st = h->stream_data || h->kp.nds > 0 || gpr::grad_smem_bytes(h->kp, 4) > 227 * 1024;
    if (e == cudaSuccess) e = gpr::launch_loglik_grad(h->kp, dg, dl, st, h->stream);
    if (e == cudaSuccess) {
        h->launches++;
        e = cudaMemcpyAsync(grad, dg, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess && likelihood)
        e = cudaMemcpyAsync(likelihood, dl, (size_t)h->N * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dg);
    cudaFree(dl);
    if (e != cudaSuccess) return fail(h, GPR_ERR_CUDA, "gpr_loglik_grad: %s", cudaGetErrorString(e));
    return gpr_sync(h);
}

int gpr_run_block_traced_first(gpr_handle* h, int steps, int random_seed, int trace_n, int n_chains,
                               float* trace) {
    if (!h) return GPR_ERR_ARG;
    if (steps < 1) return fail(h, GPR_ERR_ARG, "steps must be >= 1 (got %d)", steps);
    if (trace_n < 1 || trace_n > 32 || trace_n > h->PL || !trace)
        return fail(h, GPR_ERR_ARG, "trace_n must be in [1, min(32, program_length)] with a buffer");
    if (n_chains < 1 || n_chains > h->N)
        return fail(h, GPR_ERR_ARG, "n_chains must be in [1, %d] (got %d)", h->N, n_chains);
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t cnt = (size_t)n_chains * (size_t)steps * (size_t)trace_n;
    float* dt = nullptr;
    CUDA_TRY(h, cudaMalloc(&dt, cnt * sizeof(float)));
    h->kp.trace = dt;
    h->kp.trace_n = trace_n;
    h->kp.trace_chains = n_chains;
    int rc = run(h, steps, random_seed);
    h->kp.trace = nullptr;
    h->kp.trace_n = 0;
    h->kp.trace_chains = 0;
    cudaError_t e = cudaSuccess;
    if (rc == GPR_OK) e = cudaMemcpyAsync(trace, dt, cnt * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
    if (rc == GPR_OK && e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dt);
    if (rc != GPR_OK) return rc;
    if (e != cudaSuccess) return fail(h, GPR_ERR_CUDA, "gpr_run_block_traced: %s", cudaGetErrorString(e));
    return gpr_sync(h);
}

int gpr_run_block_traced(gpr_handle* h, int steps, int random_seed, int trace_n, float* trace) {
    if (!h) return GPR_ERR_ARG;
    return gpr_run_block_traced_first(h, steps, random_seed, trace_n, h->N, trace);
}

/* ---- selection over posteriors (gpr_resample.cu) ---- */

static int ensure_select(gpr_handle* h) {
    if (!h->dkeys) {
        CUDA_TRY(h, cudaMalloc(&h->dkeys, (size_t)h->N * sizeof(unsigned long long)));
        CUDA_TRY(h, cudaMalloc(&h->dseli, 4 * sizeof(int)));
    }
    const int need = std::max(2, h->kp.nds);   /* one selected key per dataset */
    if (h->dsel_cap < need) {
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        cudaFree(h->dsel);
        h->dsel = nullptr;
        h->dsel_cap = 0;
        CUDA_TRY(h, cudaMalloc(&h->dsel, (size_t)need * sizeof(unsigned long long)));
        h->dsel_cap = need;
    }
    return GPR_OK;
}

/* The posterior at ascending rank `rank` (reference comparator order). */
static int select_rank(gpr_handle* h, int rank, unsigned long long* key) {
    int rc = ensure_select(h);
    if (rc != GPR_OK) return rc;
    CUDA_TRY(h, gpr::launch_select(h->kp, rank, h->dkeys, h->dsel, h->stream));
    h->launches += 2;
    if (key) {
        CUDA_TRY(h, cudaMemcpyAsync(key, h->dsel, sizeof *key, cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    }
    return GPR_OK;
}

int gpr_resample_datasets(gpr_handle* h, int mode, double param, uint32_t seed, int* n_redrawn,
                          double* cutoffs) {
    if (!h) return GPR_ERR_ARG;
    NvtxRange r("gpr_resample: re-draw below the cutoff");
    if (mode != 0 && mode != 1) return fail(h, GPR_ERR_ARG, "unknown resample mode %d", mode);
    if (h->cfg.n_ops < 2)
        return fail(h, GPR_ERR_ARG, "re-drawing ops needs at least 2 ops (random_int(n_ops - 1))");
    const int nseg = h->kp.nds > 0 ? h->kp.nds : 1;
    const int seg = h->N / nseg;
    int rank = seg - 1;
    if (mode == 0) {
        const double r = (double)seg * param;
        if (!(r >= 0.0 && r < (double)seg)) return fail(h, GPR_ERR_ARG, "quantile %g is not in [0, 1)", param);
        rank = (int)r;
    } else if (!(param >= 0.0)) {
        return fail(h, GPR_ERR_ARG, "map-delta %g is not >= 0", param);
    }
    CUDA_TRY(h, cudaSetDevice(h->device));
    int rc = ensure_select(h);
    if (rc != GPR_OK) return rc;
    CUDA_TRY(h, gpr::launch_select(h->kp, rank, h->dkeys, h->dsel, h->stream, nseg));
    h->launches += 2;
    CUDA_TRY(h, cudaMemsetAsync(h->dseli, 0, sizeof(int), h->stream));
    const gpr::Magic mops1 = magic_for(divisor_for(h->cfg.n_ops - 1));
    const gpr::Magic morder = magic_for(divisor_for(8));
    CUDA_TRY(h, gpr::launch_redraw(h->kp, h->dsel, nseg > 1 ? seg : 0, mode, param, seed, mops1, morder, h->dseli,
                                   h->stream));
    h->launches++;
    if (n_redrawn || cutoffs) {
        std::vector<unsigned long long> keys((size_t)nseg);
        int cnt = 0;
        CUDA_TRY(h, cudaMemcpyAsync(keys.data(), h->dsel, (size_t)nseg * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(&cnt, h->dseli, sizeof cnt, cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        if (n_redrawn) *n_redrawn = cnt;
        if (cutoffs)
            for (int d = 0; d < nseg; ++d) cutoffs[d] = gpr_key_value(keys[d]) - (mode == 1 ? param : 0.0);
    }
    return GPR_OK;
}

int gpr_resample(gpr_handle* h, int mode, double param, uint32_t seed, int* n_redrawn, double* cutoff) {
    if (!h) return GPR_ERR_ARG;
    if (h->kp.nds > 0) {   /* batched data: per dataset; the cutoffs differ */
        if (cutoff) *cutoff = std::numeric_limits<double>::quiet_NaN();
        return gpr_resample_datasets(h, mode, param, seed, n_redrawn, nullptr);
    }
    return gpr_resample_datasets(h, mode, param, seed, n_redrawn, cutoff);
}

int gpr_resample_below(gpr_handle* h, double cutoff, uint32_t seed, int chain_offset, int* n_redrawn) {
    if (!h) return GPR_ERR_ARG;
    NvtxRange r("gpr_resample_below: re-draw below a given cutoff");
    if (h->cfg.n_ops < 2)
        return fail(h, GPR_ERR_ARG, "re-drawing ops needs at least 2 ops (random_int(n_ops - 1))");
    if (chain_offset < 0) return fail(h, GPR_ERR_ARG, "chain_offset must be >= 0 (got %d)", chain_offset);
    CUDA_TRY(h, cudaSetDevice(h->device));
    int rc = ensure_select(h);
    if (rc != GPR_OK) return rc;
    /* the cutoff as a selected key (gpr_select.h keys round-trip every value) */
    const unsigned long long key = gpr_post_key(cutoff);
    CUDA_TRY(h, cudaMemcpyAsync(h->dsel, &key, sizeof key, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemsetAsync(h->dseli, 0, sizeof(int), h->stream));
    const gpr::Magic mops1 = magic_for(divisor_for(h->cfg.n_ops - 1));
    const gpr::Magic morder = magic_for(divisor_for(8));
    CUDA_TRY(h, gpr::launch_redraw(h->kp, h->dsel, 0, 0, 0.0, seed, mops1, morder, h->dseli, h->stream,
                                   (uint32_t)chain_offset));
    h->launches++;
    /* the key's host copy must outlive the asynchronous copy: wait here */
    int cnt = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&cnt, h->dseli, sizeof cnt, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (n_redrawn) *n_redrawn = cnt;
    return GPR_OK;
}

int gpr_top_chains(gpr_handle* h, int k, double margin, int* chains, int capacity, int* n, double* threshold) {
    if (!h) return GPR_ERR_ARG;
    NvtxRange r("gpr_top_chains: tops candidates");
    if (k < 1 || k > h->N) return fail(h, GPR_ERR_ARG, "k = %d is not in [1, %d]", k, h->N);
    if (!(margin >= 0.0)) return fail(h, GPR_ERR_ARG, "margin %g is not >= 0", margin);
    if (capacity < 0 || (capacity > 0 && !chains) || !n) return fail(h, GPR_ERR_ARG, "bad output arguments");
    CUDA_TRY(h, cudaSetDevice(h->device));
    unsigned long long key = 0;
    int rc = select_rank(h, h->N - k, &key);
    if (rc != GPR_OK) return rc;
    const double t = gpr_key_value(key);
    if (threshold) *threshold = t;
    /* every non-NaN chain when fewer than k are non-NaN */
    const unsigned long long kmin = key == 0ull ? 1ull : gpr_post_key(t - margin);
    if (capacity > h->dtop_cap) {
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        cudaFree(h->dtop);
        h->dtop = nullptr;
        h->dtop_cap = 0;
        CUDA_TRY(h, cudaMalloc(&h->dtop, (size_t)capacity * sizeof(int)));
        h->dtop_cap = capacity;
    }
    CUDA_TRY(h, cudaMemsetAsync(h->dseli, 0, sizeof(int), h->stream));
    CUDA_TRY(h, gpr::launch_collect(h->dkeys, h->N, kmin, h->dtop, capacity, h->dseli, h->stream));
    h->launches++;
    int cnt = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&cnt, h->dseli, sizeof cnt, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    const int m = cnt < capacity ? cnt : capacity;
    if (m > 0) {
        CUDA_TRY(h, cudaMemcpyAsync(chains, h->dtop, (size_t)m * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        std::sort(chains, chains + m);
    }
    *n = cnt;
    return GPR_OK;
}

int gpr_map_chain(gpr_handle* h, int* chain, double* posterior) {
    if (!h) return GPR_ERR_ARG;
    if (!chain) return fail(h, GPR_ERR_ARG, "chain is NULL");
    CUDA_TRY(h, cudaSetDevice(h->device));
    int rc = select_rank(h, h->N - 1, nullptr);
    if (rc != GPR_OK) return rc;
    const int big = 0x7fffffff;
    CUDA_TRY(h, cudaMemcpyAsync(h->dseli + 1, &big, sizeof big, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, gpr::launch_first_index(h->dkeys, h->N, h->dsel, h->dseli + 1, h->stream));
    h->launches++;
    unsigned long long key = 0;
    int idx = big;
    CUDA_TRY(h, cudaMemcpyAsync(&key, h->dsel, sizeof key, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(&idx, h->dseli + 1, sizeof idx, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    *chain = key == 0ull ? -1 : idx;
    if (posterior) *posterior = gpr_key_value(key);
    return GPR_OK;
}

}  /* extern "C" */

/* ------------------------------------------------------------------------ */
/* gpr_run_block_noalloc: the MH block on chain state that the caller keeps in
 * its own device memory, with everything else the kernel reads or counts in
 * one fixed scratch array per device instead of handle allocations.
 *
 * Scratch layout (bytes):
 *   [0, 8)        int[2]: [0] next chain to claim, [1] kernel error flags.
 *                 Both must be 0 when the kernel starts; every call zeroes them
 *                 on its stream before the launch.
 *   [256, ...)    logf(k) for k = 0 .. program_length + 1 (Hastings terms).
 *   [1536, ...)   x | y | w, GPR_NOALLOC_MAX_POINTS floats each, w being the
 *                 per-point likelihood weight 2^-e / (2 sd^2), e set by the
 *                 dataset's smallest sd (as gpr_set_data sets it).
 * Every call rewrites the table and the dataset before its launch, so nothing
 * left by an earlier call is read.  Two calls in flight on one device at once
 * share the array and race. */
static const size_t kNoallocLogcount = 256;
static const size_t kNoallocData = kNoallocLogcount + ((GPR_MAX_PROGRAM_LENGTH + 2) * sizeof(float) + 255) / 256 * 256;
static const size_t kNoallocBytes = kNoallocData + 3 * (size_t)GPR_NOALLOC_MAX_POINTS * sizeof(float);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

enum { kNoallocMaxDevices = 64 };
static std::mutex g_noalloc_mu;
static int g_noalloc_sms[kNoallocMaxDevices];

/* The weights of gpr_set_data, computed in place from sd on the device (the
 * same IEEE double operations and rounding as the host code), and zero
 * padding up to nd_pad, which the kernel stages with the data. */
static __global__ void noalloc_data_kernel(float* x, float* y, float* w, int n, int nd_pad, double wscale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nd_pad) return;
    if (i < n) {
        const double s = (double)w[i];
        w[i] = (float)(wscale / (2.0 * s * s));
    } else {
        x[i] = 0.0f; y[i] = 0.0f; w[i] = 0.0f;
    }
}

/* Per call, with the device current: the scratch array's device address,
 * looked up every time (cudaGetSymbolAddress allocates nothing, and an
 * address kept from an earlier call would be stale after the context was
 * reset and the module reloaded), and the SM count, cached per device (a
 * reset does not change it). */
static int noalloc_setup(int device, unsigned char** scratch, int* sms) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
        return fail(nullptr, GPR_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_sms[device]) {
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess)
            return fail(nullptr, GPR_ERR_CUDA, "cudaDeviceGetAttribute failed: %s", cudaGetErrorString(e));
        g_noalloc_sms[device] = n;
    }
    *scratch = (unsigned char*)p;
    *sms = g_noalloc_sms[device];
    return GPR_OK;
}

/* The kernel parameters gpr_create derives from a configuration, with the
 * Hastings table written to lc (program_length + 2 entries). */
static void noalloc_params(gpr::KParams& kp, const gpr_config* cfg, int n_chains, float* lc) {
    const int PL = cfg->program_length;
    memset(&kp, 0, sizeof kp);
    kp.N = n_chains; kp.PL = PL;
    kp.nv = 1;                          /* one input variable, as gpr_create's default */
    kp.rng_mode = cfg->rng;
    kp.const_mode = cfg->const_proposal;
    kp.rw_sd = cfg->rw_sd;
    kp.nops = cfg->n_ops;
    for (int i = 0; i < cfg->n_ops; ++i) kp.opmap[i] = (int8_t)cfg->ops[i];
    kp.mag_pl = magic_for(divisor_for(PL));
    kp.mag_nops = magic_for(divisor_for(cfg->n_ops));
    kp.mag_1e6 = magic_for(divisor_for(1000000));
    const double ln1 = log((double)cfg->n_ops + 1) * 0x1p-64;
    kp.ln1_hi = (float)ln1;
    kp.ln1_lo = (float)(ln1 - (double)kp.ln1_hi);
    const double PIf = 3.141592653589;
    kp.lpi_f = logf((float)PIf);
    kp.lnorm1_f = (float)(0.5 * ((double)logf((float)(2.0 * PIf)) + 2.0 * (double)logf(1.0f)));
    const float R = 0.1f, PI_INT = 0.15f;
    kp.logf_r = logf(R);
    kp.log1mr_f = (float)log(1.0 - (double)R);
    kp.log2_f = (float)log(2.0);
    kp.logpi_f = logf(PI_INT);
    kp.log1mpi_f = (float)log(1.0 - (double)PI_INT);
    kp.geom_logr = gpr_rng_logf(R);
    set_prior_constants(kp, cfg->n_ops, PL);
    kp.lockstep = 1;
    kp.stage_wait_iters = GPR_STAGE_WAIT_DEFAULT;
    kp.struct_every = 5;
    kp.hmc_eps = 0.01f;
    kp.hmc_L = 8;
    kp.hmc_jit_eps = 0.0f;
    kp.hmc_jit_len = 0.0f;
    kp.max_instr = GPR_MAX_INSTR(PL);
    int lev = 1;
    while ((1 << lev) <= PL / 2) ++lev;
    kp.levels = lev;
    gpr::fill_lcg_jump_table(kp);
    for (int k = 0; k < PL + 2; ++k) lc[k] = logf((float)k);
}

extern "C" int gpr_run_block_noalloc(const gpr_config* cfg, int n_chains, int32_t* P, float* C,
                                     double* prior, double* likelihood, const float* x,
                                     const float* y, const float* sd, int ndata, int steps,
                                     int random_seed) {
    /* arguments first, before any CUDA call */
    if (!cfg) return fail(nullptr, GPR_ERR_ARG, "cfg is NULL");
    if (n_chains <= 0) return fail(nullptr, GPR_ERR_ARG, "n_chains must be > 0 (got %d)", n_chains);
    const int PL = cfg->program_length;
    if (PL < 1 || PL > GPR_MAX_PROGRAM_LENGTH || (PL % 2) == 0)
        return fail(nullptr, GPR_ERR_ARG, "program_length must be odd and in [1, %d] (got %d)",
                    GPR_MAX_PROGRAM_LENGTH, PL);
    if (cfg->n_ops < 1 || cfg->n_ops > GPR_MAX_OPS)
        return fail(nullptr, GPR_ERR_ARG, "n_ops must be in [1, %d] (got %d)", GPR_MAX_OPS, cfg->n_ops);
    if (cfg->n_vars != 0 && cfg->n_vars != 1)
        return fail(nullptr, GPR_ERR_ARG, "gpr_run_block_noalloc takes one input variable (n_vars 0 or 1, got %d)",
                    cfg->n_vars);
    for (int i = 0; i < cfg->n_ops; ++i)
        if (cfg->ops[i] < 0 || cfg->ops[i] >= OP_NREF)
            return fail(nullptr, GPR_ERR_ARG, "ops[%d] = %d is not an op code", i, cfg->ops[i]);
    if (cfg->rng != GPR_RNG_LCG && cfg->rng != GPR_RNG_PHILOX)
        return fail(nullptr, GPR_ERR_ARG, "unknown rng mode %d", cfg->rng);
    if (cfg->const_proposal != GPR_CONST_REFERENCE && cfg->const_proposal != GPR_CONST_RANDOM_WALK)
        return fail(nullptr, GPR_ERR_ARG, "unknown constant proposal %d", cfg->const_proposal);
    if ((long long)n_chains * PL > (1ll << 31) - 1)
        return fail(nullptr, GPR_ERR_ARG, "n_chains * program_length exceeds 2^31-1");
    if (!P || !C || !prior || !likelihood)
        return fail(nullptr, GPR_ERR_ARG, "P, C, prior and likelihood must be non-NULL device pointers");
    if (steps < 0) return fail(nullptr, GPR_ERR_ARG, "steps must be >= 0 (got %d)", steps);
    if (ndata < 0) return fail(nullptr, GPR_ERR_ARG, "ndata must be >= 0");
    if (ndata > GPR_NOALLOC_MAX_POINTS)
        return fail(nullptr, GPR_ERR_ARG,
                    "ndata = %d exceeds the %d points of the no-allocation scratch; "
                    "use gpr_create and gpr_set_data for larger datasets", ndata, GPR_NOALLOC_MAX_POINTS);
    if (ndata > 0 && (!x || !y || !sd)) return fail(nullptr, GPR_ERR_ARG, "x, y, sd must be non-NULL");
    for (int i = 0; i < ndata; ++i)
        if (!(sd[i] > 0.0f)) return fail(nullptr, GPR_ERR_ARG, "sd[%d] = %g is not > 0", i, (double)sd[i]);
    if (cfg->device < 0 || cfg->device >= kNoallocMaxDevices)
        return fail(nullptr, GPR_ERR_ARG, "invalid GPU device %d", cfg->device);

    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return fail(nullptr, GPR_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
    if (cfg->device >= ndev)
        return fail(nullptr, GPR_ERR_ARG, "invalid GPU device %d (%d present)", cfg->device, ndev);
    e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) return fail(nullptr, GPR_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    unsigned char* scratch = nullptr;
    int sms = 0;
    int rc = noalloc_setup(cfg->device, &scratch, &sms);
    if (rc != GPR_OK) return rc;

    /* A handle on the stack that points at the caller's state and the
     * scratch; the launch geometry, launch and error check are the handle
     * path's own. */
    gpr_handle h;
    h.cfg = *cfg;
    h.N = n_chains;
    h.PL = PL;
    h.device = cfg->device;
    h.stream = (cudaStream_t)cfg->stream;
    h.num_sms = sms;
    h.dP = P; h.dC = C; h.dprior = prior; h.dlik = likelihood;
    h.dcounter = (int*)scratch;
    h.dlogcount = (float*)(scratch + kNoallocLogcount);
    float* sx = (float*)(scratch + kNoallocData);
    float* sy = sx + GPR_NOALLOC_MAX_POINTS;
    float* sw = sy + GPR_NOALLOC_MAX_POINTS;
    float lc[GPR_MAX_PROGRAM_LENGTH + 2];
    gpr::KParams& kp = h.kp;
    noalloc_params(kp, cfg, n_chains, lc);
    kp.P = P; kp.C = C; kp.prior = prior; kp.lik = likelihood;
    kp.logcount = h.dlogcount;
    kp.next_chain = h.dcounter;
    kp.err = h.dcounter + 1;
    kp.stats = nullptr;

    const int nd_pad = (ndata + 3) & ~3;
    double normsum = 0.0;
    const double PIf = 3.141592653589;
    for (int i = 0; i < ndata; ++i)
        normsum += 0.5 * ((double)logf((float)(2.0 * PIf)) + 2.0 * (double)logf(sd[i]));
    h.nd = ndata;
    h.nd_pad = nd_pad;
    h.normsum = normsum;
    kp.nd = ndata; kp.nd_pad = nd_pad;
    const double ns = normsum * 0x1p-64;
    kp.normsum_hi = (float)ns;
    kp.normsum_lo = (float)(ns - (double)kp.normsum_hi);
    kp.normsum64 = normsum;
    const int we = weight_exponent(sd, (size_t)ndata);
    set_weight_scale(kp, we);
    kp.dx = sx; kp.dy = sy; kp.dw = sw;

    auto report = [&](int code) { g_create_error = h.err; return code; };
#define NA_TRY(call)                                                                            \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(nullptr, GPR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)
    NA_TRY(cudaMemsetAsync(h.dcounter, 0, 2 * sizeof(int), h.stream));
    NA_TRY(cudaMemcpyAsync(h.dlogcount, lc, (PL + 2) * sizeof(float), cudaMemcpyHostToDevice, h.stream));
    if (ndata > 0) {
        NA_TRY(cudaMemcpyAsync(sx, x, ndata * sizeof(float), cudaMemcpyHostToDevice, h.stream));
        NA_TRY(cudaMemcpyAsync(sy, y, ndata * sizeof(float), cudaMemcpyHostToDevice, h.stream));
        NA_TRY(cudaMemcpyAsync(sw, sd, ndata * sizeof(float), cudaMemcpyHostToDevice, h.stream));
        noalloc_data_kernel<<<(nd_pad + 255) / 256, 256, 0, h.stream>>>(sx, sy, sw, ndata, nd_pad, ldexp(1.0, -we));
        NA_TRY(cudaGetLastError());
    }
#undef NA_TRY
    if ((rc = choose_launch(&h)) != GPR_OK) return report(rc);
    if ((rc = run(&h, steps, random_seed)) != GPR_OK) return report(rc);
    if ((rc = gpr_sync(&h)) != GPR_OK) return report(rc);
    return GPR_OK;
}
