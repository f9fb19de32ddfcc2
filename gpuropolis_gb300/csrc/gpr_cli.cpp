/*
 * gpr_cli.cpp -- the `gpuropolis` command-line tool: a drop-in for the
 * reference's main() (main.cu:1011-1257) on top of libgpuropolis.so.
 *
 * Same options (main.cu:111-129) and defaults (main.cu:96-109), same
 * samples.txt header and lines (main.cu:1087-1117, 1170-1213), same host
 * random stream (srand(seed), one rand() per block as the kernel seed, rand()
 * for the initial state and for resampling), same outer loop.  Differences:
 * errors are reported and return 1 instead of aborting on assert; N may
 * exceed the reference's 524,160-chain limit (main.cu:1059); log.txt (named
 * in the reference's README but never written by it) receives the parameter
 * block; the samples of a block are formatted on all host cores.
 *
 * Additional options (all off by default, so the defaults reproduce the
 * reference): --program-length=PL (or --max-len=PL+1), --ops=reference|basic|
 * <comma-separated op codes>, --rng=lcg|philox, --const-proposal=reference|
 * rw:SD|hmc:EPS:L|mala:EPS (gradient moves on the constants), --struct-every=K
 * (a structure move every K steps; 0: constants only), --resample=quantile:Q|
 * map-delta:D, --threads=T, --device-resample
 * (resample on the GPU from a Philox stream keyed by the block seed, without
 * copying the state back and forth), --tops=K (write tops.txt: the K
 * lines of this run's samples.txt that `sort -g -k3 | tail -n K`, run-all.sh:45,
 * selects, found with the device's top-k instead of an external sort),
 * --vars=3 (data lines "x1 x2 x3 y sd"; the op set then also holds the leaves
 * x1, x2, x3, op codes 27-29, unless --ops gives one), --adapt=T (random-walk
 * and gradient moves: each chain's own scale adapted toward acceptance T
 * during the blocks not written out, 0..burn, then kept), --hmc-jitter=A:B
 * (gradient moves: each move's leapfrog step drawn from EPS x U(1-A, 1+A) and
 * its count from [L(1-B), L(1+B)]), --checkpoint=FILE
 * (after every block: the chains, the seed and the host stream's position)
 * and --resume=FILE (continue from such a file, appending to samples.txt:
 * the continued run writes what the uninterrupted one would have).
 */
#include <nvtx3/nvToolsExt.h>
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/gpuropolis.h"
#include "../../include/gpuropolis_host.h"

static float sdscale = 1.0f;
static int N = 1024, steps = 1000, outer = 100, thin = 1, seed = -1, burn = 0, QUIET = 0;
static int WHICH_GPU = 0, FIRST_HALF_DATA = 0, EVEN_HALF_DATA = 0, SHOW_CONSTANTS = 0;
static std::string in_file_path = "data.txt", out_path = "out/";
static int PL = 31, rng_mode = GPR_RNG_LCG, const_mode = GPR_CONST_REFERENCE, threads = 0;
static float rw_sd = 0.1f, hmc_eps = 0.01f;
static int hmc_steps = 8, struct_every = 5;
static int resample_mode = GPR_RESAMPLE_QUANTILE;
static double resample_param = 0.5;
static int device_resample = 0, tops_k = 0;
static int n_vars = 1, ops_given = 0;
static float adapt_target = 0.0f;
static float jit_eps = 0.0f, jit_len = 0.0f;
static std::string ckpt_path, resume_path;
static std::vector<int> ops;

enum { OPT_PL = 1000, OPT_MAXLEN, OPT_OPS, OPT_RNG, OPT_CONST, OPT_RESAMPLE, OPT_THREADS, OPT_DEVRES, OPT_TOPS, OPT_STRUCT,
       OPT_VARS, OPT_ADAPT, OPT_CKPT, OPT_RESUME, OPT_JITTER };

static struct option long_options[] = {
    {"in", required_argument, NULL, 'd'},
    {"steps", required_argument, NULL, 'i'},
    {"N", required_argument, NULL, 'N'},
    {"out", required_argument, NULL, 'O'},
    {"outer", required_argument, NULL, 'o'},
    {"thin", required_argument, NULL, 't'},
    {"seed", required_argument, NULL, 's'},
    {"burn", required_argument, NULL, 'b'},
    {"gpu", required_argument, NULL, 'g'},
    {"sdscale", required_argument, NULL, 'r'},
    {"first-half", no_argument, NULL, 'f'},
    {"even-half", no_argument, NULL, 'e'},
    {"show-constants", no_argument, NULL, 'C'},
    {"quiet", no_argument, NULL, 'q'},
    {"all", no_argument, NULL, '_'},
    {"program-length", required_argument, NULL, OPT_PL},
    {"max-len", required_argument, NULL, OPT_MAXLEN},
    {"ops", required_argument, NULL, OPT_OPS},
    {"rng", required_argument, NULL, OPT_RNG},
    {"const-proposal", required_argument, NULL, OPT_CONST},
    {"resample", required_argument, NULL, OPT_RESAMPLE},
    {"threads", required_argument, NULL, OPT_THREADS},
    {"device-resample", no_argument, NULL, OPT_DEVRES},
    {"tops", required_argument, NULL, OPT_TOPS},
    {"struct-every", required_argument, NULL, OPT_STRUCT},
    {"vars", required_argument, NULL, OPT_VARS},
    {"adapt", required_argument, NULL, OPT_ADAPT},
    {"checkpoint", required_argument, NULL, OPT_CKPT},
    {"resume", required_argument, NULL, OPT_RESUME},
    {"hmc-jitter", required_argument, NULL, OPT_JITTER},
    {NULL, 0, 0, 0}};

static int parse_ops(const char* s) {
    ops.clear();
    if (!strcmp(s, "reference")) { for (int i = 0; i < 27; ++i) ops.push_back(i); return 0; }
    if (!strcmp(s, "basic")) { ops = {1, 3, 4, 5, 6, 9, 11, 13, 14, 15}; return 0; }
    std::string t(s);
    size_t p = 0;
    while (p <= t.size()) {
        size_t q = t.find(',', p);
        std::string tok = t.substr(p, q == std::string::npos ? std::string::npos : q - p);
        if (tok.empty()) return 1;
        ops.push_back(atoi(tok.c_str()));
        if (q == std::string::npos) break;
        p = q + 1;
    }
    return ops.empty();
}

static int process_arguments(int argc, char** argv) {
    int option_index = 0, opt = 0;
    while ((opt = getopt_long(argc, argv, "bp", long_options, &option_index)) != -1) switch (opt) {
            case 'd': in_file_path = optarg; break;
            case 'i': steps = atoi(optarg); break;
            case 'N': N = atoi(optarg); break;
            case 'o': outer = atoi(optarg); break;
            case 'O': out_path = optarg; break;
            case 't': thin = atoi(optarg); break;
            case 'b': burn = atoi(optarg); break;
            case 'g': WHICH_GPU = atoi(optarg); break;
            case 's': seed = atoi(optarg); break;
            case 'r': sdscale = (float)atof(optarg); break;
            case 'f': FIRST_HALF_DATA = 1; break;
            case 'e': EVEN_HALF_DATA = 1; break;
            case 'C': SHOW_CONSTANTS = 1; break;
            case 'q': QUIET = 1; break;
            case '_': break;
            case OPT_PL: PL = atoi(optarg); break;
            case OPT_MAXLEN: PL = atoi(optarg) - 1; break;
            case OPT_OPS: if (parse_ops(optarg)) return 1; ops_given = 1; break;
            case OPT_VARS: n_vars = atoi(optarg); if (n_vars != 1 && n_vars != 3) return 1; break;
            case OPT_CKPT: ckpt_path = optarg; break;
            case OPT_RESUME: resume_path = optarg; break;
            case OPT_ADAPT:
                adapt_target = (float)atof(optarg);
                if (!(adapt_target > 0.0f && adapt_target < 1.0f)) return 1;
                break;
            case OPT_RNG:
                if (!strcmp(optarg, "lcg")) rng_mode = GPR_RNG_LCG;
                else if (!strcmp(optarg, "philox")) rng_mode = GPR_RNG_PHILOX;
                else return 1;
                break;
            case OPT_CONST:
                if (!strcmp(optarg, "reference")) const_mode = GPR_CONST_REFERENCE;
                else if (!strncmp(optarg, "rw:", 3)) { const_mode = GPR_CONST_RANDOM_WALK; rw_sd = (float)atof(optarg + 3); }
                else if (!strncmp(optarg, "hmc:", 4)) {
                    const_mode = GPR_CONST_HMC;
                    if (sscanf(optarg + 4, "%f:%d", &hmc_eps, &hmc_steps) != 2) return 1;
                }
                else if (!strncmp(optarg, "mala:", 5)) {
                    const_mode = GPR_CONST_HMC;
                    hmc_steps = 1;
                    if (sscanf(optarg + 5, "%f", &hmc_eps) != 1) return 1;
                }
                else return 1;
                break;
            case OPT_RESAMPLE:
                if (!strncmp(optarg, "quantile:", 9)) { resample_mode = GPR_RESAMPLE_QUANTILE; resample_param = atof(optarg + 9); }
                else if (!strncmp(optarg, "map-delta:", 10)) { resample_mode = GPR_RESAMPLE_MAP_DELTA; resample_param = atof(optarg + 10); }
                else return 1;
                break;
            case OPT_THREADS: threads = atoi(optarg); break;
            case OPT_DEVRES: device_resample = 1; break;
            case OPT_TOPS: tops_k = atoi(optarg); if (tops_k < 1) return 1; break;
            case OPT_STRUCT: struct_every = atoi(optarg); if (struct_every < 0) return 1; break;
            case OPT_JITTER:
                if (sscanf(optarg, "%f:%f", &jit_eps, &jit_len) != 2) return 1;
                if (!(jit_eps >= 0.0f && jit_eps < 1.0f && jit_len >= 0.0f && jit_len <= 1.0f)) return 1;
                break;
            default: return 1;
        }
    return 0;
}

static void progress_bar(float pct) {   /* main.cu:997-1008 */
    fprintf(stderr, "\r[");
    for (int p = 0; p < 70; p++) fprintf(stderr, p <= pct * 70 ? "=" : " ");
    fprintf(stderr, "]");
}

static void write_params(FILE* fp, int ndata, int wgpu) {   /* main.cu:1090-1104 */
    fprintf(fp, "# -----------------------------------------------------------------\n");
    fprintf(fp, "# -- Parameters:\n");
    fprintf(fp, "# -----------------------------------------------------------------\n");
    fprintf(fp, "# \tInput data path: %s\n", in_file_path.c_str());
    fprintf(fp, "# \tOutput path: %s\n", out_path.c_str());
    fprintf(fp, "# \tMCMC Iterations (per block): %i\n", steps);
    fprintf(fp, "# \tBlocks: %i\n", outer);
    fprintf(fp, "# \tN chains: %i\n", N);
    fprintf(fp, "# \tSeed: %i\n", seed);
    fprintf(fp, "# \tMax program length: %i\n", PL);
    fprintf(fp, "# \tN Constants: %i\n", PL);
    fprintf(fp, "# \tGPU: %i\n", wgpu);
    fprintf(fp, "# \tNumber of data points: %i\n", ndata);
    fprintf(fp, "#\n#\n");
}

#define FAIL(...) do { fprintf(stderr, __VA_ARGS__); fprintf(stderr, "\n"); return 1; } while (0)

/* Checkpoint file: "GPRCKPT1", int32 {version 1, N, PL, n_vars, n_ops, last
 * block done, seed, 0}, uint64 host rand() calls, int32 ops[n_ops], int32
 * P[N*PL], float C[N*PL] (the reference layout). */
static const char CKPT_MAGIC[8] = {'G', 'P', 'R', 'C', 'K', 'P', 'T', '1'};

static bool write_checkpoint(const std::string& path, int block, const std::vector<int32_t>& P,
                             const std::vector<float>& C) {
    const std::string tmp = path + ".tmp";
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return false;
    const int32_t hdr[8] = {1, N, PL, n_vars, (int32_t)ops.size(), block, seed, 0};
    const uint64_t calls = gpr_host_rand_calls();
    bool ok = fwrite(CKPT_MAGIC, 1, 8, f) == 8 && fwrite(hdr, sizeof hdr, 1, f) == 1 &&
              fwrite(&calls, sizeof calls, 1, f) == 1 &&
              fwrite(ops.data(), sizeof(int32_t), ops.size(), f) == ops.size() &&
              fwrite(P.data(), sizeof(int32_t), P.size(), f) == P.size() &&
              fwrite(C.data(), sizeof(float), C.size(), f) == C.size();
    ok = (fclose(f) == 0) && ok;
    return ok && rename(tmp.c_str(), path.c_str()) == 0;   /* a crash mid-write keeps the last good one */
}

/* Reads a checkpoint written with the same chains, program length, variables
 * and op set; returns the last block done (or -1) and sets seed and the stream
 * position. */
static int read_checkpoint(const std::string& path, std::vector<int32_t>& P, std::vector<float>& C,
                           uint64_t* calls, std::string& err) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) { err = "cannot open checkpoint " + path; return -1; }
    char magic[8];
    int32_t hdr[8];
    std::vector<int32_t> ck_ops;
    bool ok = fread(magic, 1, 8, f) == 8 && !memcmp(magic, CKPT_MAGIC, 8) && fread(hdr, sizeof hdr, 1, f) == 1 &&
              hdr[0] == 1 && fread(calls, sizeof *calls, 1, f) == 1;
    if (ok && (hdr[1] != N || hdr[2] != PL || hdr[3] != n_vars || hdr[4] != (int32_t)ops.size()))
        { err = "checkpoint was written for other chains, program length, variables or op set"; ok = false; }
    if (ok) {
        ck_ops.resize((size_t)hdr[4]);
        ok = fread(ck_ops.data(), sizeof(int32_t), ck_ops.size(), f) == ck_ops.size() &&
             std::equal(ck_ops.begin(), ck_ops.end(), ops.begin());
        if (!ok) err = "checkpoint was written for another op set";
    }
    if (ok) ok = fread(P.data(), sizeof(int32_t), P.size(), f) == P.size() &&
                 fread(C.data(), sizeof(float), C.size(), f) == C.size();
    fclose(f);
    if (!ok) { if (err.empty()) err = "checkpoint " + path + " is truncated or not a checkpoint"; return -1; }
    seed = hdr[6];
    return hdr[5];
}

int main(int argc, char** argv) {
    for (int i = 0; i < 27; ++i) ops.push_back(i);
    if (process_arguments(argc, argv) == 1) {
        fprintf(stderr, "Invalid command line arguments.\n");
        return 1;
    }
    if (!(steps > 0)) FAIL("steps must be > 0");          /* main.cu:1028-1031 */
    if (!(N > 0)) FAIL("N must be > 0");
    if (!(burn >= 0)) FAIL("burn must be >= 0");
    if (!(thin >= 1)) FAIL("thin must be >= 1");
    if (resample_mode == GPR_RESAMPLE_QUANTILE ? !(resample_param >= 0.0 && resample_param < 1.0) : !(resample_param >= 0.0))
        FAIL("--resample: the quantile must be in [0, 1), the MAP delta >= 0");
    if (adapt_target > 0.0f && (!ckpt_path.empty() || !resume_path.empty()))
        FAIL("--checkpoint / --resume do not keep the adaptation's state; run --adapt without them");
    if (adapt_target > 0.0f && const_mode == GPR_CONST_REFERENCE)
        FAIL("--adapt needs --const-proposal=rw:SD, hmc:EPS:L or mala:EPS (the reference's proposals have no scale)");
    if ((jit_eps > 0.0f || jit_len > 0.0f) && const_mode != GPR_CONST_HMC)
        FAIL("--hmc-jitter needs --const-proposal=hmc:EPS:L or mala:EPS");

    if (n_vars == 3 && !ops_given)
        for (int o = 27; o <= 29; ++o) ops.push_back(o);   /* the reference's ops and x1, x2, x3 */
    gpr_config cfg;
    gpr_default_config(&cfg);
    cfg.n_vars = n_vars;
    cfg.program_length = PL;
    cfg.n_ops = (int)ops.size();
    if (cfg.n_ops > GPR_MAX_OPS) FAIL("too many ops");
    for (int i = 0; i < cfg.n_ops; ++i) cfg.ops[i] = ops[i];
    cfg.rng = rng_mode;
    cfg.const_proposal = const_mode;
    cfg.rw_sd = rw_sd;
    cfg.device = WHICH_GPU;
    gpr_handle* h = nullptr;
    if (gpr_create(&cfg, N, &h) != GPR_OK) {
        fprintf(stderr, "%s\n", gpr_last_error(nullptr));
        if (strstr(gpr_last_error(nullptr), "invalid GPU device"))
            fprintf(stderr, "Invalid GPU device %d\n", WHICH_GPU);   /* main.cu:1045 */
        return 1;
    }
    if (gpr_set_moves(h, struct_every, hmc_eps, hmc_steps) != GPR_OK ||
        (const_mode == GPR_CONST_HMC && gpr_set_hmc_jitter(h, jit_eps, jit_len) != GPR_OK)) {
        fprintf(stderr, "%s\n", gpr_last_error(h));
        gpr_destroy(h);
        return 1;
    }
    const int wgpu = WHICH_GPU;
    /* a resumed run takes its chains, seed and host-stream position from the checkpoint */
    const size_t cnt = (size_t)N * PL;
    std::vector<int32_t> ckP;
    std::vector<float> ckC;
    uint64_t ck_calls = 0;
    int o_start = 0;
    if (!resume_path.empty()) {
        ckP.resize(cnt);
        ckC.resize(cnt);
        std::string err;
        const int last = read_checkpoint(resume_path, ckP, ckC, &ck_calls, err);
        if (last < 0) { fprintf(stderr, "*** ERROR: %s\n", err.c_str()); gpr_destroy(h); return 1; }
        o_start = last + 1;
    }
    std::string SAMPLE_PATH = out_path + "/samples.txt";
    std::string LOG_PATH = out_path + "/log.txt";
    if (seed == -1) seed = (int)time(NULL);

    float *x = nullptr, *y = nullptr, *sd = nullptr, *x2 = nullptr, *x3 = nullptr;
    int ndata = 0;
    int rc = n_vars == 3
        ? gpr_load_data_file3(in_file_path.c_str(), sdscale, FIRST_HALF_DATA, EVEN_HALF_DATA, &x, &x2, &x3, &y, &sd,
                              &ndata)
        : gpr_load_data_file(in_file_path.c_str(), sdscale, FIRST_HALF_DATA, EVEN_HALF_DATA, &x, &y, &sd, &ndata);
    if (rc != GPR_HOST_OK) { fprintf(stderr, "*** ERROR: %s\n", gpr_host_last_error()); gpr_destroy(h); return 1; }

    FILE* fp = fopen(SAMPLE_PATH.c_str(), "a");
    if (!fp) { fprintf(stderr, "*** ERROR: Cannot open file:\t%s\n", SAMPLE_PATH.c_str()); gpr_destroy(h); return 1; }
    char* head = nullptr;
    size_t head_len = 0;
    FILE* hs = open_memstream(&head, &head_len);
    if (!hs) { fclose(fp); gpr_destroy(h); FAIL("out of memory"); }
    write_params(hs, ndata, wgpu);
    gpr_host_srand((unsigned)seed);                     /* main.cu:1107 */
    fprintf(hs, "# -----------------------------------------------------------------\n");
    fprintf(hs, "# -- Data:\n");
    fprintf(hs, "# -----------------------------------------------------------------\n");
    for (int i = 0; i < ndata; i++) {
        if (n_vars == 3) fprintf(hs, "# \t%f\t%f\t%f\t%f\t%f\n", x[i], x2[i], x3[i], y[i], sd[i]);
        else fprintf(hs, "# \t%f\t%f\t%f\n", x[i], y[i], sd[i]);
    }
    fprintf(hs, "#\n#\n");
    fclose(hs);
    if (resume_path.empty()) fwrite(head, 1, head_len, fp);   /* a resumed run appends to its samples */
    fclose(fp);
    gpr_tops* tops = tops_k > 0 ? gpr_tops_new(tops_k) : nullptr;
    if (tops && resume_path.empty()) gpr_tops_add_text(tops, head, (int64_t)head_len);
    free(head);

    FILE* lg = fopen(LOG_PATH.c_str(), "a");
    if (lg) {
        write_params(lg, ndata, wgpu);
        fprintf(lg, "# \tRNG: %s\n# \tConstant proposal: %s", rng_mode == GPR_RNG_PHILOX ? "philox" : "lcg",
                const_mode == GPR_CONST_RANDOM_WALK ? "rw:" : const_mode == GPR_CONST_HMC ? "hmc:" : "reference");
        if (const_mode == GPR_CONST_RANDOM_WALK) fprintf(lg, "%g", rw_sd);
        if (const_mode == GPR_CONST_HMC) fprintf(lg, "%g:%d", hmc_eps, hmc_steps);
        if (const_mode == GPR_CONST_HMC && (jit_eps > 0.0f || jit_len > 0.0f))
            fprintf(lg, " (jitter %g:%g)", jit_eps, jit_len);
        fprintf(lg, "\n# \tStructure move every: %d steps", struct_every);
        if (adapt_target > 0.0f) fprintf(lg, "\n# \tAdapt: per-chain scales toward acceptance %g in blocks 0..%d", adapt_target, burn);
        fprintf(lg, "\n# \tResample: %s:%g%s\n# \tOps:", resample_mode == GPR_RESAMPLE_MAP_DELTA ? "map-delta" : "quantile",
                resample_param, device_resample ? " (device)" : "");
        for (int o : ops) fprintf(lg, " %d", o);
        fprintf(lg, "\n# \tLibrary: %s\n", gpr_version());
        if (!resume_path.empty()) fprintf(lg, "# \tResumed from %s after block %d\n", resume_path.c_str(), o_start - 1);
    }

    std::vector<int32_t> P(cnt);
    std::vector<float> C(cnt);
    std::vector<double> prior(N), lik(N);
    gpr_host_init_chains(P.data(), C.data(), N, PL, ops.data(), (int)ops.size());   /* main.cu:1133-1137 */
    if (!resume_path.empty()) {
        P.swap(ckP);
        C.swap(ckC);
        gpr_host_srand((unsigned)seed);                 /* the host stream where the checkpoint left it */
        gpr_host_rand_skip(ck_calls);
    }

    const int drc = n_vars == 3 ? gpr_set_data3(h, x, x2, x3, y, sd, ndata) : gpr_set_data(h, x, y, sd, ndata);
    if (drc != GPR_OK || gpr_set_state(h, P.data(), C.data()) != GPR_OK) {
        fprintf(stderr, "%s\n", gpr_last_error(h));
        gpr_destroy(h);
        return 1;
    }
    if (!QUIET) progress_bar(0.0f);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    std::vector<int> cand(tops ? (size_t)N : 0);
    float adapting = 0.0f;
    for (int o = o_start; o < outer; o++) {
        /* per-chain scales adapt while the blocks are not written out, then stay */
        const float want = (adapt_target > 0.0f && o <= burn) ? adapt_target : 0.0f;
        if (want != adapting || (o == 0 && want > 0.0f)) {
            if (gpr_adapt_scales(h, want) != GPR_OK) {
                fprintf(stderr, "%s\n", gpr_last_error(h));
                gpr_destroy(h);
                return 1;
            }
            adapting = want;
        }
        int block_seed = gpr_host_rand();                /* main.cu:1160 */
        const bool write = o > burn && o % thin == 0;    /* main.cu:1170 */
        if (gpr_run_block(h, steps, block_seed) != GPR_OK ||
            ((write || !device_resample) &&
             gpr_get_state(h, P.data(), C.data(), prior.data(), lik.data()) != GPR_OK)) {
            fprintf(stderr, "CUDA error: %s\n", gpr_last_error(h));
            gpr_destroy(h);
            return 1;
        }
        if (write) {
            nvtxRangePushA("samples.txt: format and write");
            char* buf = nullptr;
            int64_t n = gpr_format_samples(P.data(), C.data(), prior.data(), lik.data(), N, PL, o,
                                           SHOW_CONSTANTS, threads, &buf);
            fp = fopen(SAMPLE_PATH.c_str(), "a");
            if (fp && n > 0) fwrite(buf, 1, (size_t)n, fp);
            if (fp) fclose(fp);
            if (tops && n > 0) {
                /* candidates: the chains within 0.002 of the K-th best posterior,
                 * more than the %.3f rounding can move a line past it */
                int nc = 0;
                double thr = 0.0;
                if (tops_k >= N || gpr_top_chains(h, tops_k, 0.002, cand.data(), N, &nc, &thr) != GPR_OK ||
                    thr != thr) {
                    gpr_tops_add_text(tops, buf, n);
                } else {
                    gpr_tops_add_lines(tops, buf, n, cand.data(), nc < N ? nc : N);
                }
            }
            gpr_free(buf);
            nvtxRangePop();
        }
        if (device_resample) {
            /* keyed by the block seed: the re-draw streams (seed, chain | 2^31)
             * never meet the block's own (seed, chain), and the host rand()
             * stream stays the one the host path draws when nothing is re-drawn */
            if (gpr_resample(h, resample_mode, resample_param, (uint32_t)block_seed, nullptr, nullptr) != GPR_OK) {
                fprintf(stderr, "CUDA error: %s\n", gpr_last_error(h));
                gpr_destroy(h);
                return 1;
            }
        } else {
            if (gpr_host_resample(P.data(), C.data(), prior.data(), lik.data(), N, PL, ops.data(), (int)ops.size(),
                                  resample_mode, resample_param) < 0) {
                fprintf(stderr, "*** ERROR: %s\n", gpr_host_last_error());
                gpr_destroy(h);
                return 1;
            }
            if (gpr_set_state(h, P.data(), C.data()) != GPR_OK) {
                fprintf(stderr, "CUDA error: %s\n", gpr_last_error(h));
                gpr_destroy(h);
                return 1;
            }
        }
        if (!ckpt_path.empty()) {
            /* the device resampling leaves the host copy behind: refresh it first */
            if ((device_resample && gpr_get_state(h, P.data(), C.data(), nullptr, nullptr) != GPR_OK) ||
                !write_checkpoint(ckpt_path, o, P, C)) {
                fprintf(stderr, "*** ERROR: cannot write checkpoint %s (%s)\n", ckpt_path.c_str(), gpr_last_error(h));
                gpr_destroy(h);
                return 1;
            }
        }
        if (!QUIET) progress_bar(float(o) / float(outer));
    }
    if (tops) {
        std::string TOPS_PATH = out_path + "/tops.txt";
        if (gpr_tops_write(tops, TOPS_PATH.c_str()) < 0)
            fprintf(stderr, "*** ERROR: Cannot write file:\t%s\n", TOPS_PATH.c_str());
        gpr_tops_free(tops);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (!QUIET) progress_bar(1.1f);
    fprintf(stderr, " Completed. \n");
    if (lg) {
        double s = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
        fprintf(lg, "# \tSampling wall time (s): %.3f\n# \tChain-steps/s: %.4g\n", s,
                (double)N * steps * (outer - o_start) / (s > 0 ? s : 1e-9));
        fclose(lg);
    }
    gpr_free(x); gpr_free(y); gpr_free(sd); gpr_free(x2); gpr_free(x3);
    gpr_destroy(h);
    return 0;
}
