/*
 * ref_entry.cpp -- C entry points around the reference's own code, compiled
 * on the host (TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's
 * CPU baseline, never by the product).
 *
 * It #includes the substituted copy of main.cu that oracle/build_ref.py
 * writes to oracle/_ref/src/, so every function below calls the reference's
 * code unchanged: program_fold/call (main.cu:371-448), compute_likelihood
 * (main.cu:454-468), compute_prior (main.cu:529-544), count_nodes
 * (main.cu:604-608), polynomial_degree (main.cu:652-654), is_descendant
 * (main.cu:660-677), MH_simple_kernel (main.cu:679-813), displaystring /
 * display_latex (main.cu:878-976), the device and host RNG helpers
 * (main.cu:213-293) and main() itself (main.cu:1011-1257, renamed).
 */
#include "gpr_ref_main.inc"

extern "C" {

int gpr_ref_program_length(void) { return PROGRAM_LENGTH; }
int gpr_ref_nops(void) { return GPR_NOPS; }
int gpr_ref_nops_enum(void) { return NOPS; }
int gpr_ref_opmap(int k) { return GPR_OPMAP(k); }
int gpr_ref_rng_is_philox(void) { return GPR_REF_PHILOX; }
const char* gpr_ref_program_code(void) { return PROGRAM_CODE; }

/* One block of MH steps over all chains (the launch at main.cu:1160). */
void gpr_ref_run_kernel(int N, int* P, float* C, const float* D_xysd, int ndata, int steps,
                        double* prior, double* likelihood, int random_seed, int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
    int nb = N / (int)BLOCK_SIZE + (N % (int)BLOCK_SIZE == 0 ? 0 : 1);
    gpr_ref_launch(nb, (int)BLOCK_SIZE, N, P, C, (datum*)D_xysd, ndata, steps, prior, likelihood,
                   random_seed);
}

/* The same, restricted to chains [c0, c1) -- for bounded CPU-baseline samples. */
void gpr_ref_run_kernel_range(int N, int c0, int c1, int* P, float* C, const float* D_xysd,
                              int ndata, int steps, double* prior, double* likelihood,
                              int random_seed, int nthreads) {
    if (nthreads > 0) omp_set_num_threads(nthreads);
    const int bs = (int)BLOCK_SIZE;
    #pragma omp parallel for schedule(dynamic, 1)
    for (int idx = c0; idx < c1; ++idx) {
        blockIdx.x = (unsigned)(idx / bs); threadIdx.x = (unsigned)(idx % bs); blockDim.x = (unsigned)bs;
        MH_simple_kernel(N, P, C, (datum*)D_xysd, ndata, steps, prior, likelihood, random_seed);
    }
}

double gpr_ref_prior(int N, int idx, int* P, float* C) { return compute_prior(N, idx, P, C); }
double gpr_ref_likelihood(int N, int idx, int* P, float* C, const float* D_xysd, int ndata) {
    return compute_likelihood(N, idx, P, C, (datum*)D_xysd, ndata);
}
int gpr_ref_count_nodes(int N, int idx, int* P, float* C) { return count_nodes(N, idx, P, C); }
float gpr_ref_length(int N, int idx, int* P, float* C) {
    return program_fold<float>(N, idx, P, C, X_LENGTH_PRIOR, dispatch_length);
}
float gpr_ref_call(int N, int idx, int* P, float* C, float x) { return call(N, idx, P, C, x); }
float gpr_ref_degree(int N, int idx, int* P, float* C) { return polynomial_degree(N, idx, P, C); }
int gpr_ref_is_descendant(int n, int k) { return is_descendant(n, k); }
double gpr_ref_lnormalpdf(float x, float s) { return lnormalpdf(x, s); }
double gpr_ref_lcauchypdf(float x, float s) { return lcauchypdf(x, s); }

/* which: 0 = displaystring, 1 = display_latex.  Returns the length written. */
int gpr_ref_display(const char* fmt, int N, int idx, int* P, float* C, int which, char* out, int cap) {
    char* buf = NULL; size_t len = 0;
    FILE* fp = open_memstream(&buf, &len);
    if (which == 0) displaystring(fmt, N, idx, P, C, fp);
    else display_latex(fmt, N, idx, P, C, fp);
    fclose(fp);
    int n = (int)len;
    if (cap > 0) {
        int m = n < cap - 1 ? n : cap - 1;
        memcpy(out, buf, (size_t)m);
        out[m] = 0;
    }
    free(buf);
    return n;
}

/* Device RNG helpers (main.cu:213-254) on an explicit stream state. */
int gpr_ref_dev_rand(void* st) { return cuda_rand(*(GPR_RNG_T*)st); }
int gpr_ref_dev_random_int(int n, void* st) { return random_int(n, *(GPR_RNG_T*)st); }
float gpr_ref_dev_random_float(void* st) { return random_float(*(GPR_RNG_T*)st); }
float gpr_ref_dev_random_normal(void* st) { return random_normal(*(GPR_RNG_T*)st); }
float gpr_ref_dev_random_geometric(float r, void* st) { return random_geometric(r, *(GPR_RNG_T*)st); }
void gpr_ref_dev_seed(void* st, int seed, int idx) { GPR_RNG_SEED(*(GPR_RNG_T*)st, seed, idx); }
int gpr_ref_dev_state_size(void) { return (int)sizeof(GPR_RNG_T); }

/* Host RNG helpers (main.cu:262-293), glibc rand(). */
void gpr_ref_srand(unsigned s) { srand(s); }
int gpr_ref_rand(void) { return rand(); }
int gpr_ref_host_random_int(int limit) { return random_int(limit); }
float gpr_ref_host_random_normal(void) { return random_normal(); }

/* load_data_file (main.cu:319-363) with the global sdscale it reads; writes
 * up to cap points as (x, y, sd) triples.  Exits the process on bad input,
 * like the reference, so callers only pass valid files. */
int gpr_ref_load_data(const char* path, float scale, int first_half, int even_half, float* out, int cap) {
    sdscale = scale;
    vector<datum>* d = load_data_file(path, first_half, even_half);
    int n = (int)d->size();
    for (int i = 0; i < n && i < cap; ++i) {
        out[3 * i] = (*d)[i].x; out[3 * i + 1] = (*d)[i].y; out[3 * i + 2] = (*d)[i].sd;
    }
    delete d;
    return n;
}

/* The initialisation statements of main() (main.cu:1133-1137) on caller
 * buffers, after srand(seed) (main.cu:1107), using the reference's own host
 * random_int / random_normal. */
void gpr_ref_host_init(int* P, float* C, int N, unsigned seed) {
    srand(seed);
    for (int i = 0; i < PROGRAM_LENGTH * N; i++) P[i] = GPR_OPMAP(random_int(GPR_NOPS - 1));
    for (int i = 0; i < NCONSTANTS * N; i++) {
        int order = random_int(C_MAX_ORDER - C_MIN_ORDER) + C_MIN_ORDER;
        C[i] = CONSTANT_SCALE * powf(10.0, order) * random_normal();
    }
}

/* The cutoff statements of main() (main.cu:1215-1219) on caller arrays, with
 * the reference's own comparator cmp (main.cu:987-995); flags[h] = 1 for the
 * chains the test of main.cu:1223 re-draws. */
double gpr_ref_resample_cutoff(int N, const double* prior, const double* lik, int* flags) {
    bayes_t* host_posterior = (bayes_t*)malloc((size_t)N * sizeof(bayes_t));
    for (int h = 0; h < N; h++) host_posterior[h] = prior[h] + lik[h];
    qsort((void*)host_posterior, N, sizeof(bayes_t), cmp);
#if GPR_REF_MAPD
    bayes_t cutoff = host_posterior[N - 1] - (GPR_REF_MAP_DELTA);
#else
    bayes_t cutoff = host_posterior[int(N * RESAMPLE_QUANTILE)];
#endif
    free(host_posterior);
    for (int h = 0; h < N; h++) flags[h] = (prior[h] + lik[h] < cutoff) ? 1 : 0;
    return cutoff;
}

/* The reference's main() (main.cu:1011), renamed. */
int gpr_ref_cli(int argc, char** argv) { optind = 1; return gpr_ref_main(argc, argv); }

}  /* extern "C" */

#if defined(GPR_REF_WITH_MAIN)
int main(int argc, char** argv) { return gpr_ref_main(argc, argv); }
#endif
