/*
 * gpuropolis_host.h -- host-side half of the drop-in (libgpuropolis.so):
 * the data loader, the samples.txt formatter and the host-RNG initialisation
 * and resampling of chains, i.e. the parts of the reference's main.cu that
 * surround its kernel launch.  Pure CPU code; no CUDA call is made here.
 *
 * State arrays use the reference layout P[i*N + chain], C[i*N + chain].
 */
#ifndef GPUROPOLIS_HOST_H
#define GPUROPOLIS_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { GPR_HOST_OK = 0, GPR_HOST_ERR_ARG = 1, GPR_HOST_ERR_IO = 2, GPR_HOST_ERR_DATA = 3 };
enum { GPR_RESAMPLE_QUANTILE = 0, GPR_RESAMPLE_MAP_DELTA = 1 };

/* load_data_file (main.cu:319-363): lines "x<ws>y<ws>sd" (%lf, then %le),
 * '#' comment lines and blank lines skipped, sd multiplied by sdscale and
 * required > 0, optional first-half / even-half trims.  On success *x, *y, *sd
 * are malloc'ed arrays of *n floats (release with gpr_free).  Errors return a
 * GPR_HOST_ERR_* code (the reference exits) and set gpr_host_last_error(). */
int gpr_load_data_file(const char* path, float sdscale, int first_half, int even_half,
                       float** x, float** y, float** sd, int* n);

/* Data with three input variables (no reference counterpart): lines
 * "x1 x2 x3 y sd", the variables in front of the reference's y and sd, with
 * the same parse rules, sdscale and trims as gpr_load_data_file.  On success
 * *x1, *x2, *x3, *y, *sd are malloc'ed arrays of *n floats. */
int gpr_load_data_file3(const char* path, float sdscale, int first_half, int even_half, float** x1, float** x2,
                        float** x3, float** y, float** sd, int* n);
void gpr_free(void* p);
const char* gpr_host_last_error(void);

/* displaystring (main.cu:878-898) when latex == 0, display_latex
 * (main.cu:956-976) when latex != 0, for chain idx, constants printed with
 * the printf format cfmt ("C", "%.10f", "%.2f" in the reference).  Writes at
 * most cap-1 bytes plus a NUL to out; returns the full length. */
int gpr_format_expression(const int32_t* P, const float* C, int N, int PL, int idx, const char* cfmt,
                          int latex, char* out, int cap);

/* Description length (program_fold with dispatch_length, main.cu:1178) and
 * polynomial degree (main.cu:652-654; INFINITY when not a polynomial). */
float gpr_program_length_of(const int32_t* P, const float* C, int N, int PL, int idx);
float gpr_polynomial_degree(const int32_t* P, const float* C, int N, int PL, int idx);

/* The samples.txt lines of one block for all N chains (main.cu:1173-1210),
 * formatted on nthreads threads (0 = all cores), concatenated in chain order.
 * *out is malloc'ed (gpr_free); returns its length or -1. */
int64_t gpr_format_samples(const int32_t* P, const float* C, const double* prior, const double* lik,
                           int N, int PL, int block, int show_constants, int nthreads, char** out);

/* The host random stream: srand/rand of the C library (main.cu:1107,1160). */
void gpr_host_srand(unsigned seed);
int gpr_host_rand(void);
/* The host stream's position: rand() calls since gpr_host_srand (every host
 * draw of this library counts).  gpr_host_srand(seed) then
 * gpr_host_rand_skip(n) puts the stream back where a run left it. */
uint64_t gpr_host_rand_calls(void);
void gpr_host_rand_skip(uint64_t n);

/* Initial chains (main.cu:1133-1137): every op ops[random_int(n_ops-1)] in
 * memory order, then every constant 10^U{-4..3} * N(0,1), host rand(). */
void gpr_host_init_chains(int32_t* P, float* C, int N, int PL, const int* ops, int n_ops);

/* Resampling (main.cu:1216-1231): sort the posteriors with the reference's
 * comparator; cutoff = sorted[(int)(N*param)] (GPR_RESAMPLE_QUANTILE, param
 * 0.5 in the reference) or max - param (GPR_RESAMPLE_MAP_DELTA); chains
 * strictly below the cutoff are re-drawn like the initialisation, in chain
 * order.  Returns the number of chains re-drawn, or -1 (gpr_host_last_error)
 * for bad arguments: N or PL < 1, fewer than 2 ops (the re-draw takes
 * random_int(n_ops - 1)), a quantile outside [0, 1) or a negative delta. */
int gpr_host_resample(int32_t* P, float* C, const double* prior, const double* lik, int N, int PL,
                      const int* ops, int n_ops, int mode, double param);

/* tops.txt without the external sort (run-all.sh:45 writes it with
 * `sort -g -k3 samples.txt | tail -n K`): a set that keeps, of all lines
 * offered to it, the K lines that command prints in the C locale, and writes
 * them in its order.  Lines are offered as text ('\n'-separated): all of a
 * buffer, or the lines at given 0-based indices (ascending). */
typedef struct gpr_tops gpr_tops;
gpr_tops* gpr_tops_new(int k);
int gpr_tops_add_text(gpr_tops* t, const char* text, int64_t len);
int gpr_tops_add_lines(gpr_tops* t, const char* text, int64_t len, const int* lines, int n);
/* Write the kept lines, ascending; returns the number written or -1. */
int64_t gpr_tops_write(gpr_tops* t, const char* path);
void gpr_tops_free(gpr_tops* t);

#ifdef __cplusplus
}
#endif

#endif /* GPUROPOLIS_HOST_H */
