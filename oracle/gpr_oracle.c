/*
 * gpr_oracle.c -- plain-C restatement of the reference's sampler path.
 * TEST INFRASTRUCTURE ONLY: used by tests/ (and bench.py's CPU baseline when
 * the reference itself cannot be built); the product never links it.
 *
 * It restates, in this project's own code, what main.cu computes for one
 * chain, keeping the reference's float/double typing so results can be
 * compared bit for bit with the reference compiled for the host
 * (oracle/build_ref.py).  Each function names the main.cu lines it follows.
 * It also carries the extensions the reference cannot express (Philox stream,
 * random-walk constant moves, op subsets) and an FP64 evaluator used to state
 * the FP32 path's error against FP64.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#if defined(_OPENMP)
#include <omp.h>
#endif

#include "../gpuropolis_gb300/csrc/gpr_philox.h"
#include "../gpuropolis_gb300/csrc/gpr_rngmath.h"

/* op codes of the reference enum (main.cu:53) */
enum { ONE, CONST, INV, A, B, PLUS, MINUS, RMINUS, CPLUS, TIMES, CTIMES, DIV, RDIV, LOG, EXP, POW,
       CPOW, RPOW, CRPOW, SQRT, SIN, ASIN, COS, ACOS, TAN, ATAN, ABS, NREF,
       X1 = NREF, X2, X3 /* input variables of multivariate data (extension) */ };

#define PIF 3.141592653589          /* main.cu:194 */
#define MY_RAND_MAX 2147483647      /* main.cu:210 */
static const float PROPOSE_INT = 0.15f;     /* main.cu:32 */
static const float PROPOSE_GEOM_R = 0.1f;   /* main.cu:34 */

typedef struct {
    int program_length;  /* PL = NCONSTANTS */
    int n_ops;
    int ops[32];
    int rng;             /* 0 LCG, 1 Philox */
    int const_mode;      /* 0 independence (reference), 1 random walk */
    float rw_sd;
    int project_math;    /* logf/sinf of the random transforms from gpr_rngmath.h */
} port_cfg;

typedef struct {
    int rng;
    int lcg;                 /* reference: int rx (main.cu:691) */
    gpr_philox_stream ph;
} port_rng;

/* ---- random stream (main.cu:207-254) ----------------------------------- */
static int port_next(port_rng* r) {
    if (r->rng == 0) {
        /* (rx*1103515245 + 12345) & MY_RAND_MAX with 32-bit wrap-around */
        uint32_t x = (uint32_t)r->lcg * 1103515245u + 12345u;
        r->lcg = (int)(x & 0x7fffffffu);
        return r->lcg;
    }
    return gpr_philox_stream_next(&r->ph);
}
static int port_random_int(int n, port_rng* r) {
    int divisor = MY_RAND_MAX / (n + 1), v;
    do { v = port_next(r) / divisor; } while (v >= n);
    return v;
}
static float port_random_float(port_rng* r) { return (float)((double)(float)port_random_int(1000000, r) / 1000000.0); }
static float port_logf(float x, int pm) { return pm ? gpr_rng_logf(x) : logf(x); }
static float port_sinf(float x, int pm) { return pm ? gpr_rng_sinf(x) : sinf(x); }
static float port_random_normal(port_rng* r, int pm) {
    float u = port_random_float(r);
    float v = port_random_float(r);
    float a = sqrtf((float)(-2.0 * (double)port_logf(u, pm)));
    return a * port_sinf((float)(2.0 * PIF * (double)v), pm);
}
static float port_random_geometric(float rr, port_rng* r, int pm) {
    return ceilf(port_logf(port_random_float(r), pm) / port_logf(rr, pm));
}

/* ---- densities (main.cu:299-309, 190-192) ----------------------------- */
static double port_lnormalpdf(float x, float s) {
    return (double)(-(x * x)) / (2.0 * s * s) - 0.5 * ((double)logf((float)(2.0 * PIF)) + 2.0 * (double)logf(s));
}
static double port_lcauchypdf(float x, float s) {
    float t = -logf((float)PIF) - logf(s);
    return (double)(t - logf((float)(1.0 + (double)(x * x / s))));
}
static double port_lgeometricpdf(float n, float r) {
    return (double)((n - 1) * logf(r)) + log(1.0 - (double)r);
}
static double port_logplusexp(double a, double b) {
    double m = a > b ? a : b;
    return (double)logf(expf((float)(a - m)) + expf((float)(b - m))) + m;
}
static int port_is_int(float x) { return fabsf(x - (float)lroundf(x)) < 1.0e-6; }

/* ---- tree folds over the heap (main.cu:371-393) ------------------------ */
#define OP(P, N, idx, j) ((P)[(size_t)((j) - 1) * (N) + (idx)])

/* x2, x3 of the point being evaluated, for multivariate data (x1 is the
 * evaluators' x argument); set by the *_nv entry points below. */
static _Thread_local double g_x2 = 0.0, g_x3 = 0.0;
#define CV(C, N, idx, j) ((C)[(size_t)((j) - 1) * (N) + (idx)])

/* dispatch_eval (main.cu:397-444), reachable nodes only (the value of the
 * root never depends on the others). */
static float eval_node(const int32_t* P, const float* C, int N, int PL, int idx, int j, float x) {
    if (j > PL) return x;
    const int o = OP(P, N, idx, j);
    const float c = CV(C, N, idx, j);
#define L eval_node(P, C, N, PL, idx, 2 * j, x)
#define R eval_node(P, C, N, PL, idx, 2 * j + 1, x)
    switch (o) {
        case ONE: return 1.0f;
        case CONST: return c;
        case INV: return 1.0f / L;
        case A: return L;
        case B: return R;
        case PLUS: { float a = L, b = R; return a + b; }
        case CPLUS: return L + c;
        case MINUS: { float a = L, b = R; return a - b; }
        case RMINUS: { float a = L, b = R; return b - a; }
        case TIMES: { float a = L, b = R; return a * b; }
        case CTIMES: return c * L;
        case DIV: { float a = L, b = R; return a / b; }
        case RDIV: { float a = L, b = R; return b / a; }
        case SQRT: return sqrtf(L);
        case LOG: return logf(L);
        case SIN: return sinf(L);
        case ASIN: return asinf(L);
        case COS: return cosf(L);
        case ACOS: return acosf(L);
        case TAN: return tanf(L);
        case ATAN: return atanf(L);
        case EXP: return expf(L);
        case POW: { float a = L, b = R; return powf(a, b); }
        case CPOW: return powf(L, c);
        case RPOW: { float a = L, b = R; return powf(b, a); }
        case CRPOW: return powf(c, L);
        case ABS: return fabsf(L);
        case X1: return x;
        case X2: return (float)g_x2;
        case X3: return (float)g_x3;
        default: return NAN;
    }
#undef L
#undef R
}

/* The same expression evaluated in FP64 throughout (for error statements). */
static double eval_node_f64(const int32_t* P, const float* C, int N, int PL, int idx, int j, double x) {
    if (j > PL) return x;
    const int o = OP(P, N, idx, j);
    const double c = CV(C, N, idx, j);
#define L eval_node_f64(P, C, N, PL, idx, 2 * j, x)
#define R eval_node_f64(P, C, N, PL, idx, 2 * j + 1, x)
    switch (o) {
        case ONE: return 1.0;
        case CONST: return c;
        case INV: return 1.0 / L;
        case A: return L;
        case B: return R;
        case PLUS: { double a = L, b = R; return a + b; }
        case CPLUS: return L + c;
        case MINUS: { double a = L, b = R; return a - b; }
        case RMINUS: { double a = L, b = R; return b - a; }
        case TIMES: { double a = L, b = R; return a * b; }
        case CTIMES: return c * L;
        case DIV: { double a = L, b = R; return a / b; }
        case RDIV: { double a = L, b = R; return b / a; }
        case SQRT: return sqrt(L);
        case LOG: return log(L);
        case SIN: return sin(L);
        case ASIN: return asin(L);
        case COS: return cos(L);
        case ACOS: return acos(L);
        case TAN: return tan(L);
        case ATAN: return atan(L);
        case EXP: return exp(L);
        case POW: { double a = L, b = R; return pow(a, b); }
        case CPOW: return pow(L, c);
        case RPOW: { double a = L, b = R; return pow(b, a); }
        case CRPOW: return pow(c, L);
        case ABS: return fabs(L);
        case X1: return x;
        case X2: return g_x2;
        case X3: return g_x3;
        default: return NAN;
    }
#undef L
#undef R
}

/* FP64 evaluation with every node's result multiplied by (1 + rel*u), u a
 * seeded pseudo-random number in [-1, 1]: repeated with different seeds it
 * measures how far FP32 rounding (rel ~ a few 2^-24) can move the value of
 * this program at this point -- its sensitivity, whatever the libm. */
static uint32_t port_hash(uint32_t a) {
    a ^= a >> 16; a *= 0x7feb352du; a ^= a >> 15; a *= 0x846ca68bu; a ^= a >> 16;
    return a;
}
static double eval_node_f64p(const int32_t* P, const float* C, int N, int PL, int idx, int j, double x,
                             uint32_t seed, double rel) {
    if (j > PL) return x;
    const int o = OP(P, N, idx, j);
    const double c = CV(C, N, idx, j);
    double r;
#define L eval_node_f64p(P, C, N, PL, idx, 2 * j, x, seed, rel)
#define R eval_node_f64p(P, C, N, PL, idx, 2 * j + 1, x, seed, rel)
    switch (o) {
        case ONE: r = 1.0; break;
        case CONST: r = c; break;
        case INV: r = 1.0 / L; break;
        case A: return L;
        case B: return R;
        case PLUS: { double a = L, b = R; r = a + b; break; }
        case CPLUS: r = L + c; break;
        case MINUS: { double a = L, b = R; r = a - b; break; }
        case RMINUS: { double a = L, b = R; r = b - a; break; }
        case TIMES: { double a = L, b = R; r = a * b; break; }
        case CTIMES: r = c * L; break;
        case DIV: { double a = L, b = R; r = a / b; break; }
        case RDIV: { double a = L, b = R; r = b / a; break; }
        case SQRT: r = sqrt(L); break;
        case LOG: r = log(L); break;
        case SIN: r = sin(L); break;
        case ASIN: r = asin(L); break;
        case COS: r = cos(L); break;
        case ACOS: r = acos(L); break;
        case TAN: r = tan(L); break;
        case ATAN: r = atan(L); break;
        case EXP: r = exp(L); break;
        case POW: { double a = L, b = R; r = pow(a, b); break; }
        case CPOW: r = pow(L, c); break;
        case RPOW: { double a = L, b = R; r = pow(b, a); break; }
        case CRPOW: r = pow(c, L); break;
        case ABS: r = fabs(L); break;
        case X1: return x;
        case X2: return g_x2;
        case X3: return g_x3;
        default: return NAN;
    }
#undef L
#undef R
    if (o == ONE || o == CONST) return r;
    double u = (double)port_hash(seed * 2654435761u + (uint32_t)j) / 4294967295.0 * 2.0 - 1.0;
    return r * (1.0 + rel * u);
}

double gpr_port_eval_f64_perturbed(const int32_t* P, const float* C, int N, int PL, int idx, double x,
                                   unsigned seed, double rel) {
    return eval_node_f64p(P, C, N, PL, idx, 1, x, seed, rel);
}

/* dispatch_length (main.cu:477-526) with X_LENGTH_PRIOR = CONST_LENGTH_PRIOR = 1 */
static float length_node(const int32_t* P, int N, int PL, int idx, int j) {
    if (j > PL) return 1.0f;
    int o = OP(P, N, idx, j);
    switch (o) {
        case ONE: case CONST: case X1: case X2: case X3: return 1.0f;
        case A: return length_node(P, N, PL, idx, 2 * j);
        case B: return length_node(P, N, PL, idx, 2 * j + 1);
        case CPLUS: case CTIMES: case CPOW: case CRPOW: return 1.0f + length_node(P, N, PL, idx, 2 * j) + 1.0f;
        case PLUS: case MINUS: case RMINUS: case TIMES: case DIV: case RDIV: case POW: case RPOW:
            return 1.0f + length_node(P, N, PL, idx, 2 * j) + length_node(P, N, PL, idx, 2 * j + 1);
        case INV: case LOG: case EXP: case SQRT: case SIN: case ASIN: case COS: case ACOS: case TAN:
        case ATAN: case ABS:
            return 1.0f + length_node(P, N, PL, idx, 2 * j);
        default: return NAN;
    }
}
/* dispatch_countnodes (main.cu:553-601): leaves x count 0 */
static int count_node(const int32_t* P, int N, int PL, int idx, int j) {
    if (j > PL) return 0;
    int o = OP(P, N, idx, j);
    switch (o) {
        case ONE: case CONST: case X1: case X2: case X3: return 1;
        case A: return count_node(P, N, PL, idx, 2 * j);
        case B: return count_node(P, N, PL, idx, 2 * j + 1);
        case PLUS: case MINUS: case RMINUS: case TIMES: case DIV: case RDIV: case POW: case RPOW:
            return 1 + count_node(P, N, PL, idx, 2 * j) + count_node(P, N, PL, idx, 2 * j + 1);
        default: return 1 + count_node(P, N, PL, idx, 2 * j);
    }
}

float gpr_port_eval(const int32_t* P, const float* C, int N, int PL, int idx, float x) {
    return eval_node(P, C, N, PL, idx, 1, x);
}
double gpr_port_eval_f64(const int32_t* P, const float* C, int N, int PL, int idx, double x) {
    return eval_node_f64(P, C, N, PL, idx, 1, x);
}
float gpr_port_length(const int32_t* P, int N, int PL, int idx) { return length_node(P, N, PL, idx, 1); }
int gpr_port_count(const int32_t* P, int N, int PL, int idx) { return count_node(P, N, PL, idx, 1); }

/* compute_prior (main.cu:529-544) */
double gpr_port_prior(const int32_t* P, const float* C, int N, int PL, int idx, int n_ops) {
    float length = length_node(P, N, PL, idx, 1);
    double prior = (double)(-1.0f * length) * log((double)n_ops + 1);
    for (int c = 0; c < PL; c++) prior += port_lcauchypdf(C[(size_t)c * N + idx], 1.0f);
    return prior;
}

/* compute_likelihood (main.cu:454-468); D is (x, y, sd) triples */
double gpr_port_likelihood(const int32_t* P, const float* C, int N, int PL, int idx, const float* D, int nd) {
    double ll = 0.0;
    for (int d = 0; d < nd; d++) {
        float fx = eval_node(P, C, N, PL, idx, 1, D[3 * d]);
        if (isnan(fx) || !isfinite(fx)) return -INFINITY;
        double l = port_lnormalpdf(fx - D[3 * d + 1], D[3 * d + 2]);
        if (isnan(l) || !isfinite(l)) return -INFINITY;
        ll += l;
    }
    return ll;
}

/* The same likelihood with the program evaluated in FP64 and summed in FP64. */
double gpr_port_likelihood_f64(const int32_t* P, const float* C, int N, int PL, int idx, const float* D, int nd) {
    double ll = 0.0;
    for (int d = 0; d < nd; d++) {
        double fx = eval_node_f64(P, C, N, PL, idx, 1, D[3 * d]);
        if (!isfinite(fx)) return -INFINITY;
        double r = fx - (double)D[3 * d + 1], s = D[3 * d + 2];
        ll += -(r * r) / (2.0 * s * s) - 0.5 * (log(2.0 * PIF) + 2.0 * log(s));
    }
    return ll;
}

/* is_descendant (main.cu:660-677): node k (0-based) in the subtree of n */
static int port_is_descendant(int n, int k) {
    if (k == n) return 1;
    n++; k++;
    while (k > n) { k >>= 1; if (k == n) return 1; }
    return 0;
}

static int port_valid(double v) { return !(isnan(v) || !isfinite(v)); }

/* One chain for `steps` MH steps: MH_simple_kernel (main.cu:679-813). */
/* trace (optional): per step GPR_TRACE doubles -- proposal posterior, current
 * posterior, acceptance log-ratio, the uniform draw (-1 when none was drawn),
 * the decision (1 accept, 0 reject), and the conditioning of the proposal's
 * and of the current state's FP32 log-likelihood: |L32 - L64| / max(|L64|, 1)
 * with L64 the same program evaluated and summed in FP64 (inf when exactly one
 * of them is finite). */
#define GPR_TRACE 8
static double port_cond(double l32, double l64) {
    if (isfinite(l32) != isfinite(l64)) return INFINITY;
    if (!isfinite(l32)) return 0.0;
    return fabs(l32 - l64) / (fabs(l64) > 1.0 ? fabs(l64) : 1.0);
}
static void mh_chain(const port_cfg* cfg, int N, int idx, int32_t* P, float* C, const float* D, int nd,
                     int steps, double* prior_out, double* lik_out, int random_seed, double* trace) {
    const int PL = cfg->program_length;
    const int pm = cfg->project_math;
    double cur_prior = gpr_port_prior(P, C, N, PL, idx, cfg->n_ops);
    double cur_lik = gpr_port_likelihood(P, C, N, PL, idx, D, nd);
    double cur_post = cur_prior + cur_lik;
    port_rng r;
    r.rng = cfg->rng;
    r.lcg = (int)((uint32_t)random_seed + (uint32_t)idx);
    gpr_philox_stream_init(&r.ph, (uint32_t)random_seed, (uint32_t)idx);
    int32_t old_program[256];
    float old_C[256];
    double forward = 0.0, backward = 0.0;
    double cond_cur = trace ? port_cond(cur_lik, gpr_port_likelihood_f64(P, C, N, PL, idx, D, nd)) : 0.0;
    for (int step = 0; step < steps; step++) {
        if (step % 5 == 0) {
            forward = -(double)logf((float)count_node(P, N, PL, idx, 1));
            int n = port_valid(cur_post) ? port_random_int(PL, &r) : 0;
            for (int i = n; i < PL; i++) {
                old_program[i] = P[(size_t)i * N + idx];
                if (port_is_descendant(n, i)) P[(size_t)i * N + idx] = cfg->ops[port_random_int(cfg->n_ops, &r)];
            }
            backward = -(double)logf((float)count_node(P, N, PL, idx, 1));
            double pp = gpr_port_prior(P, C, N, PL, idx, cfg->n_ops);
            double pl = gpr_port_likelihood(P, C, N, PL, idx, D, nd);
            double post = pp + pl;
            double acc = post - cur_post + backward - forward;
            double udraw = -1.0;
            int accept = 0;
            if (port_valid(post)) {
                if (acc > 0.0) accept = 1;
                else { float u = port_random_float(&r); udraw = u; accept = u < expf((float)acc); }
            }
            if (!port_valid(cur_post)) accept = 1;
            double cond_prop = 0.0;
            if (trace) {
                cond_prop = port_cond(pl, gpr_port_likelihood_f64(P, C, N, PL, idx, D, nd));
                double* t = trace + GPR_TRACE * (size_t)step;
                t[0] = post; t[1] = cur_post; t[2] = acc; t[3] = udraw; t[4] = accept;
                t[5] = cond_prop; t[6] = cond_cur; t[7] = 0.0;
            }
            if (accept) cond_cur = cond_prop;
            if (accept) {
                cur_post = post; cur_lik = pl; cur_prior = pp;
            } else {
                for (int i = n; i < PL; i++) P[(size_t)i * N + idx] = old_program[i];
            }
        } else {
            for (int c = 0; c < PL; c++) {
                size_t i = (size_t)c * N + idx;
                old_C[c] = C[i];
                if (port_random_float(&r) < (cfg->const_mode == 0 ? 1.0f : 0.0f)) {
                    if (port_random_float(&r) < PROPOSE_INT) {
                        float sgn = port_random_float(&r) < 0.5 ? -1.0f : 1.0f;
                        C[i] = sgn * port_random_geometric(PROPOSE_GEOM_R, &r, pm) - 1;
                        forward += port_lgeometricpdf(C[i] + 1, PROPOSE_GEOM_R) + (C[i] == 0.0 ? 0.0 : log(2.0)) +
                                   (double)logf(PROPOSE_INT);
                    } else {
                        C[i] = 1.0f * port_random_normal(&r, pm);
                        forward += port_lnormalpdf(C[i] / 1.0f, 1.0f) + log(1.0 - (double)PROPOSE_INT);
                    }
                    if (port_is_int(old_C[c])) {
                        backward += port_logplusexp(
                            port_lgeometricpdf(old_C[c] + 1, PROPOSE_GEOM_R) + (C[i] == 0.0 ? 0.0 : log(2.0)) +
                                (double)logf(PROPOSE_INT),
                            port_lnormalpdf(old_C[c] / 1.0f, 1.0f) + log(1.0 - (double)PROPOSE_INT));
                    } else {
                        backward += port_lnormalpdf(old_C[c] / 1.0f, 1.0f) + log(1.0 - (double)PROPOSE_INT);
                    }
                } else if (cfg->const_mode == 1) {
                    C[i] = C[i] + cfg->rw_sd * port_random_normal(&r, pm);
                } else {
                    int order = port_random_int(8, &r) - 4;
                    C[i] = C[i] + 1.0f * powf(10.0f, (float)order) * port_random_normal(&r, pm);
                }
            }
            double pp = gpr_port_prior(P, C, N, PL, idx, cfg->n_ops);
            double pl = gpr_port_likelihood(P, C, N, PL, idx, D, nd);
            double post = pp + pl;
            double acc = post - cur_post + backward - forward;
            double udraw = -1.0;
            int accept = 0;
            if (port_valid(post)) {
                if (acc > 0.0) accept = 1;
                else { float u = port_random_float(&r); udraw = u; accept = u < expf((float)acc); }
            }
            if (!port_valid(cur_post)) accept = 1;
            double cond_prop = 0.0;
            if (trace) {
                cond_prop = port_cond(pl, gpr_port_likelihood_f64(P, C, N, PL, idx, D, nd));
                double* t = trace + GPR_TRACE * (size_t)step;
                t[0] = post; t[1] = cur_post; t[2] = acc; t[3] = udraw; t[4] = accept;
                t[5] = cond_prop; t[6] = cond_cur; t[7] = 0.0;
            }
            if (accept) cond_cur = cond_prop;
            if (accept) {
                cur_post = post; cur_lik = pl; cur_prior = pp;
            } else {
                for (int c = 0; c < PL; c++) C[(size_t)c * N + idx] = old_C[c];
            }
        }
    }
    prior_out[idx] = cur_prior;
    lik_out[idx] = cur_lik;
}

/* One block over chains [c0, c1) (the kernel launch of main.cu:1160). */
void gpr_port_run_block(const port_cfg* cfg, int N, int c0, int c1, int32_t* P, float* C, const float* D,
                        int nd, int steps, double* prior, double* lik, int random_seed, int nthreads) {
#if defined(_OPENMP)
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int idx = c0; idx < c1; idx++) mh_chain(cfg, N, idx, P, C, D, nd, steps, prior, lik, random_seed, NULL);
}

/* The same with a per-chain, per-step trace: trace[(idx * steps + step) * 5 + k]. */
void gpr_port_run_block_trace(const port_cfg* cfg, int N, int32_t* P, float* C, const float* D, int nd, int steps,
                              double* prior, double* lik, int random_seed, double* trace, int nthreads) {
#if defined(_OPENMP)
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int idx = 0; idx < N; idx++)
        mh_chain(cfg, N, idx, P, C, D, nd, steps, prior, lik, random_seed, trace + (size_t)idx * steps * GPR_TRACE);
}

int gpr_port_sizeof_cfg(void) { return (int)sizeof(port_cfg); }

/* ---- resampling (main.cu:1215-1231) with the device's random stream ------ */

/* cmp (main.cu:987-995): NaN sorts below every value. */
static int port_cmp_bayes(const void* a, const void* b) {
    double ap = *(const double*)a, bp = *(const double*)b;
    if (ap > bp || (bp != bp)) return 1;
    if (ap < bp || (ap != ap)) return -1;
    return 0;
}

/* The cutoff of main.cu:1216-1219 (mode 0: sorted[(int)(N*param)]) or the
 * largest posterior minus param (mode 1); then every chain strictly below it
 * is re-drawn as main.cu:1224-1228 does -- all PL ops as ops[random_int(n_ops-1)],
 * then all PL constants as powf(10, random_int(8) - 4) * random_normal() --
 * from the Philox stream keyed by (seed, chain | 2^31).  Returns the number of
 * chains re-drawn; *cutoff_out receives the cutoff. */
/* Resampling of chains [c0, c1) against their own cutoff (rank rule over
 * the c1 - c0 chains); the streams are keyed by the global chain index. */
static int port_resample_range(const port_cfg* cfg, int N, int c0, int c1, int32_t* P, float* C,
                               const double* prior, const double* lik, int mode, double param, uint32_t seed,
                               double* cutoff_out) {
    const int n = c1 - c0;
    double* post = (double*)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    for (int h = 0; h < n; ++h) post[h] = prior[c0 + h] + lik[c0 + h];
    qsort(post, (size_t)n, sizeof(double), port_cmp_bayes);
    const double cutoff = mode == 1 ? post[n - 1] - param : post[(int)(n * param)];
    free(post);
    int redrawn = 0;
    const int PL = cfg->program_length;
    for (int h = c0; h < c1; ++h) {
        if (!(prior[h] + lik[h] < cutoff)) continue;
        port_rng r;
        r.rng = 1;
        r.lcg = 0;
        gpr_philox_stream_init(&r.ph, seed, (uint32_t)h | 0x80000000u);
        for (int i = 0; i < PL; ++i) P[(size_t)i * N + h] = cfg->ops[port_random_int(cfg->n_ops - 1, &r)];
        for (int i = 0; i < PL; ++i) {
            int order = port_random_int(4 - (-4), &r) + (-4);           /* C_MAX_ORDER - C_MIN_ORDER */
            C[(size_t)i * N + h] = 1.0f * powf(10.0f, (float)order) * port_random_normal(&r, 1);
        }
        ++redrawn;
    }
    if (cutoff_out) *cutoff_out = cutoff;
    return redrawn;
}

int gpr_port_resample(const port_cfg* cfg, int N, int32_t* P, float* C, const double* prior, const double* lik,
                      int mode, double param, uint32_t seed, double* cutoff_out) {
    return port_resample_range(cfg, N, 0, N, P, C, prior, lik, mode, param, seed, cutoff_out);
}

/* Batched data: the same per dataset, chains [d*N/nseg, (d+1)*N/nseg) of
 * dataset d resampled against that dataset's cutoff (cutoffs_out[d]). */
int gpr_port_resample_segments(const port_cfg* cfg, int N, int nseg, int32_t* P, float* C, const double* prior,
                               const double* lik, int mode, double param, uint32_t seed, double* cutoffs_out) {
    const int seg = N / nseg;
    int redrawn = 0;
    for (int d = 0; d < nseg; ++d)
        redrawn += port_resample_range(cfg, N, d * seg, (d + 1) * seg, P, C, prior, lik, mode, param, seed,
                                       cutoffs_out ? cutoffs_out + d : NULL);
    return redrawn;
}

/* ---- FP64 log-likelihood gradient in the constants (extension) ----------
 * The program of chain idx evaluated in FP64 with its constants taken from
 * Cd[0..PL) (double, so finite differences can move them by less than a
 * float ulp), and the derivative of the log-likelihood of main.cu:454-468
 * in each constant by reverse mode on the heap tree. */

/* Optional jitter of every operation's result, as in eval_node_f64p, so the
 * gradient's own FP32 noise floor can be measured (0: none). */
static double g_evd_rel = 0.0;
static uint32_t g_evd_seed = 0u;

static double evd(const int32_t* P, int N, int PL, int idx, const double* Cd, int j, double x) {
    if (j > PL) return x;
    const int o = OP(P, N, idx, j);
    const double c = Cd[j - 1];
    double r;
#define L evd(P, N, PL, idx, Cd, 2 * j, x)
#define R evd(P, N, PL, idx, Cd, 2 * j + 1, x)
    switch (o) {
        case ONE: return 1.0;
        case CONST: return c;
        case INV: r = 1.0 / L; break;
        case A: return L;
        case B: return R;
        case PLUS: { double a = L, b = R; r = a + b; break; }
        case CPLUS: r = L + c; break;
        case MINUS: { double a = L, b = R; r = a - b; break; }
        case RMINUS: { double a = L, b = R; r = b - a; break; }
        case TIMES: { double a = L, b = R; r = a * b; break; }
        case CTIMES: r = c * L; break;
        case DIV: { double a = L, b = R; r = a / b; break; }
        case RDIV: { double a = L, b = R; r = b / a; break; }
        case SQRT: r = sqrt(L); break;
        case LOG: r = log(L); break;
        case SIN: r = sin(L); break;
        case ASIN: r = asin(L); break;
        case COS: r = cos(L); break;
        case ACOS: r = acos(L); break;
        case TAN: r = tan(L); break;
        case ATAN: r = atan(L); break;
        case EXP: r = exp(L); break;
        case POW: { double a = L, b = R; r = pow(a, b); break; }
        case CPOW: r = pow(L, c); break;
        case RPOW: { double a = L, b = R; r = pow(b, a); break; }
        case CRPOW: r = pow(c, L); break;
        case ABS: r = fabs(L); break;
        case X1: return x;
        case X2: return g_x2;
        case X3: return g_x3;
        default: return NAN;
    }
#undef L
#undef R
    if (g_evd_rel == 0.0) return r;
    double u = (double)port_hash(g_evd_seed * 2654435761u + (uint32_t)j) / 4294967295.0 * 2.0 - 1.0;
    return r * (1.0 + g_evd_rel * u);
}

/* d(a^b)/da and d(a^b)/db */
static double dpow_da(double a, double b) { return b * pow(a, b - 1.0); }
static double dpow_db(double a, double b) { double r = pow(a, b); return r == 0.0 ? 0.0 : r * log(a); }

/* adds adj * d f_j / d Cd[k] to g[k] for every constant of the subtree at j */
static void gradd(const int32_t* P, int N, int PL, int idx, const double* Cd, int j, double x, double adj, double* g) {
    if (j > PL) return;
    const int o = OP(P, N, idx, j);
    const double c = Cd[j - 1];
#define L evd(P, N, PL, idx, Cd, 2 * j, x)
#define R evd(P, N, PL, idx, Cd, 2 * j + 1, x)
#define GL(d) gradd(P, N, PL, idx, Cd, 2 * j, x, adj * (d), g)
#define GR(d) gradd(P, N, PL, idx, Cd, 2 * j + 1, x, adj * (d), g)
    switch (o) {
        case ONE: return;
        case CONST: g[j - 1] += adj; return;
        case A: GL(1.0); return;
        case B: GR(1.0); return;
        case INV: { double a = L; GL(-1.0 / (a * a)); return; }
        case LOG: { double a = L; GL(1.0 / a); return; }
        case EXP: { double a = L; GL(exp(a)); return; }
        case SQRT: { double a = L; GL(0.5 / sqrt(a)); return; }
        case SIN: { double a = L; GL(cos(a)); return; }
        case ASIN: { double a = L; GL(1.0 / sqrt(1.0 - a * a)); return; }
        case COS: { double a = L; GL(-sin(a)); return; }
        case ACOS: { double a = L; GL(-1.0 / sqrt(1.0 - a * a)); return; }
        case TAN: { double t = tan(L); GL(1.0 + t * t); return; }
        case ATAN: { double a = L; GL(1.0 / (1.0 + a * a)); return; }
        case ABS: { double a = L; GL(a > 0 ? 1.0 : (a < 0 ? -1.0 : 0.0)); return; }
        case CPLUS: GL(1.0); g[j - 1] += adj; return;
        case CTIMES: { double a = L; GL(c); g[j - 1] += adj * a; return; }
        case CPOW: { double a = L; GL(dpow_da(a, c)); g[j - 1] += adj * dpow_db(a, c); return; }
        case CRPOW: { double a = L; GL(dpow_db(c, a)); g[j - 1] += adj * dpow_da(c, a); return; }
        case PLUS: GL(1.0); GR(1.0); return;
        case MINUS: GL(1.0); GR(-1.0); return;
        case RMINUS: GL(-1.0); GR(1.0); return;
        case TIMES: { double a = L, b = R; GL(b); GR(a); return; }
        case DIV: { double a = L, b = R; GL(1.0 / b); GR(-a / (b * b)); return; }
        case RDIV: { double a = L, b = R; GL(-b / (a * a)); GR(1.0 / a); return; }
        case POW: { double a = L, b = R; GL(dpow_da(a, b)); GR(dpow_db(a, b)); return; }
        case RPOW: { double a = L, b = R; GL(dpow_db(b, a)); GR(dpow_da(b, a)); return; }
        default: return;
    }
#undef L
#undef R
#undef GL
#undef GR
}

double gpr_port_loglik_f64d(const int32_t* P, int N, int PL, int idx, const double* Cd, const float* D, int nd) {
    double ll = 0.0;
    for (int d = 0; d < nd; d++) {
        double fx = evd(P, N, PL, idx, Cd, 1, D[3 * d]);
        if (!isfinite(fx)) return -INFINITY;
        double r = fx - (double)D[3 * d + 1], s = D[3 * d + 2];
        ll += -(r * r) / (2.0 * s * s) - 0.5 * (log(2.0 * PIF) + 2.0 * log(s));
    }
    return ll;
}

/* Returns the FP64 log-likelihood and writes d loglik / d Cd[k] to g[k];
 * when gabs is non-NULL, also the sum over points of the absolute per-point
 * terms of each g[k] (the scale against which cancellation in the sum is
 * judged). */
double gpr_port_loglik_grad_f64(const int32_t* P, int N, int PL, int idx, const double* Cd, const float* D, int nd,
                                double* g, double* gabs) {
    double* gd = (double*)calloc((size_t)PL, sizeof(double));
    for (int k = 0; k < PL; ++k) { g[k] = 0.0; if (gabs) gabs[k] = 0.0; }
    double ll = 0.0;
    for (int d = 0; d < nd; d++) {
        double fx = evd(P, N, PL, idx, Cd, 1, D[3 * d]);
        if (!isfinite(fx)) { ll = -INFINITY; break; }
        double r = fx - (double)D[3 * d + 1], s = D[3 * d + 2];
        ll += -(r * r) / (2.0 * s * s) - 0.5 * (log(2.0 * PIF) + 2.0 * log(s));
        for (int k = 0; k < PL; ++k) gd[k] = 0.0;
        gradd(P, N, PL, idx, Cd, 1, D[3 * d], -r / (s * s), gd);
        for (int k = 0; k < PL; ++k) { g[k] += gd[k]; if (gabs) gabs[k] += fabs(gd[k]); }
    }
    free(gd);
    return ll;
}

/* The same gradient with every operation's result jittered by up to rel
 * (seeded): repeated over seeds it measures the gradient's FP32 noise floor. */
double gpr_port_loglik_grad_f64p(const int32_t* P, int N, int PL, int idx, const double* Cd, const float* D, int nd,
                                 double* g, unsigned seed, double rel) {
    g_evd_rel = rel;
    g_evd_seed = seed;
    double ll = gpr_port_loglik_grad_f64(P, N, PL, idx, Cd, D, nd, g, NULL);
    g_evd_rel = 0.0;
    return ll;
}

/* ---- multivariate data (extension): D5 holds (x1, x2, x3, y, sd) per point */

static void set_point(const float* D5, int d) { g_x2 = D5[5 * d + 1]; g_x3 = D5[5 * d + 2]; }

float gpr_port_call_nv(const int32_t* P, const float* C, int N, int PL, int idx, float x1, float x2, float x3) {
    g_x2 = x2; g_x3 = x3;
    return eval_node(P, C, N, PL, idx, 1, x1);
}

/* compute_likelihood (main.cu:454-468) over multivariate points, FP32
 * evaluation (f64 = 0) or FP64 evaluation and sum (f64 = 1). */
double gpr_port_likelihood_nv(const int32_t* P, const float* C, int N, int PL, int idx, const float* D5, int nd,
                              int f64) {
    double ll = 0.0;
    for (int d = 0; d < nd; d++) {
        set_point(D5, d);
        const float x1 = D5[5 * d], y = D5[5 * d + 3], sd = D5[5 * d + 4];
        if (f64) {
            double fx = eval_node_f64(P, C, N, PL, idx, 1, x1);
            if (!isfinite(fx)) return -INFINITY;
            double r = fx - (double)y, s = sd;
            ll += -(r * r) / (2.0 * s * s) - 0.5 * (log(2.0 * PIF) + 2.0 * log(s));
        } else {
            float fx = eval_node(P, C, N, PL, idx, 1, x1);
            if (isnan(fx) || !isfinite(fx)) return -INFINITY;
            double l = port_lnormalpdf(fx - y, sd);
            if (isnan(l) || !isfinite(l)) return -INFINITY;
            ll += l;
        }
    }
    return ll;
}

/* d loglik / d Cd over multivariate points (as gpr_port_loglik_grad_f64). */
double gpr_port_loglik_grad_f64_nv(const int32_t* P, int N, int PL, int idx, const double* Cd, const float* D5,
                                   int nd, double* g, double* gabs) {
    double* gd = (double*)calloc((size_t)PL, sizeof(double));
    for (int k = 0; k < PL; ++k) { g[k] = 0.0; if (gabs) gabs[k] = 0.0; }
    double ll = 0.0;
    for (int d = 0; d < nd; d++) {
        set_point(D5, d);
        const double x1 = D5[5 * d];
        double fx = evd(P, N, PL, idx, Cd, 1, x1);
        if (!isfinite(fx)) { ll = -INFINITY; break; }
        double r = fx - (double)D5[5 * d + 3], s = D5[5 * d + 4];
        ll += -(r * r) / (2.0 * s * s) - 0.5 * (log(2.0 * PIF) + 2.0 * log(s));
        for (int k = 0; k < PL; ++k) gd[k] = 0.0;
        gradd(P, N, PL, idx, Cd, 1, x1, -r / (s * s), gd);
        for (int k = 0; k < PL; ++k) { g[k] += gd[k]; if (gabs) gabs[k] += fabs(gd[k]); }
    }
    free(gd);
    return ll;
}
