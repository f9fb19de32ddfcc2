/*
 * gpr_host.cpp -- host side of the drop-in: data loading, the samples.txt
 * formatter, the host random initialisation and resampling of chains.  Part of
 * libgpuropolis.so (C ABI in include/gpuropolis_host.h); used by the
 * `gpuropolis` CLI (gpr_cli.cpp).
 *
 * Each function restates one piece of the reference's main.cu:
 *   gpr_load_data_file      load_data_file            main.cu:319-363
 *   gpr_format_expression   displaystring/display_latex main.cu:821-976
 *   gpr_program_length_of   program_fold(dispatch_length) main.cu:477-526
 *   gpr_polynomial_degree   polynomial_degree         main.cu:615-654
 *   gpr_format_samples      the per-chain output lines main.cu:1173-1210
 *   gpr_host_init_chains    initial programs/constants main.cu:1133-1137
 *   gpr_host_resample       median cutoff + re-draw    main.cu:1216-1231
 * The host random stream is the C library's rand() (srand(seed) at
 * main.cu:1107), so identical seeds give identical initial states and
 * resampling draws.  The formatting output is byte-identical to the
 * reference's wherever the reference stays within its 100-byte buffers
 * (main.cu:875-877); longer expressions, which overflow those buffers in the
 * reference, are written out in full.
 */
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpuropolis_host.h"
#include "gpr_common.h"

namespace {

/* ---------------------------------------------------------------- data --- */
/* nx = 1: the reference's "x y sd" lines; nx = 3: "x1 x2 x3 y sd" (the
 * variables in front, the same rules).  xs holds the nx variables of each
 * point in turn. */
int load_impl(const char* path, float sdscale, int first_half, int even_half, std::vector<float>& xs,
              std::vector<float>& ys, std::vector<float>& sds, std::string& err, int nx = 1) {
    FILE* fp = fopen(path, "r");
    if (!fp) { err = std::string("Cannot open file:\t") + path; return GPR_HOST_ERR_IO; }
    char* line = nullptr;
    size_t len = 0;
    double x, y, sd, x2 = 0.0, x3 = 0.0;
    int rc = GPR_HOST_OK;
    while (getline(&line, &len, fp) != -1) {
        if (line[0] == '#') continue;                                        /* main.cu:328 */
        const bool parsed = nx == 3
            ? (sscanf(line, "%lf\t%lf\t%lf\t%lf\t%lf\n", &x, &x2, &x3, &y, &sd) == 5 ||
               sscanf(line, "%le\t%le\t%le\t%le\t%le\n", &x, &x2, &x3, &y, &sd) == 5)
            : (sscanf(line, "%lf\t%lf\t%lf\n", &x, &y, &sd) == 3 ||
               sscanf(line, "%le\t%le\t%le\n", &x, &y, &sd) == 3);        /* main.cu:329-338 */
        if (parsed) {
            sd = sdscale * sd;
            if (!((float)sd > 0.0f)) {                                      /* main.cu:332 */
                err = std::string("sd must be > 0 in line: ") + line;
                rc = GPR_HOST_ERR_DATA;
                break;
            }
            xs.push_back((float)x);
            if (nx == 3) { xs.push_back((float)x2); xs.push_back((float)x3); }
            ys.push_back((float)y); sds.push_back((float)sd);
        } else if (strspn(line, " \r\n\t") == strlen(line)) {               /* main.cu:339 */
            continue;
        } else {
            err = std::string("ERROR IN PARSING INPUT\t") + line;             /* main.cu:343 */
            rc = GPR_HOST_ERR_DATA;
            break;
        }
    }
    free(line);
    fclose(fp);
    if (rc != GPR_HOST_OK) return rc;
    if (first_half) {                                   /* keep the first size/2 points, main.cu:350-355 */
        size_t mid = ys.size() / 2;
        xs.resize(mid * nx); ys.resize(mid); sds.resize(mid);
    }
    if (even_half) {                                    /* drop even 0-based indices, main.cu:356-360 */
        std::vector<float> a, b, c;
        for (size_t i = 1; i < ys.size(); i += 2) {
            for (int k = 0; k < nx; ++k) a.push_back(xs[i * nx + k]);
            b.push_back(ys[i]); c.push_back(sds[i]);
        }
        xs.swap(a); ys.swap(b); sds.swap(c);
    }
    return GPR_HOST_OK;
}

/* -------------------------------------------------------- expressions --- */
struct Tree {
    const int32_t* P;
    const float* C;
    int N, PL, idx;
    int op(int j) const { return P[(size_t)(j - 1) * N + idx]; }
    float c(int j) const { return C[(size_t)(j - 1) * N + idx]; }
};

void fmt_const(std::string& out, const char* cfmt, float v) {
    char b[512];
    snprintf(b, sizeof b, cfmt, (double)v);
    out += b;
}

/* string_dispatch (main.cu:821-873) / latex_dispatch (main.cu:901-953) over
 * the reachable part of the tree; unreachable nodes never reach the root's
 * string in the reference either. */
void display(const Tree& t, int j, const char* cfmt, bool latex, std::string& out) {
    if (j > t.PL) { out += "x"; return; }
    const int o = t.op(j);
    auto A = [&]() { display(t, 2 * j, cfmt, latex, out); };
    auto B = [&]() { display(t, 2 * j + 1, cfmt, latex, out); };
    auto Cc = [&]() { fmt_const(out, cfmt, t.c(j)); };
    auto S = [&](const char* s) { out += s; };
    if (!latex) {
        switch (o) {
            case OP_ONE: S("1"); break;
            case OP_CONST: Cc(); break;
            case OP_INV: S("(1/"); A(); S(")"); break;
            case OP_A: A(); break;
            case OP_B: B(); break;
            case OP_PLUS: S("("); A(); S("+"); B(); S(")"); break;
            case OP_CPLUS: S("("); A(); S("+"); Cc(); S(")"); break;
            case OP_MINUS: S("("); A(); S("-"); B(); S(")"); break;
            case OP_RMINUS: S("("); B(); S("-"); A(); S(")"); break;
            case OP_TIMES: S("("); B(); S("*"); A(); S(")"); break;
            case OP_CTIMES: S("("); A(); S("*"); Cc(); S(")"); break;
            case OP_DIV: S("("); A(); S("/"); B(); S(")"); break;
            case OP_RDIV: S("("); B(); S("/"); A(); S(")"); break;
            case OP_LOG: S("log("); A(); S(")"); break;
            case OP_SIN: S("sin("); A(); S(")"); break;
            case OP_ASIN: S("asin("); A(); S(")"); break;
            case OP_COS: S("cos("); A(); S(")"); break;
            case OP_ACOS: S("acos("); A(); S(")"); break;
            case OP_TAN: S("tan("); A(); S(")"); break;
            case OP_ATAN: S("atan("); A(); S(")"); break;
            case OP_SQRT: S("sqrt("); A(); S(")"); break;
            case OP_EXP: S("exp("); A(); S(")"); break;
            case OP_POW: S("("); A(); S("^"); B(); S(")"); break;
            case OP_CPOW: S("("); A(); S("^"); Cc(); S(")"); break;
            case OP_RPOW: S("("); B(); S("^"); A(); S(")"); break;
            case OP_CRPOW: S("("); Cc(); S("^"); A(); S(")"); break;
            case OP_ABS: S("abs("); A(); S(")"); break;
            case OP_X1: S("x1"); break;
            case OP_X2: S("x2"); break;
            case OP_X3: S("x3"); break;
            default: S("NAN"); break;
        }
    } else {
        switch (o) {
            case OP_ONE: S("1"); break;
            case OP_CONST: Cc(); break;
            case OP_INV: S("1/"); A(); break;
            case OP_A: A(); break;
            case OP_B: B(); break;
            case OP_PLUS: A(); S("+"); B(); break;
            case OP_CPLUS: A(); S("+"); Cc(); break;
            case OP_MINUS: A(); S("-"); B(); break;
            case OP_RMINUS: B(); S("-"); A(); break;
            case OP_TIMES: B(); S(" "); A(); break;
            case OP_CTIMES: A(); S(" \\cdot "); Cc(); break;
            case OP_DIV: S("\\frac{"); A(); S("}{"); B(); S("}"); break;
            case OP_RDIV: S("\\frac{"); B(); S("}{"); A(); S("}"); break;
            case OP_LOG: S("\\log("); A(); S(")"); break;
            case OP_SIN: S("sin("); A(); S(")"); break;
            case OP_ASIN: S("asin("); A(); S(")"); break;
            case OP_COS: S("cos("); A(); S(")"); break;
            case OP_ACOS: S("acos("); A(); S(")"); break;
            case OP_TAN: S("tan("); A(); S(")"); break;
            case OP_ATAN: S("atan("); A(); S(")"); break;
            case OP_SQRT: S("\\sqrt{"); A(); S("}"); break;
            case OP_EXP: S("e^{"); A(); S("}"); break;
            case OP_POW: A(); S("^{"); B(); S("}"); break;
            case OP_CPOW: A(); S("^{"); Cc(); S("}"); break;
            case OP_RPOW: B(); S("^{"); A(); S("}"); break;
            case OP_CRPOW: Cc(); S("^{"); A(); S("}"); break;
            case OP_ABS: S("\\mid "); A(); S("\\mid "); break;
            case OP_X1: S("x_1"); break;
            case OP_X2: S("x_2"); break;
            case OP_X3: S("x_3"); break;
            default: S("NAN"); break;
        }
    }
}

/* dispatch_length fold with X_LENGTH_PRIOR leaves (main.cu:477-526, 532). */
float length_of(const Tree& t, int j) {
    if (j > t.PL) return 1.0f;
    const int o = t.op(j);
    switch (gpr_op_class(o)) {
        case CLS_LEAF0: return 1.0f;
        case CLS_PASS_A: return length_of(t, 2 * j);
        case CLS_PASS_B: return length_of(t, 2 * j + 1);
        case CLS_UNARY: return 1.0f + length_of(t, 2 * j);
        case CLS_CUNARY: return 1.0f + length_of(t, 2 * j) + 1.0f;
        case CLS_BINARY: return 1.0f + length_of(t, 2 * j) + length_of(t, 2 * j + 1);
        default: return NAN;
    }
}

/* dispatch_degree fold, leaf 1 (main.cu:615-654). */
float degree_of(const Tree& t, int j) {
    if (j > t.PL) return 1.0f;
    const int o = t.op(j);
    const float c = t.c(j);
    auto mx = [](float a, float b) { return a > b ? a : b; };   /* the max macro, main.cu:186 */
    switch (o) {
        case OP_ONE: case OP_CONST: return 0.0f;
        case OP_X1: case OP_X2: case OP_X3: return 1.0f;   /* total degree over the variables */
        case OP_A: return degree_of(t, 2 * j);
        case OP_B: return degree_of(t, 2 * j + 1);
        case OP_PLUS: case OP_MINUS: case OP_RMINUS:
            return mx(degree_of(t, 2 * j), degree_of(t, 2 * j + 1));
        case OP_CPLUS: case OP_CTIMES: return degree_of(t, 2 * j);
        case OP_TIMES: return degree_of(t, 2 * j) + degree_of(t, 2 * j + 1);
        case OP_CPOW: return degree_of(t, 2 * j) * c;
        case OP_POW: {
            float a = degree_of(t, 2 * j), b = degree_of(t, 2 * j + 1);
            return (b == 0.0f) ? a * c : INFINITY;
        }
        case OP_DIV: {
            float a = degree_of(t, 2 * j), b = degree_of(t, 2 * j + 1);
            return (b == 0.0f) ? a : INFINITY;
        }
        default: return INFINITY;
    }
}

void format_line(std::string& out, const int32_t* P, const float* C, const double* prior,
                 const double* lik, int N, int PL, int h, int block, int show_constants) {
    Tree t{P, C, N, PL, h};
    char b[256];
    snprintf(b, sizeof b, "%d\t%d\t", h, block);
    out += b;
    snprintf(b, sizeof b, "%.3f\t%.3f\t%.3f\t", prior[h] + lik[h], prior[h], lik[h]);
    out += b;
    snprintf(b, sizeof b, "%.1f\t", (double)length_of(t, 1));
    out += b;
    float deg = degree_of(t, 1);
    if (deg == INFINITY) out += "NA\t";
    else { snprintf(b, sizeof b, "%.2f\t", (double)deg); out += b; }
    out += "\"";
    display(t, 1, "C", false, out);
    out += "\"\t\"";
    display(t, 1, "%.10f", false, out);
    out += "\"\t\"";
    display(t, 1, "%.2f", true, out);
    out += "\"\t\"";
    static const char* code = GPR_PROGRAM_CODE;
    for (int i = 0; i < PL; ++i) {
        int o = P[(size_t)i * N + h];
        out += (o >= 0 && o < OP_NALL) ? code[o] : '?';
    }
    out += "\"\t";
    if (show_constants) {
        for (int i = 0; i < PL; ++i) {
            snprintf(b, sizeof b, "%.10f\t", (double)C[(size_t)i * N + h]);
            out += b;
        }
    }
    out += "\n";
}

/* ---------------------------------------------------------- host RNG --- */
/* Every host draw goes through counted_rand(): the number of rand() calls
 * since srand() is the whole state a checkpoint needs to continue the stream
 * (re-seed, then skip that many draws). */
uint64_t g_rand_calls = 0;
int counted_rand() {
    ++g_rand_calls;
    return rand();
}

/* host random_int / random_float / random_normal (main.cu:262-284) */
int host_random_int(int limit) {
    int divisor = RAND_MAX / limit;
    int retval;
    do { retval = counted_rand() / divisor; } while (retval > limit - 1);
    return retval;
}
float host_random_float() { return float(counted_rand()) / RAND_MAX; }
float host_random_normal() {
    float u = host_random_float();
    float v = host_random_float();
    float lu = logf(u);                              /* log(float) resolves to the float overload */
    double s = sin(2.0 * 3.141592653589 * (double)v);
    return (float)((double)sqrtf((float)(-2.0 * (double)lu)) * s);
}

void redraw_chain(int32_t* P, float* C, int N, int PL, int h, const int* ops, int n_ops) {
    for (int i = 0; i < PL; ++i) P[(size_t)i * N + h] = ops[host_random_int(n_ops - 1)];
    for (int i = 0; i < PL; ++i) {
        int order = host_random_int(4 - (-4)) + (-4);  /* C_MAX_ORDER - C_MIN_ORDER */
        C[(size_t)i * N + h] = 1.0f * powf(10.0f, (float)order) * host_random_normal();
    }
}

/* cmp (main.cu:987-995) */
int cmp_bayes(const void* a, const void* b) {
    double ap = *static_cast<const double*>(a);
    double bp = *static_cast<const double*>(b);
    if (ap > bp || (bp != bp)) return 1;
    if (ap < bp || (ap != ap)) return -1;
    return 0;
}

thread_local std::string g_host_err;

}  // namespace

extern "C" {

/* load_impl with host-memory exhaustion as an error code (no exception may
 * leave a C entry point) */
static int load_guarded(const char* path, float sdscale, int first_half, int even_half, std::vector<float>& xs,
                        std::vector<float>& ys, std::vector<float>& sds, int nx) {
    try {
        return load_impl(path, sdscale, first_half, even_half, xs, ys, sds, g_host_err, nx);
    } catch (const std::bad_alloc&) {
        g_host_err = std::string("not enough host memory to load ") + path;
        return GPR_HOST_ERR_DATA;
    }
}

int gpr_load_data_file(const char* path, float sdscale, int first_half, int even_half,
                       float** x, float** y, float** sd, int* n) {
    if (!path || !x || !y || !sd || !n) return GPR_HOST_ERR_ARG;
    std::vector<float> xs, ys, sds;
    int rc = load_guarded(path, sdscale, first_half, even_half, xs, ys, sds, 1);
    if (rc != GPR_HOST_OK) return rc;
    size_t m = xs.size();
    *x = (float*)malloc((m + 1) * sizeof(float));
    *y = (float*)malloc((m + 1) * sizeof(float));
    *sd = (float*)malloc((m + 1) * sizeof(float));
    if (!*x || !*y || !*sd) return GPR_HOST_ERR_ARG;
    std::copy(xs.begin(), xs.end(), *x);
    std::copy(ys.begin(), ys.end(), *y);
    std::copy(sds.begin(), sds.end(), *sd);
    *n = (int)m;
    return GPR_HOST_OK;
}

int gpr_load_data_file3(const char* path, float sdscale, int first_half, int even_half, float** x1, float** x2,
                        float** x3, float** y, float** sd, int* n) {
    if (!path || !x1 || !x2 || !x3 || !y || !sd || !n) return GPR_HOST_ERR_ARG;
    std::vector<float> xs, ys, sds;
    int rc = load_guarded(path, sdscale, first_half, even_half, xs, ys, sds, 3);
    if (rc != GPR_HOST_OK) return rc;
    const size_t m = ys.size();
    float** outs[5] = {x1, x2, x3, y, sd};
    for (float** o : outs) *o = nullptr;
    for (float** o : outs) {
        *o = (float*)malloc((m + 1) * sizeof(float));
        if (!*o) {
            for (float** q : outs) { free(*q); *q = nullptr; }
            return GPR_HOST_ERR_ARG;
        }
    }
    for (size_t i = 0; i < m; ++i) {
        (*x1)[i] = xs[3 * i]; (*x2)[i] = xs[3 * i + 1]; (*x3)[i] = xs[3 * i + 2];
    }
    std::copy(ys.begin(), ys.end(), *y);
    std::copy(sds.begin(), sds.end(), *sd);
    *n = (int)m;
    return GPR_HOST_OK;
}

void gpr_free(void* p) { free(p); }

const char* gpr_host_last_error(void) { return g_host_err.c_str(); }

int gpr_format_expression(const int32_t* P, const float* C, int N, int PL, int idx, const char* cfmt,
                          int latex, char* out, int cap) {
    if (!P || !C || !cfmt || idx < 0 || idx >= N) return -1;
    Tree t{P, C, N, PL, idx};
    std::string s;
    display(t, 1, cfmt, latex != 0, s);
    if (out && cap > 0) {
        int m = (int)std::min(s.size(), (size_t)cap - 1);
        memcpy(out, s.data(), (size_t)m);
        out[m] = 0;
    }
    return (int)s.size();
}

float gpr_program_length_of(const int32_t* P, const float* C, int N, int PL, int idx) {
    Tree t{P, C, N, PL, idx};
    return length_of(t, 1);
}

float gpr_polynomial_degree(const int32_t* P, const float* C, int N, int PL, int idx) {
    Tree t{P, C, N, PL, idx};
    return degree_of(t, 1);
}

static int64_t format_samples_body(const int32_t* P, const float* C, const double* prior, const double* lik,
                                   int N, int PL, int block, int show_constants, int nthreads, char** out);

int64_t gpr_format_samples(const int32_t* P, const float* C, const double* prior, const double* lik,
                           int N, int PL, int block, int show_constants, int nthreads, char** out) {
    if (!P || !C || !prior || !lik || !out || N <= 0) return -1;
    try {
        return format_samples_body(P, C, prior, lik, N, PL, block, show_constants, nthreads, out);
    } catch (const std::exception&) {   /* host memory, or a thread that could not start */
        g_host_err = "gpr_format_samples: out of host resources";
        return -1;
    }
}

static int64_t format_samples_body(const int32_t* P, const float* C, const double* prior, const double* lik,
                                   int N, int PL, int block, int show_constants, int nthreads, char** out) {
    int T = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
    T = std::min(T, N);
    std::vector<std::string> parts(T);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) {
        th.emplace_back([&, t]() {
            int h0 = (int)((long long)N * t / T), h1 = (int)((long long)N * (t + 1) / T);
            std::string& s = parts[t];
            s.reserve((size_t)(h1 - h0) * 256);
            for (int h = h0; h < h1; ++h) format_line(s, P, C, prior, lik, N, PL, h, block, show_constants);
        });
    }
    for (auto& x : th) x.join();
    size_t total = 0;
    for (auto& s : parts) total += s.size();
    char* buf = (char*)malloc(total + 1);
    if (!buf) return -1;
    size_t off = 0;
    for (auto& s : parts) { memcpy(buf + off, s.data(), s.size()); off += s.size(); }
    buf[total] = 0;
    *out = buf;
    return (int64_t)total;
}

void gpr_host_srand(unsigned seed) {
    srand(seed);
    g_rand_calls = 0;
}
int gpr_host_rand(void) { return counted_rand(); }
uint64_t gpr_host_rand_calls(void) { return g_rand_calls; }
void gpr_host_rand_skip(uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) counted_rand();
}

void gpr_host_init_chains(int32_t* P, float* C, int N, int PL, const int* ops, int n_ops) {
    /* main.cu:1133-1137: every op first (in memory order), then every constant */
    for (long long i = 0; i < (long long)PL * N; ++i) P[i] = ops[host_random_int(n_ops - 1)];
    for (long long i = 0; i < (long long)PL * N; ++i) {
        int order = host_random_int(4 - (-4)) + (-4);
        C[i] = 1.0f * powf(10.0f, (float)order) * host_random_normal();
    }
}

int gpr_host_resample(int32_t* P, float* C, const double* prior, const double* lik, int N, int PL,
                      const int* ops, int n_ops, int mode, double param) {
    if (!P || !C || !prior || !lik || !ops || N <= 0 || PL <= 0 || n_ops < 2) {
        g_host_err = "gpr_host_resample: bad arguments";
        return -1;
    }
    if (mode == GPR_RESAMPLE_QUANTILE ? !((double)N * param >= 0.0 && (double)N * param < (double)N)
                                      : (mode != GPR_RESAMPLE_MAP_DELTA || !(param >= 0.0))) {
        g_host_err = "gpr_host_resample: mode must be quantile with param in [0, 1) or map-delta with param >= 0";
        return -1;
    }
    std::vector<double> post;
    try {
        post.resize((size_t)N);
    } catch (const std::bad_alloc&) {
        g_host_err = "gpr_host_resample: not enough host memory";
        return -1;
    }
    for (int h = 0; h < N; ++h) post[h] = prior[h] + lik[h];
    qsort(post.data(), (size_t)N, sizeof(double), cmp_bayes);          /* main.cu:1216-1218 */
    double cutoff;
    if (mode == GPR_RESAMPLE_MAP_DELTA) cutoff = post[N - 1] - param;
    else cutoff = post[(int)(N * param)];                               /* main.cu:1219 */
    int redrawn = 0;
    for (int h = 0; h < N; ++h) {
        if (prior[h] + lik[h] < cutoff) {                               /* main.cu:1223 */
            redraw_chain(P, C, N, PL, h, ops, n_ops);
            ++redrawn;
        }
    }
    return redrawn;
}

}  /* extern "C" */
