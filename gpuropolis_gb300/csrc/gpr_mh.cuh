/*
 * gpr_mh.cuh -- the GB300 (sm_103a) hot path of the sampler.
 *
 * One warp owns one chain at a time (the reference runs one thread per chain,
 * MH_simple_kernel, main.cu:679-813).  For each MH step the warp
 *   1. proposes: a structure move every 5th step (main.cu:699-742) or a move
 *      of every constant (main.cu:743-806), the constants spread over the 32
 *      lanes with a speculative jump-ahead of the chain's random stream;
 *   2. compiles the heap tree (main.cu:371-393) into a reachable-only postfix
 *      program (only after structure moves: constant moves keep the program);
 *   3. evaluates the program with data points strided across lanes, K points
 *      per lane per pass, every opcode warp-uniform (no divergence), value
 *      stack in shared memory, FP32 arithmetic (main.cu:397-444);
 *   4. forms the Gaussian log-likelihood from a warp-shuffle reduction
 *      (main.cu:454-468) and the description-length + Cauchy prior
 *      (main.cu:529-544), then applies the reference's accept rule
 *      (main.cu:728-740, 790-802) with its exact short-circuit order of draws.
 * The grid is persistent (a few CTAs per SM); warps fetch the next chain from
 * a global counter, which balances chains of very different program sizes.
 * Each CTA stages the dataset into shared memory with one bulk TMA copy
 * (cp.async.bulk + mbarrier) before any warp starts.
 */
#ifndef GPR_MH_CUH
#define GPR_MH_CUH
#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include <math.h>

#include "gpr_common.h"
#include "gpr_rngmath.h"
#include "gpr_philox.h"
#include "gpr_kernels.cuh"
#include "gpr_fastmath.cuh"

namespace gpr {

#define FULLMASK 0xffffffffu

__host__ __device__ __forceinline__ size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

/* ------------------------------------------------------------------------ */
/* Double-float ("df") numbers: value = hi + lo, |lo| <= ulp(hi)/2, built from
 * error-free transforms (Knuth's TwoSum, Dekker's Fast2Sum).  Every Bayes
 * quantity of a chain (prior, likelihood, posterior, the accumulated
 * forward/backward proposal log-densities, the acceptance log-ratio) is a df
 * times 2^64, i.e. stored at the scale 2^-64: FP32 exponents then cover the
 * whole range the reference's doubles reach in practice (|x| < 6e57), while
 * every operation stays on the FP32 pipes. */
#define GPR_DF_SCALE 5.42101086242752217e-20f  /* 2^-64 */
#define GPR_DF_UNSCALE 1.8446744073709552e19   /* 2^64  */

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_make(float hi, float lo) { df r; r.hi = hi; r.lo = lo; return r; }
__device__ __forceinline__ df df_neg(df a) { return df_make(-a.hi, -a.lo); }
__device__ __forceinline__ df df_add(df a, df b) {
    const float s = __fadd_rn(a.hi, b.hi);
    if (!isfinite(s)) return df_make(s, 0.0f);
    const float v = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, e);
    return df_make(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ bool df_invalid(df a) { return !isfinite(a.hi); }
__device__ __forceinline__ bool df_gt0(df a) { return a.hi > 0.0f || (a.hi == 0.0f && a.lo > 0.0f); }
__device__ __forceinline__ double df_to_double_unscaled(df a) {
    return ((double)a.hi + (double)a.lo) * GPR_DF_UNSCALE;
}
__device__ __forceinline__ df warp_sum_df(df a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        df b = df_make(__shfl_xor_sync(FULLMASK, a.hi, o), __shfl_xor_sync(FULLMASK, a.lo, o));
        a = df_add(a, b);
    }
    return a;
}
/* -PRIOR_MULTIPLIER * length * log(NOPS+1) (main.cu:536), exact product of the
 * integer-valued length with the double-float constant. */
__device__ __forceinline__ df length_prior(float length, const KParams& p) {
    const float L = -length;
    const float ph = __fmul_rn(L, p.ln1_hi);
    float e = __fmaf_rn(L, p.ln1_hi, -ph);
    e = __fmaf_rn(L, p.ln1_lo, e);
    if (!isfinite(ph)) return df_make(ph, 0.0f);
    const float h = __fadd_rn(ph, e);
    return df_make(h, __fsub_rn(e, __fsub_rn(h, ph)));
}


/* ------------------------------------------------------------------------ */
/* Random stream of one chain.  LCG: s is the 31-bit state.  Philox: s is the
 * index of the next draw; a 4-word block is cached. */
struct Rng {
    uint32_t s;
    uint32_t key0, key1;
    uint32_t blk;
    uint32_t w0, w1, w2, w3;
    uint32_t drawn;      /* draws consumed since the last reset */
};

__device__ __forceinline__ uint32_t magic_div(uint32_t x, Magic m) {
    return (uint32_t)(((uint64_t)x * (uint64_t)m.m) >> m.s);
}

template <int RNG>
__device__ __forceinline__ uint32_t rng_next(Rng& r) {
    r.drawn++;
    if (RNG == 0) {
        r.s = (r.s * 1103515245u + 12345u) & 0x7fffffffu;
        return r.s;
    } else {
        uint32_t b = r.s >> 2;
        if (b != r.blk) {
            uint32_t c[4] = {b, 0u, 0u, 0u};
            gpr_philox4x32_10(c, r.key0, r.key1);
            r.w0 = c[0]; r.w1 = c[1]; r.w2 = c[2]; r.w3 = c[3];
            r.blk = b;
        }
        uint32_t i = r.s & 3u;
        uint32_t v = (i == 0) ? r.w0 : (i == 1) ? r.w1 : (i == 2) ? r.w2 : r.w3;
        r.s++;
        return v >> 1;
    }
}

/* Advance by k draws without producing them. */
template <int RNG>
__device__ __forceinline__ void rng_jump(Rng& r, uint32_t k, const KParams& p) {
    if (RNG == 0) {
        uint32_t x = r.s;
#pragma unroll
        for (int b = 0; b < 20; ++b)
            if ((k >> b) & 1u) x = p.lcgA[b] * x + p.lcgC[b];
        r.s = x & 0x7fffffffu;
    } else {
        r.s += k;
    }
}

/* random_int (main.cu:218-228): divisor = MY_RAND_MAX/(n+1), reject >= n. */
template <int RNG>
__device__ __forceinline__ int random_int(Rng& r, int n, Magic m) {
    uint32_t v;
    do { v = magic_div(rng_next<RNG>(r), m); } while (v >= (uint32_t)n);
    return (int)v;
}

/* random_float (main.cu:230-232). */
template <int RNG>
__device__ __forceinline__ float random_float(Rng& r, const KParams& p) {
    return gpr_rng_k_over_1e6(random_int<RNG>(r, 1000000, p.mag_1e6));
}

/* random_normal (main.cu:237-241), Box-Muller with the project log/sin. */
template <int RNG>
__device__ __forceinline__ float random_normal(Rng& r, const KParams& p) {
    float u = random_float<RNG>(r, p);
    float v = random_float<RNG>(r, p);
    float a = __fsqrt_rn(__fmul_rn(-2.0f, gpr_rng_logf(u)));
    return __fmul_rn(a, gpr_rng_sinf(gpr_rng_twopi_times(v)));
}

/* random_geometric (main.cu:251-254). */
template <int RNG>
__device__ __forceinline__ float random_geometric(Rng& r, const KParams& p) {
    return ceilf(__fdiv_rn(gpr_rng_logf(random_float<RNG>(r, p)), p.geom_logr));
}


/* ------------------------------------------------------------------------ */
/* Heap-tree compiler.  Node j is 1-based, children 2j and 2j+1; a child index
 * beyond PL is the leaf x (main.cu:374-385).  The reachable nodes become a
 * postfix program (gpr_common.h); length and node count come with it. */


struct CompileOut {
    int ninstr;
    float length;   /* dispatch_length fold, main.cu:477-526 (X_LENGTH_PRIOR = 1) */
    int count;      /* dispatch_countnodes fold, main.cu:553-601                 */
};

__device__ __forceinline__ int unary_code(int o) {
    switch (o) {
        case OP_INV: return U_INV;   case OP_LOG: return U_LOG;   case OP_EXP: return U_EXP;
        case OP_SQRT: return U_SQRT; case OP_SIN: return U_SIN;   case OP_ASIN: return U_ASIN;
        case OP_COS: return U_COS;   case OP_ACOS: return U_ACOS; case OP_TAN: return U_TAN;
        case OP_ATAN: return U_ATAN; default: return U_ABS;
    }
}
/* base op and operand order of a binary heap op: value = bop(u, v) with
 * u, v the (left, right) child values or (right, left) for the R-variants */
__device__ __forceinline__ int binary_bop(int o, int& swapped) {
    swapped = (o == OP_RMINUS || o == OP_RDIV || o == OP_RPOW);
    switch (o) {
        case OP_PLUS: return BOP_ADD;
        case OP_MINUS: case OP_RMINUS: return BOP_SUB;
        case OP_TIMES: return BOP_MUL;
        case OP_DIV: case OP_RDIV: return BOP_DIV;
        default: return BOP_POW;
    }
}

/* ------------------------------------------------------------------------ */
/* Lane-parallel compiler: the program a depth-first post-order walk would
 * emit, built level by level over the heap instead.
 *  1. bottom-up over the heap levels: resolve A/B pass-through chains, classify
 *     each node as leaf (x, 1, a constant) or subtree, and for subtrees compute
 *     the number of instructions, the description length and the node count;
 *  2. top-down: every reachable subtree root writes its own one or two
 *     instructions at its post-order position and hands its children their
 *     start positions.
 * The per-node scratch (resolved node, instruction count, length, count,
 * start) lives in the warp's shared region, free between proposal and
 * evaluation.  Resolved codes: j > 0 a subtree rooted at node j (1-based),
 * PL_X (x1 beyond the heap) / PL_ONE / PL_NAN / PL_X1N (an x1 node) / PL_X2 /
 * PL_X3 leaves, PL_C0 - i the constant of node i. */
#define PL_X 0
#define PL_ONE (-1)
#define PL_NAN (-2)
#define PL_X1N (-3)
#define PL_X2 (-4)
#define PL_X3 (-5)
#define PL_C0 (-6)

/* NV: input variables of the kernel; with one, x2 and x3 never occur (the
 * host rejects them), and their cases are compiled out to keep the
 * compiler's code small. */
template <int NV>
__device__ __forceinline__ uint32_t pl_load_instr(int r) {
    if (r == PL_X || r == PL_X1N) return I_LDX;
    if (r == PL_ONE) return I_LD1;
    if (r == PL_NAN) return I_LDNAN;
    if (NV > 1 && (r == PL_X2 || r == PL_X3)) return r == PL_X2 ? I_LDX2 : I_LDX3;
    return I_LDC | ((uint32_t)(PL_C0 - r) << 8);
}
template <int NV>
__device__ __forceinline__ uint32_t pl_bin_instr(int bop, int accleft, int r, bool pop) {
    if (pop) return GPR_BIN(bop, accleft, SRC_POP);
    if (r == PL_X || r == PL_X1N) return GPR_BIN(bop, accleft, SRC_X);
    if (r == PL_ONE) return GPR_BIN(bop, accleft, SRC_ONE);
    if (NV > 1 && (r == PL_X2 || r == PL_X3)) return GPR_BIN(bop, accleft, r == PL_X2 ? SRC_X2 : SRC_X3);
    if (r == PL_NAN) return GPR_BIN(bop, accleft, SRC_C) | (255u << 8);
    return GPR_BIN(bop, accleft, SRC_C) | ((uint32_t)(PL_C0 - r) << 8);
}

struct CompileScratch {
    int* res;      /* resolved code per heap node (index j, 1-based)        */
    int* icnt;     /* instructions of the subtree rooted at j               */
    float* len;    /* description length of that subtree                    */
    int* cnt;      /* node count of that subtree                            */
    int* start;    /* first instruction of that subtree, -1 if unreachable  */
};

__device__ __forceinline__ CompileScratch compile_scratch(float* region, int PL) {
    const size_t n = align16((size_t)PL + 1);
    CompileScratch c;
    c.res = (int*)region;
    c.icnt = c.res + n;
    c.len = (float*)(c.icnt + n);
    c.cnt = (int*)(c.len + n);
    c.start = c.cnt + n;
    return c;
}

__device__ __forceinline__ int child_res(const CompileScratch& cs, int PL, int j) {
    return j > PL ? PL_X : cs.res[j];
}
__device__ __forceinline__ float leaf_len(int r) { return r == PL_NAN ? __int_as_float(0x7fc00000) : 1.0f; }
__device__ __forceinline__ int leaf_cnt(int r) { return r == PL_X ? 0 : 1; }

template <int NV>
static __device__ CompileOut compile_parallel(const uint8_t* ops, int PL, gpr_word* prog, const CompileScratch& cs,
                                       int lane) {
    int D = 0;
    while ((2 << D) <= PL) ++D;     /* deepest heap level */
    /* 1. bottom-up */
#pragma unroll 1
    for (int d = D; d >= 0; --d) {
        const int lo = 1 << d, hi = min((2 << d) - 1, PL);
#pragma unroll 1
        for (int j = lo + lane; j <= hi; j += 32) {
            const int o = ops[j - 1];
            const int cls = gpr_op_class(o);
            int r = j;
            if (cls == CLS_PASS_A) r = child_res(cs, PL, 2 * j);
            else if (cls == CLS_PASS_B) r = child_res(cs, PL, 2 * j + 1);
            else if (o == OP_ONE) r = PL_ONE;
            else if (o == OP_CONST) r = PL_C0 - (j - 1);
            else if (o >= OP_X1 && o <= (NV > 1 ? OP_X3 : OP_X1)) r = PL_X1N - (o - OP_X1);   /* x1, x2, x3 */
            else if (cls == CLS_INVALID) r = PL_NAN;
            cs.res[j] = r;
            cs.start[j] = -1;
            if (r == j) {
                int ic;
                float ln;
                int cn;
                if (cls == CLS_UNARY || cls == CLS_CUNARY) {
                    const int L = child_res(cs, PL, 2 * j);
                    const bool lc = L > 0;
                    ic = lc ? cs.icnt[L] + 1 : 2;
                    ln = (cls == CLS_CUNARY ? 2.0f : 1.0f) + (lc ? cs.len[L] : leaf_len(L));
                    cn = 1 + (lc ? cs.cnt[L] : leaf_cnt(L));
                } else {
                    const int L = child_res(cs, PL, 2 * j), R = child_res(cs, PL, 2 * j + 1);
                    const bool lc = L > 0, rc = R > 0;
                    ic = (lc ? cs.icnt[L] : 0) + (rc ? cs.icnt[R] : 0) + ((lc && rc) ? 2 : (lc || rc) ? 1 : 2);
                    ln = 1.0f + (lc ? cs.len[L] : leaf_len(L)) + (rc ? cs.len[R] : leaf_len(R));
                    cn = 1 + (lc ? cs.cnt[L] : leaf_cnt(L)) + (rc ? cs.cnt[R] : leaf_cnt(R));
                }
                cs.icnt[j] = ic; cs.len[j] = ln; cs.cnt[j] = cn;
            }
        }
        __syncwarp();
    }
    CompileOut out;
    const int r0 = PL >= 1 ? cs.res[1] : PL_X;
    if (r0 <= 0) {
        if (lane == 0) { prog[0] = pl_load_instr<NV>(r0); prog[1] = I_END; }
        out.ninstr = 2; out.length = leaf_len(r0); out.count = leaf_cnt(r0);
        __syncwarp();
        return out;
    }
    out.ninstr = cs.icnt[r0] + 1;
    out.length = cs.len[r0];
    out.count = cs.cnt[r0];
    if (lane == 0) { cs.start[r0] = 0; prog[cs.icnt[r0]] = I_END; }
    __syncwarp();
    /* 2. top-down */
#pragma unroll 1
    for (int d = 0; d <= D; ++d) {
        const int lo = 1 << d, hi = min((2 << d) - 1, PL);
#pragma unroll 1
        for (int j = lo + lane; j <= hi; j += 32) {
            const int st = cs.start[j];
            if (st < 0 || cs.res[j] != j) continue;
            const int o = ops[j - 1];
            const int cls = gpr_op_class(o);
            if (cls == CLS_UNARY || cls == CLS_CUNARY) {
                uint32_t ui;
                if (o == OP_CPLUS) ui = GPR_BIN(BOP_ADD, 1, SRC_C);
                else if (o == OP_CTIMES) ui = GPR_BIN(BOP_MUL, 1, SRC_C);
                else if (o == OP_CPOW) ui = GPR_BIN(BOP_POW, 1, SRC_C);
                else if (o == OP_CRPOW) ui = GPR_BIN(BOP_POW, 0, SRC_C);
                else ui = (uint32_t)unary_code(o);
                ui |= ((uint32_t)(j - 1) << 8);
                const int L = child_res(cs, PL, 2 * j);
                if (L > 0) { cs.start[L] = st; prog[st + cs.icnt[L]] = ui; }
                else { prog[st] = pl_load_instr<NV>(L); prog[st + 1] = ui; }
            } else {
                int sw;
                const int bop = binary_bop(o, sw);
                const int U = child_res(cs, PL, sw ? 2 * j + 1 : 2 * j);
                const int V = child_res(cs, PL, sw ? 2 * j : 2 * j + 1);
                if (U <= 0 && V <= 0) {
                    prog[st] = pl_load_instr<NV>(U);
                    prog[st + 1] = pl_bin_instr<NV>(bop, 1, V, false);
                } else if (U > 0 && V <= 0) {
                    cs.start[U] = st;
                    prog[st + cs.icnt[U]] = pl_bin_instr<NV>(bop, 1, V, false);
                } else if (U <= 0 && V > 0) {
                    cs.start[V] = st;
                    prog[st + cs.icnt[V]] = pl_bin_instr<NV>(bop, 0, U, false);
                } else {
                    cs.start[U] = st;
                    prog[st + cs.icnt[U]] = I_PUSH;
                    cs.start[V] = st + cs.icnt[U] + 1;
                    prog[st + cs.icnt[U] + 1 + cs.icnt[V]] = pl_bin_instr<NV>(bop, 0, 0, true);
                }
            }
        }
        __syncwarp();
    }
    return out;
}

/* An estimate of a compiled program's evaluation time per pass, in issued
 * instructions at four points per lane: the interpreter's dispatch plus the
 * operation (pow, log, exp and division are tens of instructions each, an
 * add one per point).  It orders a CTA's evaluation tasks longest first. */
__device__ __forceinline__ int instr_cost(uint32_t ins) {
    const uint32_t code = ins & 0xffu;
    int body;
    if (code >= I_BIN0) {
        const uint32_t bop = GPR_BIN_BOP(code);
        body = bop == BOP_POW ? 280 : bop == BOP_DIV ? 36 : 4;
    } else {
        switch (code) {
            case I_END: return 0;
            case U_EXP: body = 60; break;
            case U_LOG: body = 100; break;
            case U_SQRT: case U_INV: body = 36; break;
            case U_SIN: case U_ASIN: case U_COS: case U_ACOS: case U_TAN: case U_ATAN: body = 160; break;
            default: body = 4; break;
        }
    }
    return 25 + body;
}
__device__ __forceinline__ int program_cost(const gpr_word* prog, int ninstr, int lane) {
    int c = 0;
#pragma unroll 1
    for (int i = lane; i < ninstr; i += 32) c += instr_cost(prog[i]);
    return (int)__reduce_add_sync(FULLMASK, (unsigned)c);
}

/* The program the evaluator runs: each instruction word paired with the
 * constant it reads (NaN for the invalid-op marker), so one 64-bit shared
 * load fetches both.  Rebuilt for every proposal, lanes in parallel. */
__device__ __forceinline__ void build_eval_program(const gpr_word* prog, const float* Cs, int ninstr,
                                                   uint2* eprog, int lane) {
#pragma unroll 1
    for (int i = lane; i < ninstr; i += 32) {
        const uint32_t ins = prog[i];
        const uint32_t node = (ins >> 8) & 0xffu;
        const float c = (node == 255u) ? __int_as_float(0x7fc00000) : Cs[node];
        eprog[i] = make_uint2(ins, __float_as_uint(c));
    }
}

/* ------------------------------------------------------------------------ */
/* The evaluator: acc[k] = f(x[k]) for this lane's K points.
 *
 * Arithmetic, exp, log, pow and sqrt run unrolled over the K values in
 * registers, with the compact routines of gpr_fastmath.cuh.  The trigonometric
 * ops (CUDA's math library, with large-argument reduction paths) run through
 * one non-unrolled loop over the K values staged in the warp's shared scratch,
 * so the kernel carries a single copy of each: with every warp of an SM
 * executing a different program, instruction-cache footprint, not FP32
 * throughput, limits an interpreter. */
enum gpr_hop { H_EXP, H_LOG, H_SQRT, H_INV, H_DIV, H_POW, H_SIN, H_ASIN, H_COS, H_ACOS, H_TAN, H_ATAN };

__device__ __forceinline__ int trig_hop(uint32_t code) {
    switch (code) {
        case U_SIN: return H_SIN;   case U_ASIN: return H_ASIN; case U_COS: return H_COS;
        case U_ACOS: return H_ACOS; case U_TAN: return H_TAN;   case U_ATAN: return H_ATAN;
        default: return -1;
    }
}

/* One non-unrolled pass over this lane's K staged values: scr[k*32 + lane]
 * holds first operands u, scr[(K+k)*32 + lane] second operands w; results
 * replace u.  The single copy of each routine keeps the code footprint small. */
template <int K>
__device__ __noinline__ void heavy_loop(float* __restrict__ scr, int hop, int lane) {
#pragma unroll 1
    for (int k = 0; k < K; ++k) {
        const float u = scr[k * 32 + lane];
        const float w = scr[(K + k) * 32 + lane];
        float r;
        switch (hop) {
            case H_EXP: r = gx_exp(u); break;
            case H_LOG: r = gx_log(u); break;
            case H_SQRT: r = __fsqrt_rn(u); break;
            case H_INV: r = __fdiv_rn(1.0f, u); break;
            case H_DIV: r = __fdiv_rn(u, w); break;
            case H_POW: r = gx_pow(u, w); break;
            case H_SIN: r = sinf(u); break;
            case H_ASIN: r = asinf(u); break;
            case H_COS: r = cosf(u); break;
            case H_ACOS: r = acosf(u); break;
            case H_TAN: r = tanf(u); break;
            default: r = atanf(u); break;
        }
        scr[k * 32 + lane] = r;
    }
}

template <int K>
__device__ __forceinline__ void heavy_staged(float (&acc)[K], const float (&w)[K], float* scr, int hop,
                                             int lane) {
#pragma unroll
    for (int k = 0; k < K; ++k) { scr[k * 32 + lane] = acc[k]; scr[(K + k) * 32 + lane] = w[k]; }
    heavy_loop<K>(scr, hop, lane);
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = scr[k * 32 + lane];
}

/* acc = f(acc) / acc = op(acc, v) / acc = op(v, acc) for one instruction.
 * ROLLED: division, pow, exp, log, sqrt and 1/x go through heavy_loop (small
 * code, one value at a time); otherwise they are unrolled over K in registers
 * (more code, full ILP).  Which is faster depends on how much of the kernel
 * the instruction cache holds; gpr_autotune measures it. */
/* Where the interpreter fetches instruction i and the constant it reads:
 * an evaluation program of (instruction, constant) pairs, or (PCProg) the
 * compiled program and the chain's constants array, the constant of heap node
 * n being cs[n] (NaN for the invalid-op marker 255). */
struct PCProg {
    const gpr_word* p;
    const float* cs;
};
__device__ __forceinline__ uint2 prog_at(const uint2* e, int i) { return e[i]; }
__device__ __forceinline__ uint2 prog_at(const PCProg& q, int i) {
    const uint32_t ins = q.p[i];
    const uint32_t node = (ins >> 8) & 0xffu;
    const float c = node == 255u ? __int_as_float(0x7fc00000) : q.cs[node];
    return make_uint2(ins, __float_as_uint(c));
}

template <int K, bool ROLLED, int NV, class PR>
__device__ __forceinline__ void run_program(const PR prog,
                                            const float (&x)[NV][K], float (&acc)[K],
                                            float* __restrict__ stk, float* __restrict__ scr,
                                            int lane) {
    int sp = 0;
    int pc = 0;
    uint2 insw = prog_at(prog, 0);
#pragma unroll 1
    for (;;) {
        const uint32_t ins = insw.x;
        const uint32_t code = ins & 0xffu;
        if (code == I_END) break;
        const uint2 nxt = prog_at(prog, pc + 1);   /* the program ends with I_END: always in bounds */
        ++pc;
        const float c = __uint_as_float(insw.y);
        if (code >= I_BIN0) {
            const uint32_t bop = GPR_BIN_BOP(code);
            const uint32_t accleft = GPR_BIN_ACCLEFT(code);
            const uint32_t src = GPR_BIN_SRC(code);
            float v[K];
            if (src == SRC_X) {
#pragma unroll
                for (int k = 0; k < K; ++k) v[k] = x[0][k];
            } else if (src == SRC_C) {
#pragma unroll
                for (int k = 0; k < K; ++k) v[k] = c;
            } else if (src == SRC_ONE) {
#pragma unroll
                for (int k = 0; k < K; ++k) v[k] = 1.0f;
            } else if (NV > 1 && src != SRC_POP) {
                const int vi = NV > 1 ? (int)(src - SRC_X2) + 1 : 0;
#pragma unroll
                for (int k = 0; k < K; ++k) v[k] = x[vi][k];
            } else {
                --sp;
#pragma unroll
                for (int k = 0; k < K; ++k) v[k] = stk[(sp * K + k) * 32 + lane];
            }
            if (bop == BOP_ADD) {            /* commutative: operand order is irrelevant */
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = __fadd_rn(acc[k], v[k]);
            } else if (bop == BOP_MUL) {
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = __fmul_rn(acc[k], v[k]);
            } else if (bop == BOP_SUB) {
                if (accleft) {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = __fsub_rn(acc[k], v[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = __fsub_rn(v[k], acc[k]);
                }
            } else {
                /* DIV, POW: bring the operands into (u, w) order */
                if (!accleft) {
#pragma unroll
                    for (int k = 0; k < K; ++k) { const float t = acc[k]; acc[k] = v[k]; v[k] = t; }
                }
                if (ROLLED) {
                    heavy_staged<K>(acc, v, scr, bop == BOP_DIV ? H_DIV : H_POW, lane);
                } else if (bop == BOP_DIV) {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = __fdiv_rn(acc[k], v[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = gx_pow(acc[k], v[k]);
                }
            }
            goto next_ins;
        }
        if (NV > 1 && (code == I_LDX2 || code == I_LDX3)) {
            const int vi = NV > 1 ? (code == I_LDX2 ? 1 : 2) : 0;
#pragma unroll
            for (int k = 0; k < K; ++k) acc[k] = x[vi][k];
            goto next_ins;
        }
        switch (code) {
            case I_LDX:
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = x[0][k];
                break;
            case I_LDC:
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = c;
                break;
            case I_LD1:
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = 1.0f;
                break;
            case I_LDNAN:
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = __int_as_float(0x7fc00000);
                break;
            case I_PUSH:
#pragma unroll
                for (int k = 0; k < K; ++k) stk[(sp * K + k) * 32 + lane] = acc[k];
                ++sp;
                break;
            case U_ABS:
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = fabsf(acc[k]);
                break;
            case U_EXP:
            case U_LOG:
            case U_SQRT:
            case U_INV:
                if (ROLLED) {
                    heavy_staged<K>(acc, acc, scr,
                                    code == U_EXP ? H_EXP : code == U_LOG ? H_LOG : code == U_SQRT ? H_SQRT : H_INV,
                                    lane);
                } else if (code == U_EXP) {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = gx_exp(acc[k]);
                } else if (code == U_LOG) {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = gx_log(acc[k]);
                } else if (code == U_SQRT) {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = __fsqrt_rn(acc[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = __fdiv_rn(1.0f, acc[k]);
                }
                break;
            default: {
                const int hop = trig_hop(code);
                if (hop >= 0) heavy_staged<K>(acc, acc, scr, hop, lane);
                break;
            }
        }
    next_ins:
        insw = nxt;
    }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
    return v;
}

/* Shared-memory pointers of one warp.  The constant-move records (off, ndr,
 * fw, bw) are only live during a constant proposal, the value stack and the
 * transcendental scratch only during an evaluation, so they share one region. */
struct WarpSmem {
    uint8_t* ops[2];
    float* Cs[2];
    gpr_word* prog[2];
    uint2* eprog;    /* evaluation program: (instruction, constant) pairs */
    int* off;        /* per constant: offset of its first draw   */
    int* ndr;        /* per constant: draws used                 */
    float* fw;       /* per constant: forward log-density term   */
    float* bw;       /* per constant: backward log-density term  */
    float* stk;      /* value stack: [levels][K][32]             */
    float* scr;      /* transcendental staging: [2K][32]         */
};


__host__ __device__ __forceinline__ size_t shared_region_bytes(int PL, int levels, int K) {
    const size_t eval = (size_t)(levels + 2) * K * 32 * 4;
    const size_t cmove = 4 * align16((size_t)PL) * 4;
    const size_t comp = 5 * align16((size_t)PL + 1) * 4;
    size_t m = eval > cmove ? eval : cmove;
    m = m > comp ? m : comp;
    return align16(m);
}

/* eprog: with an evaluation program of (instruction, constant) pairs; the MH
 * kernels interpret program and constants in place and have none. */
__host__ __device__ __forceinline__ size_t warp_smem_bytes(int PL, int max_instr, int levels, int K,
                                                           bool eprog = true) {
    size_t plp = align16((size_t)PL);
    size_t b = 0;
    b += 2 * plp;                                /* ops */
    b += align16(2 * plp * 4);                   /* Cs */
    b += align16(2 * (size_t)max_instr * sizeof(gpr_word));     /* prog */
    if (eprog) b += align16((size_t)max_instr * 8);   /* eprog */
    b += shared_region_bytes(PL, levels, K);     /* stack + scratch | constant-move records */
    return align16(b);
}

template <int K>
__device__ __forceinline__ WarpSmem carve_warp(uint8_t* base, int PL, int max_instr, int levels, bool eprog = true) {
    WarpSmem w;
    size_t plp = align16((size_t)PL);
    uint8_t* p = base;
    w.ops[0] = p; w.ops[1] = p + plp; p += 2 * plp;
    w.Cs[0] = (float*)p; w.Cs[1] = (float*)p + plp; p += align16(2 * plp * 4);
    w.prog[0] = (gpr_word*)p; w.prog[1] = (gpr_word*)p + max_instr; p += align16(2 * (size_t)max_instr * sizeof(gpr_word));
    w.eprog = nullptr;
    if (eprog) { w.eprog = (uint2*)p; p += align16((size_t)max_instr * 8); }
    w.stk = (float*)p;
    w.scr = w.stk + (size_t)levels * K * 32;
    w.off = (int*)p;
    w.ndr = w.off + plp;
    w.fw = (float*)(w.ndr + plp);
    w.bw = w.fw + plp;
    return w;
}

/* The dataset as the evaluators read it: the CTA's shared-memory copy
 * (arrays of nd_pad floats in the staging order x1 | y | w | x2 | x3, 16
 * bytes into the dynamic shared memory, after the staging barrier), or the
 * device arrays when streamed.  x[1], x[2] only for multivariate data. */
struct DataView {
    const float* x[3];
    const float* y;
    const float* w;
    int nd, nd_pad;           /* points, and the padded array length       */
    float ns_hi, ns_lo;       /* 2^-64 * its normalising sum, double-float (Hamiltonian kernel) */
    double ns64;              /* its normalising sum (MH kernels)          */
};

/* The dynamic shared memory of the kernel running (every extern __shared__
 * array starts at its base).  Staged data are addressed from this symbol, so
 * the loads are shared-memory loads at constant offsets. */
extern __shared__ __align__(128) uint8_t gpr_dyn_smem[];
#define GPR_STAGED_OFFSET 16

/* Dataset array indices in the staging order. */
#define DA_X1 0
#define DA_Y 1
#define DA_W 2
#define DA_X2 3
#define DA_X3 4

/* Point i of dataset array a: from the staged copy in shared memory, or from
 * the device arrays when streamed. */
template <bool STREAM>
__device__ __forceinline__ float data_at(const DataView& dv, int a, int i) {
    if (STREAM) {
        const float* q = a == DA_X1 ? dv.x[0] : a == DA_Y ? dv.y : a == DA_W ? dv.w : a == DA_X2 ? dv.x[1] : dv.x[2];
        return q[i];
    }
    return ((const float*)(gpr_dyn_smem + GPR_STAGED_OFFSET))[a * dv.nd_pad + i];
}

/* This lane's K points of one pass: the NV input variables, and which points
 * exist (bit k). */
template <int K, int NV, bool STREAM>
__device__ __forceinline__ uint32_t load_points(const DataView& dv, const KParams& p, int base,
                                                float (&x)[NV][K]) {
    uint32_t valid = 0u;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = base + 32 * k;
        const bool v = i < dv.nd;
#pragma unroll
        for (int j = 0; j < NV; ++j) x[j][k] = v ? data_at<STREAM>(dv, j == 0 ? DA_X1 : DA_X1 + 2 + j, i) : 0.0f;
        valid |= (v ? 1u : 0u) << k;
    }
    return valid;
}

/* Per-lane data of the single-pass layout (nd <= 32*K). */
template <int K>
struct LaneData {
    float x[K];
    uint32_t valid;  /* bit k: point lane + 32k exists */
};

/* ---- the likelihood's reduction tree ----
 * Fixed by point index, so that every layout (points per lane, data staged
 * or streamed, chains balanced over a CTA or not) gives the same bits: the
 * points are taken in chunks of 128 (chunk c = points 128c .. 128c+127, lane
 * l holding points 128c + l + 32k, k = 0..3); each lane sums its four terms
 * (f - y)^2 w in FP32 in k order, the 32 lane sums are combined by an FP32
 * xor butterfly, and the chunk sums are added as double-floats in chunk
 * order (main.cu:454-468 sums every point in double).  The weights carry the
 * factor 2^-e (KParams::lik_unscale), so S, the sum of a chain's terms, is a
 * double-float at the scale 2^-e that cannot overflow. */
#define GPR_CHUNK_POINTS 128

__device__ __forceinline__ int chunk_count(int nd) { return (nd + GPR_CHUNK_POINTS - 1) / GPR_CHUNK_POINTS; }

/* One pass of a program over this lane's K points (pass q covers points
 * [32Kq, 32K(q+1)), lane l holding points 32Kq + l + 32k): the FP32 sums of
 * the pass's K/4 chunks, the same in every lane, and whether any point is
 * invalid (main.cu:459,462), the same in every lane. */
template <int K, bool ONEPASS, bool ROLLED, int NV, bool STREAM, class PR>
__device__ __forceinline__ bool eval_pass_chunks(const PR prog, float* stk, float* scr, const LaneData<K>& ld,
                                                 const DataView& dv, const KParams& p, int lane, int pass,
                                                 float (&cs)[K / 4]) {
    float x[NV][K], acc[K];
    uint32_t valid;
    const int base = pass * 32 * K + lane;
    if (ONEPASS) {
#pragma unroll
        for (int k = 0; k < K; ++k) x[0][k] = ld.x[k];
        valid = ld.valid;
    } else {
        valid = load_points<K, NV, STREAM>(dv, p, base, x);
    }
    run_program<K, ROLLED, NV>(prog, x, acc, stk, scr, lane);
    bool bad = false;
#pragma unroll
    for (int j = 0; j < K / 4; ++j) {
        float s = 0.0f;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int k = 4 * j + kk;
            if (valid & (1u << k)) {
                const int i = base + 32 * k;
                const float r = __fsub_rn(acc[k], data_at<STREAM>(dv, DA_Y, i));
                const float q = __fmul_rn(r, r);
                bad |= !(q <= FLT_MAX);
                s = __fmaf_rn(q, data_at<STREAM>(dv, DA_W, i), s);
            }
        }
        cs[j] = s;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int j = 0; j < K / 4; ++j) cs[j] = __fadd_rn(cs[j], __shfl_xor_sync(FULLMASK, cs[j], o));
    return __any_sync(FULLMASK, bad);
}

/* S of an invalid likelihood (-inf, main.cu:459,462). */
__device__ __forceinline__ df lik_invalid() { return df_make(INFINITY, 0.0f); }

/* S of one program evaluated by one warp: the double-float sum of its chunk
 * sums in chunk order, or +inf when any point is invalid. */
template <int K, bool ONEPASS, bool ROLLED, int NV, bool STREAM, class PR>
__device__ __forceinline__ df eval_loglik_S(const PR prog, float* stk, float* scr, const LaneData<K>& ld,
                                            const DataView& dv, const KParams& p, int lane, int& pts) {
    const int npass = ONEPASS ? 1 : (dv.nd + 32 * K - 1) / (32 * K);
    const int nch = chunk_count(dv.nd);
    df S = df_make(0.0f, 0.0f);
#pragma unroll 1
    for (int pass = 0; pass < npass; ++pass) {
        float cs[K / 4];
        const bool bad = eval_pass_chunks<K, ONEPASS, ROLLED, NV, STREAM>(prog, stk, scr, ld, dv, p, lane, pass, cs);
        pts += ONEPASS ? dv.nd : min(32 * K, dv.nd - pass * 32 * K);
        if (bad) return lik_invalid();
#pragma unroll
        for (int j = 0; j < K / 4; ++j)
            if (pass * (K / 4) + j < nch) S = df_add(S, df_make(cs[j], 0.0f));
    }
    return S;
}

/* The log-likelihood (main.cu:454-468) of a chain with sum S, in FP64, for
 * the scores a block writes: -S 2^e - the normalising sum. */
__device__ __forceinline__ double lik_of(df S, const DataView& dv, const KParams& p) {
    if (!isfinite(S.hi)) return -INFINITY;
    return (0.0 - ((double)S.hi + (double)S.lo) * p.lik_unscale) - dv.ns64;
}

/* -length log(NOPS + 1) (main.cu:536): the exact product of the
 * integer-valued length with the double-float constant. */
__device__ __forceinline__ df length_prior_u(float length, const KParams& p) {
    const float L = -length;
    const float ph = __fmul_rn(L, p.ln1u_hi);
    float e = __fmaf_rn(L, p.ln1u_hi, -ph);
    e = __fmaf_rn(L, p.ln1u_lo, e);
    if (!isfinite(ph)) return df_make(ph, 0.0f);
    const float h = __fadd_rn(ph, e);
    return df_make(h, __fsub_rn(e, __fsub_rn(h, ph)));
}

/* Sum over all constants of lcauchypdf(C, 1) (main.cu:303-305, 537-540): the
 * -log(1 + C^2) terms are FP32 (the reference's logf), added exactly as
 * double-floats across the warp; the constant part PL log(PIf) once. */
__device__ __forceinline__ df cauchy_sum_u(const float* Cs, const KParams& p, int lane) {
    df s = df_make(0.0f, 0.0f);
#pragma unroll 1
    for (int c = lane; c < p.PL; c += 32) {
        const float x = Cs[c];
        s = df_add(s, df_make(-gx_log(__fadd_rn(1.0f, __fmul_rn(x, x))), 0.0f));
    }
    s = warp_sum_df(s);
    return df_sub(s, df_make(p.cauchy_c_hi, p.cauchy_c_lo));
}

/* The same sum at the Hamiltonian kernel's bookkeeping scale 2^-64, each
 * FP32 term added exactly (double-float). */
__device__ __forceinline__ df cauchy_sum(const float* Cs, const KParams& p, int lane) {
    df s = df_make(0.0f, 0.0f);
#pragma unroll 1
    for (int c = lane; c < p.PL; c += 32) {
        const float x = Cs[c];
        const float a = __fadd_rn(1.0f, __fmul_rn(x, x));
        s = df_add(s, df_make(__fmul_rn(__fsub_rn(-p.lpi_f, gx_log(a)), GPR_DF_SCALE), 0.0f));
    }
    return warp_sum_df(s);
}

/* The prior (main.cu:529-544) of a program with this length and Cauchy sum. */
__device__ __forceinline__ df prior_u(float length, df cauchy, const KParams& p) {
    return df_add(length_prior_u(length, p), cauchy);
}

/* The acceptance log-ratio of main.cu:728 / 790,
 *   ((proposal posterior - current posterior) + backward) - forward,
 * for two valid states, from the prior difference and the difference of the
 * likelihood sums (the normalising sum cancels): ((dprior - dS 2^e) + bw) - fw
 * as a double-float.  Sets huge when |dS 2^e| >= 2^100 while the other terms
 * are finite: the ratio's sign is then that of -dS and its exponential 0
 * (only that sign is returned). */
__device__ __forceinline__ df accept_ratio(df prior_p, df S_p, df prior_c, df S_c, df bw, df fw, const KParams& p,
                                           bool& huge) {
    const df dS = df_sub(S_p, S_c);
    const df dprior = df_sub(prior_p, prior_c);
    /* |dS.hi| < 2^ex (an upper bound for subnormals too) */
    const int ex = (int)((__float_as_uint(dS.hi) >> 23) & 0xffu) - 126;
    huge = dS.hi != 0.0f && ex + p.lik_e > 100;
    if (huge) {
        const df rest = df_sub(df_add(dprior, bw), fw);
        if (isfinite(rest.hi)) return df_make(dS.hi > 0.0f ? -1.0f : 1.0f, 0.0f);
        huge = false;
    }
    /* dS 2^e, exact: two power-of-two factors, no overflow (|result| < 2^100) */
    const df L = df_make(__fmul_rn(__fmul_rn(dS.hi, p.unscale1), p.unscale2),
                         __fmul_rn(__fmul_rn(dS.lo, p.unscale1), p.unscale2));
    return df_sub(df_add(df_sub(dprior, L), bw), fw);
}

/* The accept rule of main.cu:728-740 / 790-802, in its exact evaluation
 * order: the uniform draw is consumed only when the proposal is valid and the
 * acceptance ratio is not > 0; an invalid current state accepts anything.  A
 * posterior is NaN when its prior is (an invalid op's length), -inf when its
 * prior or likelihood is -inf; a NaN current posterior makes the ratio NaN (a
 * draw, then acceptance), a -inf one makes it +inf (acceptance, no draw).
 * prob, when given, receives min(1, exp(ratio)) for step-size adaptation. */
template <int RNG>
__device__ __forceinline__ bool mh_accept_u(df prior_p, df S_p, df prior_c, df S_c, df bw, df fw, Rng& r,
                                            const KParams& p, float* prob = nullptr) {
    const bool pp_valid = isfinite(prior_p.hi) && isfinite(S_p.hi);
    const bool cp_nan = isnan(prior_c.hi);
    const bool cp_valid = isfinite(prior_c.hi) && isfinite(S_c.hi);
    if (!pp_valid) {
        if (prob) *prob = cp_valid ? 0.0f : 1.0f;
        return !cp_valid;
    }
    if (!cp_valid) {
        if (prob) *prob = 1.0f;
        if (cp_nan) (void)random_float<RNG>(r, p);
        return true;
    }
    bool huge;
    const df a = accept_ratio(prior_p, S_p, prior_c, S_c, bw, fw, p, huge);
    if (huge) {
        if (a.hi > 0.0f) { if (prob) *prob = 1.0f; return true; }
        if (prob) *prob = 0.0f;
        (void)random_float<RNG>(r, p);
        return false;
    }
    if (df_gt0(a)) { if (prob) *prob = 1.0f; return true; }
    const float e = expf(a.hi);
    if (prob) *prob = e;
    return random_float<RNG>(r, p) < e;
}

/* lnormalpdf(x, 1.0) (main.cu:299-301) */
__device__ __forceinline__ float lnormal1(float x, const KParams& p) {
    return __fsub_rn(__fmul_rn(-__fmul_rn(x, x), 0.5f), p.lnorm1_f);
}
/* lgeometricpdf(n, r) (main.cu:307-309) with n = v + 1 */
__device__ __forceinline__ float lgeom_plus1(float v, const KParams& p) {
    float n = __fadd_rn(v, 1.0f);
    return __fadd_rn(__fmul_rn(__fsub_rn(n, 1.0f), p.logf_r), p.log1mr_f);
}
/* is_int (main.cu:192): |x - lroundf(x)| < 1e-6 */
__device__ __forceinline__ bool is_int_ref(float x) {
    if (!(fabsf(x) < 9.2233720368547758e18f)) return false;
    float d = __fsub_rn(x, roundf(x));
    return fabsf(d) <= 9.99999997e-07f;
}

/* One constant's proposal (main.cu:746-785) starting at the stream position
 * held in r.  Writes the new value and the forward/backward terms. */
template <int RNG>
__device__ __forceinline__ void propose_constant(Rng& r, float old, float& nc, float& dfw,
                                                 float& dbw, const KParams& p, float rw_sd) {
    dfw = 0.0f; dbw = 0.0f;
    float u0 = random_float<RNG>(r, p);
    const float p_geom = (p.const_mode == 0) ? 1.0f : 0.0f;   /* P_PROPOSE_C_GEOMETRIC */
    if (u0 < p_geom) {
        float u1 = random_float<RNG>(r, p);
        if (u1 < 0.15f) {                                     /* PROPOSE_INT */
            float u2 = random_float<RNG>(r, p);
            float sgn = (u2 < 0.5f) ? -1.0f : 1.0f;
            float g = random_geometric<RNG>(r, p);
            nc = __fsub_rn(__fmul_rn(sgn, g), 1.0f);
            dfw = __fadd_rn(__fadd_rn(lgeom_plus1(nc, p), (nc == 0.0f) ? 0.0f : p.log2_f), p.logpi_f);
        } else {
            nc = random_normal<RNG>(r, p);
            dfw = __fadd_rn(lnormal1(nc, p), p.log1mpi_f);
        }
        float bn = __fadd_rn(lnormal1(old, p), p.log1mpi_f);
        if (is_int_ref(old)) {
            float bg = __fadd_rn(__fadd_rn(lgeom_plus1(old, p), (nc == 0.0f) ? 0.0f : p.log2_f), p.logpi_f);
            float m = fmaxf(bg, bn);
            dbw = gx_log(gx_exp(bg - m) + gx_exp(bn - m)) + m;
        } else {
            dbw = bn;
        }
    } else {
        float z = random_normal<RNG>(r, p);
        nc = __fadd_rn(old, __fmul_rn(rw_sd, z));
    }
}

/* Constant move of one chain, lanes in parallel.  Draw counts vary (rejection
 * in random_int), so each constant first assumes the nominal count for all
 * earlier constants; a warp prefix sum then gives the true offsets and the
 * constants whose offset changed are redone, until nothing changes. */
/* Affine maps that move an LCG state to the nominal first draw of this
 * lane's constants: c = lane (map) and c -> c + 32 (stride). */
struct LaneJump {
    uint32_t a, c;     /* state -> state after nominal*lane draws        */
    uint32_t sa, sc;   /* state -> state after nominal*32 draws          */
    uint32_t da, dc;   /* state -> state after lane+1 draws              */
};

__device__ __forceinline__ void affine_power(uint32_t k, const KParams& p, uint32_t& A, uint32_t& C) {
    A = 1u; C = 0u;
#pragma unroll 1
    for (int b = 0; b < 20; ++b)
        if ((k >> b) & 1u) { C = p.lcgA[b] * C + p.lcgC[b]; A = p.lcgA[b] * A; }
}

__device__ __forceinline__ LaneJump make_lane_jump(const KParams& p, int lane) {
    const uint32_t nominal = (p.const_mode == 0) ? 4u : 3u;
    LaneJump j;
    affine_power(nominal * (uint32_t)lane, p, j.a, j.c);
    affine_power(nominal * 32u, p, j.sa, j.sc);
    affine_power((uint32_t)lane + 1u, p, j.da, j.dc);
    return j;
}

template <int RNG>
__device__ void constant_move(Rng& r, const WarpSmem& w, const float* Cold, float* Cnew,
                              df& fw_sum, df& bw_sum, const KParams& p, const LaneJump& lj, int lane,
                              float rw_sd) {
    const int PL = p.PL;
    const int nominal = (p.const_mode == 0) ? 4 : 3;
    /* first pass: every constant at its nominal offset, streams positioned by
     * one affine map each (LCG) or a counter offset (Philox) */
    /* the LCG state after the last constant's draws: the stream's state once
     * the offsets have converged */
    uint32_t endst = 0u;
    bool all_nominal = true;   /* this lane's constants drew exactly `nominal` each */
    {
        uint32_t st = (lj.a * r.s + lj.c) & 0x7fffffffu;
#pragma unroll 1
        for (int c = lane; c < PL; c += 32) {
            Rng rc = r;
            if (RNG == 0) rc.s = st;
            else rc.s = r.s + (uint32_t)(nominal * c);
            rc.drawn = 0;
            float nc, dfw, dbw;
            propose_constant<RNG>(rc, Cold[c], nc, dfw, dbw, p, rw_sd);
            Cnew[c] = nc; w.fw[c] = dfw; w.bw[c] = dbw; w.ndr[c] = (int)rc.drawn;
            w.off[c] = nominal * c;
            all_nominal = all_nominal && rc.drawn == (uint32_t)nominal;
            if (c == PL - 1) endst = rc.s;
            st = (lj.sa * st + lj.sc) & 0x7fffffffu;
        }
    }
    __syncwarp();
    bool converged = false;
    /* The usual case (random_int rejects a draw with probability about 1e-6):
     * every constant drew its nominal count, so the nominal offsets are the
     * true ones and the stream continues after the last constant's draws. */
    if (__all_sync(FULLMASK, all_nominal)) {
        if (RNG == 0) r.s = __shfl_sync(FULLMASK, endst, (PL - 1) & 31);
        else rng_jump<RNG>(r, (uint32_t)(nominal * PL), p);
        converged = true;
    }
#pragma unroll 1
    for (int iter = 0; iter <= PL && !converged; ++iter) {
        /* redo the constants whose offset moved (marked ndr < 0) */
        #pragma unroll 1
        for (int c = lane; c < PL; c += 32) {
            if (w.ndr[c] >= 0) continue;
            Rng rc = r;
            rng_jump<RNG>(rc, (uint32_t)w.off[c], p);
            rc.drawn = 0;
            float nc, dfw, dbw;
            propose_constant<RNG>(rc, Cold[c], nc, dfw, dbw, p, rw_sd);
            Cnew[c] = nc; w.fw[c] = dfw; w.bw[c] = dbw; w.ndr[c] = (int)rc.drawn;
            if (c == PL - 1) endst = rc.s;
        }
        __syncwarp();
        /* exclusive prefix sum of draw counts, 32 constants at a time */
        bool changed = false;
        int base = 0;
        #pragma unroll 1
        for (int c0 = 0; c0 < PL; c0 += 32) {
            int c = c0 + lane;
            int v = (c < PL) ? w.ndr[c] : 0;
            int incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(FULLMASK, incl, o);
                if (lane >= o) incl += t;
            }
            int excl = base + incl - v;
            if (c < PL && w.off[c] != excl) { changed = true; w.off[c] = excl; w.ndr[c] = -1; }
            base += __shfl_sync(FULLMASK, incl, 31);
        }
        __syncwarp();
        if (!__any_sync(FULLMASK, changed)) {
            if (RNG == 0) r.s = __shfl_sync(FULLMASK, endst, (PL - 1) & 31);
            else rng_jump<RNG>(r, (uint32_t)base, p);
            converged = true;
        }
    }
    if (!converged && lane == 0) atomicOr(p.err, 2);
    __syncwarp();
    df f = df_make(0.0f, 0.0f), b = df_make(0.0f, 0.0f);
    if (p.const_mode != 0) { fw_sum = f; bw_sum = b; return; }   /* random walk: symmetric, no terms */
    #pragma unroll 1
    for (int c = lane; c < PL; c += 32) {
        f = df_add(f, df_make(w.fw[c], 0.0f));
        b = df_add(b, df_make(w.bw[c], 0.0f));
    }
    fw_sum = warp_sum_df(f);
    bw_sum = warp_sum_df(b);
}

/* ------------------------------------------------------------------------ */
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* Stage the dataset with one bulk TMA copy per array; bounded wait. */
/* Number of float arrays of the staged dataset: x1, y, w, then x2, x3 for
 * multivariate data. */
__host__ __device__ __forceinline__ int data_arrays(const KParams& p) { return p.nv == 3 ? 5 : 3; }

/* The dataset arrays in the order they are staged (device memory). */
__device__ __forceinline__ const float* data_src(const KParams& p, int a) {
    return a == 0 ? p.dx : a == 1 ? p.dy : a == 2 ? p.dw : a == 3 ? p.dx2 : p.dx3;
}

/* Batched data (p.nds > 0): the dataset of chain `chain`. */
__device__ __forceinline__ int chain_dataset(const KParams& p, int chain) {
    return p.nds > 0 ? chain / p.chains_per_ds : -1;
}

/* The view of dataset d (-1: the single dataset): staged at dst (arrays of
 * nd_pad floats, staging order; the region is sized for the largest dataset),
 * or, streamed, the device arrays at the dataset's offset. */
__device__ __forceinline__ DataView data_view(const KParams& p, const float* dst, bool streamed, int d = -1) {
    DataView dv;
    size_t off = 0;
    if (d < 0) {
        dv.nd = p.nd; dv.nd_pad = p.nd_pad; dv.ns_hi = p.normsum_hi; dv.ns_lo = p.normsum_lo;
        dv.ns64 = p.normsum64;
    } else {
        off = (size_t)p.ds_off[d];
        dv.nd = p.ds_n[d]; dv.nd_pad = (dv.nd + 3) & ~3;
        dv.ns_hi = p.ds_ns[2 * d]; dv.ns_lo = p.ds_ns[2 * d + 1];
        dv.ns64 = p.ds_ns64[d];
    }
    if (streamed) {
        dv.x[0] = p.dx + off; dv.y = p.dy + off; dv.w = p.dw + off;
        dv.x[1] = p.dx2 ? p.dx2 + off : nullptr; dv.x[2] = p.dx3 ? p.dx3 + off : nullptr;
    } else {
        const size_t n = (size_t)dv.nd_pad;
        dv.x[0] = dst; dv.y = dst + n; dv.w = dst + 2 * n; dv.x[1] = dst + 3 * n; dv.x[2] = dst + 4 * n;
    }
    return dv;
}

/* Iterations of the staging wait after a timed-out one: the drain of the
 * copy still in flight. */
#define GPR_STAGE_DRAIN_ITERS (1 << 22)

/* Stage the dataset into dst with one bulk TMA copy per array; bounded wait.
 * dv: the view it is staged for (its nd_pad); d: the dataset (-1: the single
 * one).  Re-staging for another dataset (reinit) invalidates and
 * re-initialises the barrier, so every thread must have left the previous
 * wait (a __syncthreads) before.  Returns false, the same in every thread of
 * the CTA, when the copy did not complete within the wait's limit. */
static __device__ bool stage_dataset(float* dst, uint64_t* bar, const KParams& p, const DataView& dv, int d = -1,
                                     bool reinit = false) {
    const uint32_t bytes = (uint32_t)dv.nd_pad * 4u;
    if (bytes == 0) return true;
    const size_t off = d < 0 ? 0 : (size_t)p.ds_off[d];
    const int na = data_arrays(p);
    if (threadIdx.x == 0) {
        uint32_t b = smem_u32(bar);
        if (reinit) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(b) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"((uint32_t)na * bytes)
                     : "memory");
        for (int a = 0; a < na; ++a)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         ::"r"(smem_u32(dst + (size_t)a * dv.nd_pad)), "l"(data_src(p, a) + off), "r"(bytes), "r"(b)
                         : "memory");
    }
    __syncthreads();
    const uint32_t b = smem_u32(bar);
    auto wait = [&](int limit) {
        uint32_t done = 0;
        for (int it = 0; it < limit && !done; ++it) {
            asm volatile("{\n\t.reg .pred P1;\n\t"
                         "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
                         "selp.b32 %0, 1, 0, P1;\n\t}"
                         : "=r"(done) : "r"(b), "r"(0u) : "memory");
        }
        return done;
    };
    uint32_t done = wait(p.stage_wait_iters);
    if (!done) {
        /* report, then wait (bounded again) for this CTA's own copy, so that
         * none is in flight into shared memory when the CTA gives up */
        atomicOr(p.err, 1);
        (void)wait(GPR_STAGE_DRAIN_ITERS);
    }
    return !__syncthreads_or(!done);
}

/* The accept rule of main.cu:728-740 / 790-802, in its exact evaluation order:
 * acceptance = proposal - current + backward - forward; the uniform draw is
 * consumed only when the proposal is valid and acceptance <= 0; an invalid
 * current state accepts anything. */
template <int RNG>
__device__ __forceinline__ bool mh_accept(df ppost, df cur_post, df backward, df forward, Rng& r,
                                          const KParams& p) {
    const df acc = df_sub(df_add(df_sub(ppost, cur_post), backward), forward);
    bool accept = false;
    if (!df_invalid(ppost)) {
        if (df_gt0(acc)) accept = true;
        else accept = random_float<RNG>(r, p) < expf(__fmul_rn(acc.hi, (float)GPR_DF_UNSCALE));
    }
    if (df_invalid(cur_post)) accept = true;
    return accept;
}

/* min(1, exp(acceptance)) of the rule above: the probability the move is
 * taken (1 from an invalid current state, 0 for an invalid proposal).  For
 * step-size adaptation only; the decision itself is mh_accept's. */
__device__ __forceinline__ float accept_prob(df ppost, df cur_post, df backward, df forward) {
    if (df_invalid(cur_post)) return 1.0f;
    if (df_invalid(ppost)) return 0.0f;
    const df acc = df_sub(df_add(df_sub(ppost, cur_post), backward), forward);
    if (df_gt0(acc)) return 1.0f;
    return expf(__fmul_rn(acc.hi, (float)GPR_DF_UNSCALE));
}

/* Robbins-Monro step on the log of a random-walk proposal scale toward a
 * target acceptance rate: log s += (alpha - target) / (m + 10)^0.6 after the
 * m-th move. */
__device__ __forceinline__ float rm_update(float log_s, float alpha, float target, int m) {
    const float gain = __powf((float)(m + 10), -0.6f);
    return fminf(fmaxf(__fadd_rn(log_s, __fmul_rn(gain, __fsub_rn(alpha, target))), -30.0f), 10.0f);
}

/* The value of Philox draw number ctr of a chain's stream (rng_next). */
__device__ __forceinline__ uint32_t philox_draw(uint32_t key0, uint32_t key1, uint32_t ctr) {
    uint32_t c[4] = {ctr >> 2, 0u, 0u, 0u};
    gpr_philox4x32_10(c, key0, key1);
    const uint32_t i = ctr & 3u;
    const uint32_t v = (i == 0) ? c[0] : (i == 1) ? c[1] : (i == 2) ? c[2] : c[3];
    return v >> 1;
}

/* Structure proposal (main.cu:699-742): a node n uniform in [0, PL) -- the
 * root when the current state is invalid -- and every node of its subtree
 * redrawn from the op set in increasing heap order (is_descendant,
 * main.cu:660-677, 711-720), each a random_int(NOPS) with its rejection
 * loop (main.cu:218-228).  The draws are made 32 stream positions at a time,
 * one per lane (the LCG jumped by per-lane affine maps, Philox by counter);
 * the accepted ones, ranked by a ballot, go to the subtree's nodes in order,
 * and the stream is left after the draw that filled the last node -- the
 * sequence of values and the stream position a one-draw-at-a-time loop gives.
 * opn receives the proposal, a copy of oc with that subtree replaced. */
template <int RNG>
__device__ __forceinline__ void structure_move(Rng& r, const uint8_t* oc, uint8_t* opn, bool cur_invalid,
                                               const KParams& p, const LaneJump& lj, int lane) {
    const int PL = p.PL;
    const int n = cur_invalid ? 0 : random_int<RNG>(r, PL, p.mag_pl);
#pragma unroll 1
    for (int i = lane; i < PL; i += 32) opn[i] = oc[i];
    __syncwarp();
    const int m = n + 1;                          /* subtree root, 1-based */
    int T = 0;                                    /* nodes in the subtree  */
#pragma unroll 1
    for (int d = 0; (m << d) <= PL; ++d) T += min((m << d) + (1 << d) - 1, PL) - (m << d) + 1;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t s = r.s;          /* LCG: the state before this round; Philox: the counter of its first draw */
    uint32_t consumed = 0u;
    int filled = 0;
#pragma unroll 1
    while (filled < T) {
        const uint32_t x = (RNG == 0) ? ((lj.da * s + lj.dc) & 0x7fffffffu) : philox_draw(r.key0, r.key1, s + lane);
        const uint32_t v = magic_div(x, p.mag_nops);
        const bool ok = v < (uint32_t)p.nops;
        const uint32_t bal = __ballot_sync(FULLMASK, ok);
        const int rank = filled + __popc(bal & lt);
        if (ok && rank < T) {
            int t = rank, idx = m;
#pragma unroll 1
            for (int d = 0;; ++d) {
                const int lo = m << d;
                const int cnt = min(lo + (1 << d) - 1, PL) - lo + 1;
                if (t < cnt) { idx = lo + t; break; }
                t -= cnt;
            }
            opn[idx - 1] = (uint8_t)p.opmap[v];
        }
        const int got = __popc(bal);
        if (filled + got >= T) {
            /* the lane that drew the subtree's last node */
            const uint32_t hit = __ballot_sync(FULLMASK, ok && rank == T - 1);
            const int last = __ffs(hit) - 1;
            consumed += (uint32_t)last + 1u;
            if (RNG == 0) s = __shfl_sync(FULLMASK, x, last);
            filled = T;
        } else {
            consumed += 32u;
            if (RNG == 0) s = (p.lcgA[5] * s + p.lcgC[5]) & 0x7fffffffu;   /* 2^5 = 32 draws */
            else s += 32u;
            filled += got;
        }
    }
    if (RNG == 0) r.s = s;
    else r.s += consumed;
    r.drawn += consumed;
}

/* Resident CTAs (of 8 warps) per SM the register allocation is sized for. */
#ifndef GPR_MIN_CTAS
#define GPR_MIN_CTAS 3
#endif

/* The SM clock, read by an asm statement with a memory clobber: the compiler
 * keeps it in program order with the shared-memory accesses around it.  The
 * hardware need not: a mark right after a __syncthreads() can be read before
 * the warp stalls on the barrier, and that wait then counts in the next phase. */
__device__ __forceinline__ long long ph_clock() {
    long long t;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t) :: "memory");
    return t;
}

/* Phase timing of the instrumented builds (PROF): lane 0 of each warp adds
 * the clock cycles since the last mark to the warp's counter `i`. */
#define GPR_PH(i)                                                                     \
    do {                                                                              \
        if constexpr (PROF) {                                                         \
            const long long t_ = ph_clock();                                          \
            if (lane == 0) s_ph[warp][(i)] += (unsigned long long)(t_ - ph_t);         \
            ph_t = t_;                                                                \
        }                                                                             \
    } while (0)
#define GPR_PH_COUNT(i, v)                                                            \
    do {                                                                              \
        if constexpr (PROF) {                                                         \
            if (lane == 0) s_ph[warp][(i)] += (unsigned long long)(v);                \
        }                                                                             \
    } while (0)

/* A chain's random stream at the start of a block (rx = random_seed + idx,
 * main.cu:691; Philox keyed by (seed, chain)). */
template <int RNG>
__device__ __forceinline__ Rng rng_start(uint32_t seed, int chain) {
    Rng r;
    r.key0 = seed; r.key1 = (uint32_t)chain; r.blk = 0xffffffffu; r.drawn = 0;
    r.w0 = r.w1 = r.w2 = r.w3 = 0u;
    r.s = (RNG == 0) ? ((seed + (uint32_t)chain) & 0x7fffffffu) : 0u;
    return r;
}

/* STREAM: the dataset is read from device memory (L2-resident for a few MB)
 * instead of being staged into each CTA's shared memory -- the layout for
 * datasets too large to stage.  BATCHED: many datasets (p.nds > 0), the view
 * switched per chain group; a compile-time switch, so that the single-dataset
 * kernel keeps its dataset view in constant memory rather than registers.
 * PROF: the phase-timed variant (gpr_mh_prof.cu only).
 *
 * Chains advance in one of three ways, by p.lockstep: 1, the CTA's warps step
 * together and share the evaluation of every proposal (CTA-balanced: two
 * barriers per step); k > 1, they realign every k steps; 0, they run freely. */
template <int K, bool ONEPASS, int RNG, bool ROLLED, bool STREAM, int NV, bool BATCHED, bool PROF = false>
__global__ void __launch_bounds__(256, GPR_MIN_CTAS) mh_block_kernel(const __grid_constant__ KParams p) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __shared__ unsigned long long s_ph[PROF ? 8 : 1][PROF ? GPR_PH_SLOTS : 1];
    long long ph_t = 0;
    if constexpr (PROF) {
        for (int i = threadIdx.x; i < 8 * GPR_PH_SLOTS; i += blockDim.x) (&s_ph[0][0])[i] = 0ull;
        __syncthreads();
        ph_t = ph_clock();
    }

    /* CTA-shared dataset (or the device arrays when streamed); with batched
     * data, the dataset of the current chain group (staged per group) */
    uint64_t* bar = (uint64_t*)smem;
    float* fx = (float*)(smem + GPR_STAGED_OFFSET);
    constexpr bool batched = BATCHED;
    DataView dv = data_view(p, fx, STREAM);
    int staged_ds = -1;
    bool bar_live = false;   /* the barrier has been initialised (batched restaging) */
    uint8_t* wbase = smem + GPR_STAGED_OFFSET;
    if (!STREAM) {
        wbase += align16((size_t)data_arrays(p) * p.nd_pad * 4);
        /* a copy that did not arrive in time: the error flag is set, the CTA leaves */
        if (!batched && !stage_dataset(fx, bar, p, dv)) return;
    }
    const size_t wbytes = warp_smem_bytes(p.PL, p.max_instr, p.levels, K);
    const WarpSmem ws = carve_warp<K>(wbase + (size_t)warp * wbytes, p.PL, p.max_instr, p.levels);

    LaneData<K> ld;
    if (ONEPASS) {
        ld.valid = 0u;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            int i = lane + 32 * k;
            bool v = i < dv.nd;
            ld.x[k] = v ? data_at<STREAM>(dv, DA_X1, i) : 0.0f;
            ld.valid |= (v ? 1u : 0u) << k;
        }
    }
    const int PL = p.PL;
    /* Each lane's LCG jump maps (the same in every warp), read around each
     * proposal instead of held in registers. */
    __shared__ LaneJump s_lj[32];
    if (warp == 0) s_lj[lane] = make_lane_jump(p, lane);
    __syncthreads();

    __shared__ int s_group_base;
    /* The block's counters (GPR_STAT_*), per warp in shared memory rather than
     * in registers (that measured 3-8% faster: the interpreter spills less),
     * added to p.stats once when the warp leaves. */
    __shared__ unsigned long long s_st[8][GPR_NSTATS];
    for (int i = lane; i < GPR_NSTATS; i += 32) s_st[warp][i] = 0ull;
    __syncwarp();
#define ST_ADD(i, v) do { if (lane == 0) s_st[warp][(i)] += (unsigned long long)(v); } while (0)
    const int nwarps = blockDim.x >> 5;
    /* CTA-balanced evaluation (lockstep == 1): each warp publishes its chain's
     * program; all warps then pull (chain, pass) tasks, longest programs
     * first, and leave the chunk sums of each pass here. */
    __shared__ const uint2* s_prog[8];    /* the published evaluation program */
    __shared__ int s_cost[8];             /* its estimated cost (-1: none)     */
    __shared__ int s_ninstr[8];           /* its length                       */
    __shared__ int s_count[8];
    __shared__ int s_bad[8];
    __shared__ int s_next;
    __shared__ float s_part[8][GPR_MAX_PASSES * (K / 4)];
    int npass = ONEPASS ? 1 : (dv.nd + 32 * K - 1) / (32 * K);
    int nch = chunk_count(dv.nd);
    bool balanced = p.lockstep == 1 && npass <= GPR_MAX_PASSES;
    float inv_npass = __frcp_rn((float)max(npass, 1));
    GPR_PH(GPR_PH_CLAIM);

#pragma unroll 1
    for (;;) {
        int chain = 0;
        if (p.lockstep) {
            /* CTA-wide chain groups: every warp of the CTA runs the same step at
             * the same time, so the warps share instruction-cache lines */
            __syncthreads();
            if (threadIdx.x == 0) {
                int b = atomicAdd(p.next_chain, nwarps);
                /* batched: claim groups in the host's order, largest datasets first */
                if (batched && b < p.N) b = p.ds_order[b / p.chains_per_ds] * p.chains_per_ds + b % p.chains_per_ds;
                s_group_base = b;
            }
            __syncthreads();
            const int base = s_group_base;
            if (base >= p.N) break;
            chain = base + warp;
            if constexpr (BATCHED) {
                const int d = chain_dataset(p, base);   /* a group never straddles datasets */
                if (d != staged_ds) {
                    dv = data_view(p, fx, STREAM, d);
                    /* a copy that did not arrive leaves the CTA (the error flag is set) */
                    if (!STREAM && !stage_dataset(fx, bar, p, dv, d, bar_live)) break;
                    bar_live = bar_live || dv.nd_pad > 0;
                    staged_ds = d;
                    npass = (dv.nd + 32 * K - 1) / (32 * K);
                    nch = chunk_count(dv.nd);
                    balanced = p.lockstep == 1 && npass <= GPR_MAX_PASSES;
                    inv_npass = __frcp_rn((float)max(npass, 1));
                }
            }
        } else {
            if (lane == 0) chain = atomicAdd(p.next_chain, 1);
            chain = __shfl_sync(FULLMASK, chain, 0);
            if (chain >= p.N) break;
        }
        const bool active = chain < p.N;
        GPR_PH(GPR_PH_CLAIM);

        /* load the chain (reference layout) into buffer 0 */
        if (active)
        for (int i = lane; i < PL; i += 32) {
            int o = p.P[(size_t)i * p.N + chain];
            ws.ops[0][i] = (uint8_t)((o >= 0 && o < OP_NALL) ? o : 255);
            ws.Cs[0][i] = p.C[(size_t)i * p.N + chain];
        }
        __syncwarp();

        int cur = 0;           /* ops/prog buffer of the current state */
        int ccur = 0;          /* constants buffer of the current state */
        float cur_len = 0.0f;
        int cur_count = 0;
        int cur_cost = 0;      /* program_cost of the current program */
        /* the current state's prior, likelihood sum S (scale 2^-e) and Cauchy
         * sum; the forward/backward terms (main.cu:702,723,761-775) */
        df cur_prior = df_make(0.f, 0.f), cur_S = df_make(0.f, 0.f), cur_cs = df_make(0.f, 0.f);
        df forward = df_make(0.f, 0.f), backward = df_make(0.f, 0.f);

        Rng r = rng_start<RNG>(p.seed, chain);
        /* random-walk scale: the configured one, or this chain's own (adapted) */
        float rw_sd = (p.chain_scale && active) ? p.chain_scale[chain] : p.rw_sd;
        float log_sd = logf(rw_sd);
        int n_cmoves = 0;


        /* step -1 evaluates the loaded state (main.cu:683-685); steps 0..steps-1
         * are the MH iterations (main.cu:697-808).  One call site each for
         * compile, prior and likelihood keeps the kernel's hot code small. */
        int cur_ninstr = 0;
        GPR_PH(GPR_PH_LOAD);
#pragma unroll 1
        for (int step = -1; step < p.steps; ++step) {
          if (!balanced && p.lockstep > 0 && (step + 1) % p.lockstep == 0) __syncthreads();
          GPR_PH(GPR_PH_STEPBAR);
          const bool init = step < 0;
          const bool structural = !init && p.struct_every > 0 && (step % p.struct_every == 0);
          int pbuf = cur, cbuf = ccur;
          float len = cur_len;
          int count = cur_count, ninstr = cur_ninstr, cost = cur_cost;
          df cs = cur_cs;
          if (active) {
            bool need_compile = init, need_cauchy = init;
            if (structural) {
                /* ---- structure move (main.cu:699-742) ---- */
                int cc = cur_count;
                if constexpr (PROF) {
                    /* and that the chain's node count is in range */
                    if ((unsigned)cc > (unsigned)PL) { if (lane == 0) atomicOr(p.err, 4); cc = 0; }
                }
                forward = df_make(-p.logcount[cc], 0.0f);
                const bool cur_invalid = !(isfinite(cur_prior.hi) && isfinite(cur_S.hi));
                structure_move<RNG>(r, ws.ops[cur], ws.ops[cur ^ 1], cur_invalid, p, s_lj[lane], lane);
                pbuf = cur ^ 1;
                need_compile = true;
                GPR_PH(GPR_PH_STRUCT);
            } else if (!init) {
                /* ---- constant move (main.cu:743-806) ---- */
                df fws, bws;
                constant_move<RNG>(r, ws, ws.Cs[ccur], ws.Cs[ccur ^ 1], fws, bws, p, s_lj[lane], lane, rw_sd);
                if (p.const_mode == 0) { forward = df_add(forward, fws); backward = df_add(backward, bws); }
                cbuf = ccur ^ 1;
                need_cauchy = true;
                GPR_PH(GPR_PH_CONST);
            }
            __syncwarp();
            if (need_compile) {
                const CompileOut co = compile_parallel<NV>(ws.ops[pbuf], PL, ws.prog[pbuf],
                                                       compile_scratch(ws.stk, PL), lane);
                len = co.length;
                count = co.count;
                ninstr = co.ninstr;
                __syncwarp();
                cost = program_cost(ws.prog[pbuf], ninstr, lane);
                GPR_PH(GPR_PH_COMPILE);
            }
            if (need_cauchy) { cs = cauchy_sum_u(ws.Cs[cbuf], p, lane); GPR_PH(GPR_PH_CAUCHY); }
            if (structural) backward = df_make(-p.logcount[count], 0.0f);
            build_eval_program(ws.prog[pbuf], ws.Cs[cbuf], ninstr, ws.eprog, lane);
            __syncwarp();
            GPR_PH(GPR_PH_EPROG);
          }
          df S = df_make(0.0f, 0.0f);
          int pts = 0;
          if (balanced) {
            if (lane == 0) {
                s_prog[warp] = ws.eprog;
                s_cost[warp] = active ? cost : -1;
                s_ninstr[warp] = ninstr;
                s_count[warp] = count;
                s_bad[warp] = 0;
            }
            if (threadIdx.x == 0) s_next = 0;
            __syncthreads();
            GPR_PH(GPR_PH_BAR1);
            /* rank of this lane's chain (lane < nwarps) by program length, longest first */
            int my_rank = 64, nact = 0;
            {
                const int cl = lane < nwarps ? s_cost[lane] : -1;
                int rk = 0;
                for (int j = 0; j < nwarps; ++j) {
                    const int cj = s_cost[j];
                    nact += cj >= 0;
                    rk += (cj > cl) || (cj == cl && j < lane);
                }
                if (cl >= 0) my_rank = rk;
            }
            const int ntasks = nact * npass;
            GPR_PH(GPR_PH_RANK);
#pragma unroll 1
            for (;;) {
                int t = 0;
                if (lane == 0) t = atomicAdd(&s_next, 1);
                t = __shfl_sync(FULLMASK, t, 0);
                if (t >= ntasks) break;
                /* task t: pass t mod npass of the chain of rank t / npass (exact for t < 2^16) */
                const int q = (int)__fmul_rz(__int2float_rn(t) + 0.5f, inv_npass), pass = t - q * npass;
                const int w = __ffs(__ballot_sync(FULLMASK, my_rank == q)) - 1;
                if constexpr (PROF) {
                    /* the instrumented build checks that the task has a chain */
                    if (w < 0) { if (lane == 0) atomicOr(p.err, 4); break; }
                }
                if (s_bad[w]) continue;
                float csum[K / 4];
                const bool anybad = eval_pass_chunks<K, ONEPASS, ROLLED, NV, STREAM>(s_prog[w], ws.stk, ws.scr, ld,
                                                                                   dv, p, lane, pass, csum);
                const int np = ONEPASS ? dv.nd : min(32 * K, dv.nd - pass * 32 * K);
                pts += np;
                if (lane == 0) {
#pragma unroll
                    for (int j = 0; j < K / 4; ++j) s_part[w][pass * (K / 4) + j] = csum[j];
                    if (anybad) s_bad[w] = 1;
                }
                ST_ADD(GPR_STAT_EVAL_NODE_POINTS, (unsigned long long)(s_count[w] + 4) * (unsigned)np);
                GPR_PH_COUNT(GPR_PH_NPASSES, 1);
                GPR_PH_COUNT(GPR_PH_NINSTR, s_ninstr[w]);
            }
            GPR_PH(GPR_PH_EVAL);
            __syncthreads();
            GPR_PH(GPR_PH_BAR2);
            if (active) {
                if (s_bad[warp]) {
                    S = lik_invalid();
                } else {
                    for (int c = 0; c < nch; ++c) S = df_add(S, df_make(s_part[warp][c], 0.0f));
                }
            }
            GPR_PH(GPR_PH_COMBINE);
          } else if (active) {
            S = eval_loglik_S<K, ONEPASS, ROLLED, NV, STREAM>(ws.eprog, ws.stk, ws.scr, ld, dv, p, lane, pts);
            ST_ADD(GPR_STAT_EVAL_NODE_POINTS, (unsigned long long)(count + 4) * (unsigned)pts);
            GPR_PH_COUNT(GPR_PH_NPASSES, npass);
            GPR_PH_COUNT(GPR_PH_NINSTR, (unsigned long long)ninstr * npass);
            GPR_PH(GPR_PH_EVAL);
          }
          ST_ADD(GPR_STAT_EVAL_POINTS, pts);
          if (active) {
            const df prior = prior_u(len, cs, p);
            ST_ADD(GPR_STAT_EVALS, 1); ST_ADD(GPR_STAT_EVAL_NODES, count);
            bool accept = true;
            if (!init) {
                float prob;
                accept = mh_accept_u<RNG>(prior, S, cur_prior, cur_S, backward, forward, r, p, &prob);
                if (!structural && p.adapt_target > 0.0f && p.const_mode == 1) {
                    log_sd = rm_update(log_sd, prob, p.adapt_target, n_cmoves++);
                    rw_sd = expf(log_sd);
                }
                if (structural) { ST_ADD(GPR_STAT_STRUCT_PROPOSED, 1); ST_ADD(GPR_STAT_STRUCT_ACCEPTED, accept); }
                else { ST_ADD(GPR_STAT_CONST_PROPOSED, 1); ST_ADD(GPR_STAT_CONST_ACCEPTED, accept); }
            }
            if (accept) {
                cur = pbuf; ccur = cbuf;
                cur_len = len; cur_count = count; cur_ninstr = ninstr; cur_cost = cost; cur_cs = cs;
                cur_prior = prior; cur_S = S;
            }
            __syncwarp();
            if (p.trace && !init && lane < p.trace_n && chain < p.trace_chains)
                p.trace[((size_t)chain * p.steps + step) * p.trace_n + lane] = ws.Cs[ccur][lane];
          }
          GPR_PH(GPR_PH_ACCEPT);
        }

        /* write back (main.cu:811-812 and the in-place P, C) */
        if (active)
        for (int i = lane; i < PL; i += 32) {
            uint8_t o = ws.ops[cur][i];
            if (o != 255) p.P[(size_t)i * p.N + chain] = (int32_t)o;
            p.C[(size_t)i * p.N + chain] = ws.Cs[ccur][i];
        }
        if (active && lane == 0) {
            p.prior[chain] = (double)cur_prior.hi + (double)cur_prior.lo;
            p.lik[chain] = lik_of(cur_S, dv, p);
            if (p.chain_scale && p.adapt_target > 0.0f && p.const_mode == 1) p.chain_scale[chain] = rw_sd;
        }
        __syncwarp();
        GPR_PH(GPR_PH_STORE);
    }
    if (lane == 0 && p.stats)
        for (int i = 0; i < GPR_NSTATS; ++i) atomicAdd(&p.stats[i], s_st[warp][i]);
#undef ST_ADD
    if constexpr (PROF) {
        if (lane == 0 && p.phase)
            for (int i = 0; i < GPR_PH_SLOTS; ++i) atomicAdd(&p.phase[i], s_ph[warp][i]);
    }
}

}  // namespace gpr

#endif /* GPR_MH_CUH */
