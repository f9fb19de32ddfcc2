/*
 * gpr_hmc.cuh -- reverse-mode adjoint of the program evaluator, and the MH
 * kernel whose constant moves are Hamiltonian (HMC; MALA with one leapfrog
 * step) instead of the reference's independence / random-walk proposals.
 *
 * Adjoint.  The compiled postfix program (gpr_common.h) is run forward once
 * per batch of K data points per lane with every instruction's result kept on
 * a tape in the thread's local memory (one 16-byte row per instruction for
 * K = 4; L1-resident for programs of realistic length, and leaving shared
 * memory to occupancy); the backward sweep then walks the instructions in reverse,
 * carrying d loglik / d acc, splitting it at each binary instruction into the
 * accumulator's and the operand's share, and adding the operand's share to
 * the constant it read (an instruction with a constant operand, or a constant
 * load, reads exactly one heap node's constant).  A popped operand's share is
 * parked on an adjoint stack and handed back at its PUSH.  The value a POP
 * reads is the tape entry of its matching PUSH, so the forward sweep needs no
 * value stack.  d loglik / d f at a point is 2 w (y - f) with w = 1/(2 sd^2)
 * (lnormalpdf, main.cu:299-301); sums run per lane in FP32 at the
 * bookkeeping scale 2^-64 and are reduced across lanes per constant.
 *
 * HMC move (no reference counterpart).  Momentum m ~ N(0, I) over all PL
 * constants; leapfrog with step eps, L steps, on the log-posterior
 * prior + likelihood (main.cu:529-544, 454-468), whose constant part is the
 * Cauchy(0, 1) prior (gradient -2c / (1 + c^2)); accepted with the
 * reference's rule (main.cu:728-740) with forward = -|m0|^2/2 and
 * backward = -|m1|^2/2.  Structure moves are the reference's, every
 * struct_every steps.
 */
#ifndef GPR_HMC_CUH
#define GPR_HMC_CUH

#include "gpr_mh.cuh"

namespace gpr {

#define GPR_HMC_K 4          /* points per lane of the adjoint and Hamiltonian kernels */
#define GPR_ASTK_MAX 8       /* adjoint-stack rows: value-stack depth for PROGRAM_LENGTH <= 255 */

/* One tape row: an instruction's result at this lane's K points. */
template <int K>
struct alignas(K == 4 ? 16 : (K == 2 ? 8 : 4)) Row {
    float v[K];
};

/* Per-warp shared memory of the gradient evaluator and the HMC kernel. */
struct GradSmem {
    uint8_t* ops[2];
    float* Cs[2];       /* [0], [1]: current and proposed constants            */
    gpr_word* prog[2];
    uint2* eprog;
    int16_t* match;     /* POP instruction -> index of its PUSH                 */
    float* gacc;        /* [PL]: the gradient sums (lane 0 adds each warp-summed
                         * share); also the compiler's scratch                   */
    float* gcur;        /* gradient of the log-posterior at the current state   */
    float* gnew;        /* ... at the trajectory's position                     */
    float* mom;         /* momentum                                             */
};

__host__ __device__ __forceinline__ size_t grad_rows_bytes(int PL) {
    const size_t gacc = (size_t)PL * 4;
    const size_t comp = 5 * align16((size_t)PL + 1) * 4;
    return align16(gacc > comp ? gacc : comp);
}

__host__ __device__ __forceinline__ size_t grad_warp_bytes(int PL, int max_instr) {
    const size_t plp = align16((size_t)PL);
    size_t b = 0;
    b += 2 * plp;                                              /* ops */
    b += align16(2 * plp * 4);                                 /* Cs */
    b += align16(2 * (size_t)max_instr * sizeof(gpr_word));    /* prog */
    b += align16((size_t)max_instr * 8);                       /* eprog */
    b += align16((size_t)max_instr * 2);                       /* match */
    b += grad_rows_bytes(PL);                                  /* gradient rows | compiler scratch */
    b += 3 * align16(plp * 4);                                 /* gcur, gnew, mom */
    return align16(b);
}

__device__ __forceinline__ GradSmem carve_grad(uint8_t* base, int PL, int max_instr) {
    GradSmem w;
    const size_t plp = align16((size_t)PL);
    uint8_t* p = base;
    w.ops[0] = p; w.ops[1] = p + plp; p += 2 * plp;
    w.Cs[0] = (float*)p; w.Cs[1] = (float*)p + plp; p += align16(2 * plp * 4);
    w.prog[0] = (gpr_word*)p; w.prog[1] = (gpr_word*)p + max_instr; p += align16(2 * (size_t)max_instr * sizeof(gpr_word));
    w.eprog = (uint2*)p; p += align16((size_t)max_instr * 8);
    w.match = (int16_t*)p; p += align16((size_t)max_instr * 2);
    w.gacc = (float*)p; p += grad_rows_bytes(PL);
    w.gcur = (float*)p; p += align16(plp * 4);
    w.gnew = (float*)p; p += align16(plp * 4);
    w.mom = (float*)p;
    return w;
}

/* For each POP instruction of the program, the index of the PUSH whose value
 * it pops (the stack discipline is a property of the program alone). */
__device__ __forceinline__ void pop_match(const gpr_word* prog, int ninstr, int16_t* match, int lane) {
    if (lane == 0) {
        int16_t st[32];
        int sp = 0;
#pragma unroll 1
        for (int i = 0; i < ninstr; ++i) {
            const uint32_t code = prog[i] & 0xffu;
            if (code == I_PUSH) {
                if (sp < 32) st[sp] = (int16_t)i;
                ++sp;
            } else if (code >= I_BIN0 && GPR_BIN_SRC(code) == SRC_POP) {
                --sp;
                match[i] = (sp >= 0 && sp < 32) ? st[sp] : (int16_t)0;
            }
        }
    }
    __syncwarp();
}

/* Value of an operand for instruction i: x, the constant, 1 or the popped
 * value (the tape entry of the matching PUSH). */
template <int K, int NV>
__device__ __forceinline__ void operand(uint32_t src, float c, int i, const int16_t* match,
                                        const float (&x)[NV][K], const Row<K>* tape, float (&v)[K]) {
    if (src == SRC_X) {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = x[0][k];
    } else if (NV > 1 && (src == SRC_X2 || src == SRC_X3)) {
        const int vi = NV > 1 ? (int)(src - SRC_X2) + 1 : 0;
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = x[vi][k];
    } else if (src == SRC_C) {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = c;
    } else if (src == SRC_ONE) {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = 1.0f;
    } else {
        const Row<K> t = tape[match[i]];
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = t.v[k];
    }
}

/* f(x) for this lane's K points, every instruction's result kept on the tape.
 * The arithmetic is the evaluator's (run_program), operation for operation. */
template <int K, int NV>
__device__ __forceinline__ void forward_tape(const uint2* __restrict__ prog, int ninstr, const int16_t* match,
                                             const float (&x)[NV][K], Row<K>* __restrict__ tape) {
    float acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0f;
#pragma unroll 1
    for (int i = 0; i < ninstr - 1; ++i) {
        const uint2 insw = prog[i];
        const uint32_t code = insw.x & 0xffu;
        const float c = __uint_as_float(insw.y);
        if (code >= I_BIN0) {
            const uint32_t bop = GPR_BIN_BOP(code);
            const uint32_t accleft = GPR_BIN_ACCLEFT(code);
            float v[K];
            operand<K, NV>(GPR_BIN_SRC(code), c, i, match, x, tape, v);
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float u = accleft ? acc[k] : v[k];
                const float w = accleft ? v[k] : acc[k];
                float r;
                if (bop == BOP_ADD) r = __fadd_rn(acc[k], v[k]);
                else if (bop == BOP_MUL) r = __fmul_rn(acc[k], v[k]);
                else if (bop == BOP_SUB) r = __fsub_rn(u, w);
                else if (bop == BOP_DIV) r = __fdiv_rn(u, w);
                else r = gx_pow(u, w);
                acc[k] = r;
            }
        } else {
            switch (code) {
                case I_LDX:
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = x[0][k];
                    break;
                case I_LDX2:
                case I_LDX3: {
                    const int vi = NV > 1 ? (code == I_LDX2 ? 1 : 2) : 0;
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = NV > 1 ? x[vi][k] : 0.0f;
                    break;
                }
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
                case I_PUSH: break;
                default:
#pragma unroll 1
                    for (int k = 0; k < K; ++k) {
                        const float a = acc[k];
                        float r;
                        switch (code) {
                            case U_INV: r = __fdiv_rn(1.0f, a); break;
                            case U_LOG: r = gx_log(a); break;
                            case U_EXP: r = gx_exp(a); break;
                            case U_SQRT: r = __fsqrt_rn(a); break;
                            case U_SIN: r = sinf(a); break;
                            case U_ASIN: r = asinf(a); break;
                            case U_COS: r = cosf(a); break;
                            case U_ACOS: r = acosf(a); break;
                            case U_TAN: r = tanf(a); break;
                            case U_ATAN: r = atanf(a); break;
                            default: r = fabsf(a); break;
                        }
                        acc[k] = r;
                    }
                    break;
            }
        }
        Row<K> row;
#pragma unroll
        for (int k = 0; k < K; ++k) row.v[k] = acc[k];
        tape[i] = row;
    }
}

/* adj * d, where a zero adjoint contributes zero even through a partial that
 * left the FP32 range (0 * inf would poison the sums). */
__device__ __forceinline__ float adj_mul(float adj, float d) { return adj == 0.0f ? 0.0f : __fmul_rn(adj, d); }

/* The backward sweep: adj holds d loglik / d f per point on entry; the
 * per-constant shares are added to this lane's gradient rows. */
template <int K, int NV>
__device__ __forceinline__ void backward_tape(const uint2* __restrict__ prog, int ninstr, const int16_t* match,
                                              const float (&x)[NV][K], const Row<K>* __restrict__ tape,
                                              float (&adj)[K], Row<K>* __restrict__ astk, float* __restrict__ gacc,
                                              int PL, int lane) {
    int sp = 0;
#pragma unroll 1
    for (int i = ninstr - 2; i >= 0; --i) {
        const uint2 insw = prog[i];
        const uint32_t code = insw.x & 0xffu;
        const uint32_t node = (insw.x >> 8) & 0xffu;
        const float c = __uint_as_float(insw.y);
        if (code >= I_BIN0) {
            const uint32_t bop = GPR_BIN_BOP(code);
            const uint32_t accleft = GPR_BIN_ACCLEFT(code);
            const uint32_t src = GPR_BIN_SRC(code);
            float v[K];
            operand<K, NV>(src, c, i, match, x, tape, v);
            float share = 0.0f;
            /* the accumulator's input; the result only where a partial needs it */
            const Row<K> ain = tape[i - 1];
            Row<K> rres;
            if (bop == BOP_DIV || bop == BOP_POW) rres = tape[i];
            Row<K> spill;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float a = ain.v[k];
                const float res = (bop == BOP_DIV || bop == BOP_POW) ? rres.v[k] : 0.0f;
                const float u = accleft ? a : v[k];
                const float w = accleft ? v[k] : a;
                float du, dw;
                if (bop == BOP_ADD) { du = 1.0f; dw = 1.0f; }
                else if (bop == BOP_SUB) { du = 1.0f; dw = -1.0f; }
                else if (bop == BOP_MUL) { du = w; dw = u; }
                else if (bop == BOP_DIV) { du = __fdiv_rn(1.0f, w); dw = -__fdiv_rn(res, w); }
                else {
                    du = __fmul_rn(w, gx_pow(u, __fsub_rn(w, 1.0f)));
                    dw = res == 0.0f ? 0.0f : __fmul_rn(res, gx_log(u));
                }
                const float au = adj_mul(adj[k], du), aw = adj_mul(adj[k], dw);
                const float av = accleft ? aw : au;
                adj[k] = accleft ? au : aw;
                spill.v[k] = av;
                share = __fadd_rn(share, av);
            }
            if (src == SRC_POP) astk[sp++] = spill;
            else if (src == SRC_C && (int)node < PL) {
                const float tot = warp_sum(share);
                if (lane == 0) gacc[node] += tot;
            }
        } else if (code == I_LDC) {
            float share = 0.0f;
#pragma unroll
            for (int k = 0; k < K; ++k) { share = __fadd_rn(share, adj[k]); adj[k] = 0.0f; }
            if ((int)node < PL) {
                const float tot = warp_sum(share);
                if (lane == 0) gacc[node] += tot;
            }
        } else if (code == I_LDX || code == I_LD1 || code == I_LDNAN || code == I_LDX2 || code == I_LDX3) {
#pragma unroll
            for (int k = 0; k < K; ++k) adj[k] = 0.0f;
        } else if (code == I_PUSH) {
            const Row<K> t = astk[--sp];
#pragma unroll
            for (int k = 0; k < K; ++k) adj[k] = t.v[k];
        } else {
            const Row<K> ain = tape[i - 1], rres = tape[i];
#pragma unroll 1
            for (int k = 0; k < K; ++k) {
                const float a = ain.v[k];
                const float res = rres.v[k];
                float d;
                switch (code) {
                    case U_INV: d = -__fmul_rn(res, res); break;
                    case U_LOG: d = __fdiv_rn(1.0f, a); break;
                    case U_EXP: d = res; break;
                    case U_SQRT: d = __fdiv_rn(0.5f, res); break;
                    case U_SIN: d = cosf(a); break;
                    case U_ASIN: d = __fdiv_rn(1.0f, __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(a, a)))); break;
                    case U_COS: d = -sinf(a); break;
                    case U_ACOS: d = -__fdiv_rn(1.0f, __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(a, a)))); break;
                    case U_TAN: d = __fadd_rn(1.0f, __fmul_rn(res, res)); break;
                    case U_ATAN: d = __fdiv_rn(1.0f, __fadd_rn(1.0f, __fmul_rn(a, a))); break;
                    default: d = a > 0.0f ? 1.0f : (a < 0.0f ? -1.0f : 0.0f); break;
                }
                adj[k] = adj_mul(adj[k], d);
            }
        }
    }
}

/* Log-likelihood of one program (double-float at scale 2^-64, -inf when any
 * point is invalid, as eval_loglik) and its gradient over all PL constants:
 * g[i] = 2^-64 d loglik / d C[i] in FP32, at the bookkeeping scale like the
 * likelihood (0 for constants the program does not read).  The gradient is
 * meaningful only when the likelihood is finite. */
template <int K, int MAXI, int NV, bool STREAM>
__device__ df eval_loglik_grad(const uint2* prog, int ninstr, const GradSmem& ws, const DataView& dv,
                               const KParams& p, int lane, int& pts, float* g) {
    const int PL = p.PL;
    Row<K> tape[MAXI];             /* thread-local: results of every instruction */
    Row<K> astk[GPR_ASTK_MAX];     /* adjoints of pushed values                  */
#pragma unroll 1
    for (int j = lane; j < PL; j += 32) ws.gacc[j] = 0.0f;
    __syncwarp();
    float s = 0.0f;
    bool bad = false;
    const int npass = (dv.nd + 32 * K - 1) / (32 * K);
#pragma unroll 1
    for (int pass = 0; pass < npass && !bad; ++pass) {
        float x[NV][K], adj[K];
        const int base = pass * 32 * K + lane;
        const uint32_t valid = load_points<K, NV, STREAM>(dv, p, base, x);
        forward_tape<K, NV>(prog, ninstr, ws.match, x, tape);
        pts += min(32 * K, dv.nd - pass * 32 * K);
        const Row<K> fres = tape[ninstr - 2];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            adj[k] = 0.0f;
            if (valid & (1u << k)) {
                const int i = base + 32 * k;
                const float f = fres.v[k];
                /* the 2^-64-scaled weight: dw carries 2^-e; the factor 2^(e-64) is exact */
                const float wi = __fmul_rn(data_at<STREAM>(dv, DA_W, i), p.w_to_df);
                const float r = __fsub_rn(f, data_at<STREAM>(dv, DA_Y, i));
                const float q = __fmul_rn(r, r);
                bad |= !(q <= FLT_MAX);
                s = fmaf(q, wi, s);
                adj[k] = __fmul_rn(__fmul_rn(-2.0f, wi), r);
            }
        }
        bad = __any_sync(FULLMASK, bad);
        if (!bad) backward_tape<K, NV>(prog, ninstr, ws.match, x, tape, adj, astk, ws.gacc, PL, lane);
    }
    __syncwarp();
#pragma unroll 1
    for (int c = lane; c < PL; c += 32) g[c] = ws.gacc[c];
    __syncwarp();
    if (bad) return df_make(-INFINITY, 0.0f);
    df S = warp_sum_df(df_make(s, 0.0f));
    if (!isfinite(S.hi)) return df_make(-INFINITY, 0.0f);
    return df_sub(df_neg(S), df_make(dv.ns_hi, dv.ns_lo));
}

/* d/dc of lcauchypdf(c, 1) (main.cu:303-305). */
__device__ __forceinline__ float dcauchy(float c) {
    return __fdiv_rn(__fmul_rn(-2.0f, c), __fadd_rn(1.0f, __fmul_rn(c, c)));
}

/* Standard normal momentum for constant i at MH step t of a chain: Philox
 * keyed by (seed ^ 0x484d43, chain), counter (t, i), Box-Muller on two
 * 24-bit uniforms with the project's exactly reproducible log and sin
 * (gpr_rngmath.h), so a host restatement draws the same values. */
__device__ __forceinline__ float hmc_momentum(uint32_t seed, uint32_t chain, uint32_t t, uint32_t i) {
    uint32_t c[4] = {t, i, 0x4d4f4du, 0u};
    gpr_philox4x32_10(c, seed ^ 0x484d43u, chain);
    const float u1 = __fmul_rn((float)((c[0] >> 8) + 1u), 5.9604644775390625e-08f);   /* (0, 1] */
    const float u2 = __fmul_rn((float)(c[1] >> 8), 5.9604644775390625e-08f);          /* [0, 1) */
    const float a = __fsqrt_rn(__fmul_rn(-2.0f, gpr_rng_logf(u1)));
    return __fmul_rn(a, gpr_rng_sinf(gpr_rng_twopi_times(u2)));
}

/* Two uniforms in [0, 1) for move t of a chain's trajectory jitter, from the
 * momentum's Philox stream at a counter the momenta never use. */
__device__ __forceinline__ void hmc_jitter_uniforms(uint32_t seed, uint32_t chain, uint32_t t, float& u1, float& u2) {
    uint32_t c[4] = {t, 0xffffffffu, 0x4a4954u, 0u};
    gpr_philox4x32_10(c, seed ^ 0x484d43u, chain);
    u1 = __fmul_rn((float)(c[0] >> 8), 5.9604644775390625e-08f);
    u2 = __fmul_rn((float)(c[1] >> 8), 5.9604644775390625e-08f);
}

/* ------------------------------------------------------------------------ */
/* d loglik / d C for every chain's current state (gpr_loglik_grad): one warp
 * per chain, grad[i*N + chain] (double, unscaled) and lik[chain]. */
/* The dataset: staged into this CTA's shared memory, or (STREAM) read from
 * device memory.  Returns where the per-warp regions start, or nullptr (the
 * same in every thread) when the staging copy timed out. */
template <bool STREAM>
__device__ __forceinline__ uint8_t* grad_dataset(uint8_t* smem, const KParams& p, DataView& dv) {
    float* fx = (float*)(smem + GPR_STAGED_OFFSET);
    dv = data_view(p, fx, STREAM);
    if (STREAM) return smem + GPR_STAGED_OFFSET;
    if (!stage_dataset(fx, (uint64_t*)smem, p, dv)) return nullptr;
    return smem + GPR_STAGED_OFFSET + align16((size_t)data_arrays(p) * p.nd_pad * 4);
}

template <int K, int MAXI, bool STREAM, int NV>
__global__ void __launch_bounds__(128) loglik_grad_kernel(const __grid_constant__ KParams p, double* grad,
                                                          double* lik_out) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    DataView dv;
    uint8_t* wbase = grad_dataset<STREAM>(smem, p, dv);
    if (!wbase) return;   /* the staging copy timed out: the error flag is set */
    const GradSmem ws = carve_grad(wbase + (size_t)warp * grad_warp_bytes(p.PL, p.max_instr), p.PL, p.max_instr);
    const int chain = blockIdx.x * (blockDim.x >> 5) + warp;
    if (chain >= p.N) return;
    if (STREAM && p.nds > 0) dv = data_view(p, nullptr, true, chain_dataset(p, chain));   /* batched: streamed */
    const int PL = p.PL;
    for (int i = lane; i < PL; i += 32) {
        const int o = p.P[(size_t)i * p.N + chain];
        ws.ops[0][i] = (uint8_t)((o >= 0 && o < OP_NALL) ? o : 255);
        ws.Cs[0][i] = p.C[(size_t)i * p.N + chain];
    }
    __syncwarp();
    const CompileOut co = compile_parallel<NV>(ws.ops[0], PL, ws.prog[0], compile_scratch(ws.gacc, PL), lane);
    __syncwarp();
    build_eval_program(ws.prog[0], ws.Cs[0], co.ninstr, ws.eprog, lane);
    pop_match(ws.prog[0], co.ninstr, ws.match, lane);
    int pts = 0;
    const df lik = eval_loglik_grad<K, MAXI, NV, STREAM>(ws.eprog, co.ninstr, ws, dv, p, lane, pts, ws.gnew);
    for (int i = lane; i < PL; i += 32) grad[(size_t)i * p.N + chain] = (double)ws.gnew[i] * GPR_DF_UNSCALE;
    if (lane == 0) lik_out[chain] = df_to_double_unscaled(lik);
}

/* ------------------------------------------------------------------------ */
/* The MH block with Hamiltonian constant moves.  One warp per chain, chains
 * claimed from the global counter; evaluation with the adjoint on K points
 * per lane. */
template <int K, int MAXI, int RNG, bool STREAM, int NV>
__global__ void __launch_bounds__(256) mh_hmc_kernel(const __grid_constant__ KParams p) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    DataView dv;
    uint8_t* wbase = grad_dataset<STREAM>(smem, p, dv);
    if (!wbase) return;   /* the staging copy timed out: the error flag is set */
    const GradSmem ws = carve_grad(wbase + (size_t)warp * grad_warp_bytes(p.PL, p.max_instr), p.PL, p.max_instr);
    const int PL = p.PL;
    const bool adapt = p.chain_scale && p.adapt_target > 0.0f;
    const uint32_t seed = p.seed;
    const float unscale = (float)GPR_DF_UNSCALE;
    const LaneJump ljump = make_lane_jump(p, lane);

#pragma unroll 1
    for (;;) {
        int chain = 0;
        if (lane == 0) chain = atomicAdd(p.next_chain, 1);
        chain = __shfl_sync(FULLMASK, chain, 0);
        if (chain >= p.N) break;
        if (STREAM && p.nds > 0) dv = data_view(p, nullptr, true, chain_dataset(p, chain));   /* batched: streamed */

        for (int i = lane; i < PL; i += 32) {
            const int o = p.P[(size_t)i * p.N + chain];
            ws.ops[0][i] = (uint8_t)((o >= 0 && o < OP_NALL) ? o : 255);
            ws.Cs[0][i] = p.C[(size_t)i * p.N + chain];
        }
        __syncwarp();

        Rng r;
        r.key0 = seed; r.key1 = (uint32_t)chain; r.blk = 0xffffffffu; r.drawn = 0;
        r.w0 = r.w1 = r.w2 = r.w3 = 0u;
        r.s = (RNG == 0) ? ((seed + (uint32_t)chain) & 0x7fffffffu) : 0u;

        /* leapfrog step: the configured one or this chain's own; with
         * adaptation, dual averaging of log(step) toward the target acceptance
         * (Hoffman and Gelman, JMLR 2014, section 3.2: gamma 0.05, t0 10,
         * kappa 0.75, mu = log(10 step0)) */
        const float eps0 = p.chain_scale ? p.chain_scale[chain] : p.hmc_eps;
        float log_eps = logf(eps0), log_eps_bar = log_eps, hbar = 0.0f;
        const float mu = logf(__fmul_rn(10.0f, eps0));
        int n_adapt = 0;

        int cur = 0, ccur = 0, cur_count = 0, cur_ninstr = 0;
        float cur_len = 0.0f;
        df cur_prior = df_make(0.f, 0.f), cur_lik = df_make(0.f, 0.f), cur_post = df_make(0.f, 0.f);
        df cur_cs = df_make(0.f, 0.f);
        unsigned long long st_nodes = 0, st_np = 0, st_pts = 0;
        int st_evals = 0, st_sp = 0, st_sa = 0, st_cp = 0, st_ca = 0;

#pragma unroll 1
        for (int step = -1; step < p.steps; ++step) {
            const bool init = step < 0;
            const bool structural = init || (p.struct_every > 0 && step % p.struct_every == 0);
            if (structural) {
                /* the reference's structure move (or the initial evaluation) */
                int pbuf = cur;
                df forward = df_make(0.f, 0.f);
                if (!init) {
                    forward = df_make(__fmul_rn(-p.logcount[cur_count], GPR_DF_SCALE), 0.0f);
                    structure_move<RNG>(r, ws.ops[cur], ws.ops[cur ^ 1], df_invalid(cur_post), p, ljump, lane);
                    pbuf = cur ^ 1;
                }
                __syncwarp();
                const CompileOut co = compile_parallel<NV>(ws.ops[pbuf], PL, ws.prog[pbuf],
                                                       compile_scratch(ws.gacc, PL), lane);
                __syncwarp();
                const df backward = df_make(__fmul_rn(-p.logcount[co.count], GPR_DF_SCALE), 0.0f);
                const df cs = init ? cauchy_sum(ws.Cs[ccur], p, lane) : cur_cs;
                build_eval_program(ws.prog[pbuf], ws.Cs[ccur], co.ninstr, ws.eprog, lane);
                pop_match(ws.prog[pbuf], co.ninstr, ws.match, lane);
                int pe = 0;
                const df lik = eval_loglik_grad<K, MAXI, NV, STREAM>(ws.eprog, co.ninstr, ws, dv, p, lane, pe, ws.gnew);
                st_pts += (unsigned)pe;
                const df prior = df_add(length_prior(co.length, p), cs);
                const df post = df_add(prior, lik);
                st_evals++; st_nodes += (unsigned)co.count; st_np += (unsigned long long)(co.count + 4) * pe;
                bool accept = true;
                if (!init) {
                    accept = mh_accept<RNG>(post, cur_post, backward, forward, r, p);
                    st_sp++; st_sa += accept;
                }
                if (accept) {
                    cur = pbuf; cur_len = co.length; cur_count = co.count; cur_ninstr = co.ninstr; cur_cs = cs;
                    cur_prior = prior; cur_lik = lik; cur_post = post;
                    for (int i = lane; i < PL; i += 32)
                        ws.gcur[i] = __fadd_rn(__fmul_rn(ws.gnew[i], unscale), dcauchy(ws.Cs[ccur][i]));
                }
                __syncwarp();
            } else {
                /* ---- Hamiltonian constant move ---- */
                st_cp++;
                if (!df_invalid(cur_post)) {
                    float eps = expf(log_eps);
                    int nleap = p.hmc_L;
                    if (p.hmc_jit_eps > 0.0f || p.hmc_jit_len > 0.0f) {
                        /* this move's trajectory: jittered step and leapfrog count */
                        float ue, ul;
                        hmc_jitter_uniforms(seed, (uint32_t)chain, (uint32_t)step, ue, ul);
                        eps = __fmul_rn(eps, __fadd_rn(1.0f, __fmul_rn(p.hmc_jit_eps, __fsub_rn(__fmul_rn(2.0f, ue), 1.0f))));
                        if (p.hmc_jit_len > 0.0f) {
                            const float L = (float)p.hmc_L;
                            const int lo = max(1, __float2int_rn(__fmul_rn(L, __fsub_rn(1.0f, p.hmc_jit_len))));
                            const int hi = max(lo, __float2int_rn(__fmul_rn(L, __fadd_rn(1.0f, p.hmc_jit_len))));
                            nleap = lo + min((int)__fmul_rn(ul, (float)(hi - lo + 1)), hi - lo);
                        }
                    }
                    const float heps = __fmul_rn(0.5f, eps);
                    /* the last structure step may have left match[] for a
                     * rejected proposal: rebuild it for the current program */
                    pop_match(ws.prog[cur], cur_ninstr, ws.match, lane);
                    const float* q0 = ws.Cs[ccur];
                    float* q = ws.Cs[ccur ^ 1];
                    float k0 = 0.0f;
                    for (int i = lane; i < PL; i += 32) {
                        const float m = hmc_momentum(seed, (uint32_t)chain, (uint32_t)step, (uint32_t)i);
                        k0 = fmaf(m, m, k0);
                        ws.mom[i] = __fadd_rn(m, __fmul_rn(heps, ws.gcur[i]));
                        q[i] = q0[i];
                    }
                    k0 = __fmul_rn(0.5f, warp_sum(k0));
                    df lik = df_make(-INFINITY, 0.0f);
                    bool ok = true;
#pragma unroll 1
                    for (int l = 1; l <= nleap && ok; ++l) {
                        bool fin = true;
                        for (int i = lane; i < PL; i += 32) {
                            q[i] = __fadd_rn(q[i], __fmul_rn(eps, ws.mom[i]));
                            fin &= isfinite(q[i]);
                        }
                        ok = __all_sync(FULLMASK, fin);
                        __syncwarp();
                        if (!ok) break;
                        build_eval_program(ws.prog[cur], q, cur_ninstr, ws.eprog, lane);
                        __syncwarp();
                        int pe = 0;
                        lik = eval_loglik_grad<K, MAXI, NV, STREAM>(ws.eprog, cur_ninstr, ws, dv, p, lane, pe, ws.gnew);
                        st_pts += (unsigned)pe;
                        st_evals++; st_nodes += (unsigned)cur_count;
                        st_np += (unsigned long long)(cur_count + 4) * (unsigned)pe;
                        if (df_invalid(lik)) { ok = false; break; }
                        const float f = l < nleap ? eps : heps;
                        for (int i = lane; i < PL; i += 32) {
                            const float gt = __fadd_rn(__fmul_rn(ws.gnew[i], unscale), dcauchy(q[i]));
                            ws.gnew[i] = gt;
                            ws.mom[i] = __fadd_rn(ws.mom[i], __fmul_rn(f, gt));
                        }
                        __syncwarp();
                    }
                    bool accept = false;
                    float alpha = 0.0f;
                    if (ok) {
                        float k1 = 0.0f;
                        for (int i = lane; i < PL; i += 32) k1 = fmaf(ws.mom[i], ws.mom[i], k1);
                        k1 = __fmul_rn(0.5f, warp_sum(k1));
                        const df cs = cauchy_sum(q, p, lane);
                        const df prior = df_add(length_prior(cur_len, p), cs);
                        const df post = df_add(prior, lik);
                        const df forward = df_make(__fmul_rn(-k0, GPR_DF_SCALE), 0.0f);
                        const df backward = df_make(__fmul_rn(-k1, GPR_DF_SCALE), 0.0f);
                        if (isfinite(k1)) alpha = accept_prob(post, cur_post, backward, forward);
                        accept = isfinite(k1) && mh_accept<RNG>(post, cur_post, backward, forward, r, p);
                        if (accept) {
                            ccur ^= 1;
                            cur_cs = cs; cur_prior = prior; cur_lik = lik; cur_post = post;
                            for (int i = lane; i < PL; i += 32) ws.gcur[i] = ws.gnew[i];
                        }
                    }
                    st_ca += accept;
                    if (adapt) {
                        ++n_adapt;
                        const float t = (float)(n_adapt + 10);
                        hbar = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, __fdiv_rn(1.0f, t)), hbar),
                                         __fdiv_rn(__fsub_rn(p.adapt_target, alpha), t));
                        log_eps = fminf(fmaxf(__fsub_rn(mu, __fmul_rn(sqrtf((float)n_adapt) * 20.0f, hbar)),
                                              -30.0f), 5.0f);
                        const float w = __powf((float)n_adapt, -0.75f);
                        log_eps_bar = __fadd_rn(__fmul_rn(w, log_eps), __fmul_rn(__fsub_rn(1.0f, w), log_eps_bar));
                    }
                    __syncwarp();
                }
            }
            if (p.trace && !init && lane < p.trace_n && chain < p.trace_chains)
                p.trace[((size_t)chain * p.steps + step) * p.trace_n + lane] = ws.Cs[ccur][lane];
        }

        for (int i = lane; i < PL; i += 32) {
            const uint8_t o = ws.ops[cur][i];
            if (o != 255) p.P[(size_t)i * p.N + chain] = (int32_t)o;
            p.C[(size_t)i * p.N + chain] = ws.Cs[ccur][i];
        }
        if (lane == 0) {
            p.prior[chain] = df_to_double_unscaled(cur_prior);
            p.lik[chain] = df_to_double_unscaled(cur_lik);
            if (adapt && n_adapt > 0) p.chain_scale[chain] = expf(log_eps_bar);
            if (p.stats) {
                atomicAdd(&p.stats[GPR_STAT_EVALS], (unsigned long long)st_evals);
                atomicAdd(&p.stats[GPR_STAT_EVAL_NODES], st_nodes);
                atomicAdd(&p.stats[GPR_STAT_EVAL_POINTS], st_pts);
                atomicAdd(&p.stats[GPR_STAT_EVAL_NODE_POINTS], st_np);
                atomicAdd(&p.stats[GPR_STAT_STRUCT_PROPOSED], (unsigned long long)st_sp);
                atomicAdd(&p.stats[GPR_STAT_STRUCT_ACCEPTED], (unsigned long long)st_sa);
                atomicAdd(&p.stats[GPR_STAT_CONST_PROPOSED], (unsigned long long)st_cp);
                atomicAdd(&p.stats[GPR_STAT_CONST_ACCEPTED], (unsigned long long)st_ca);
            }
        }
        __syncwarp();
    }
}

/* The kernels for three input variables (gpr_hmc_v.cu). */
const void* grad_kernel_v3(int maxi, int stream);
const void* hmc_kernel_v3(const KParams& p, int stream);

}  // namespace gpr

#endif /* GPR_HMC_CUH */
