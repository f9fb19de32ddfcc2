/*
 * gpr_pipe.cuh -- the pipelined MH block kernel: two chains per warp, one
 * CTA barrier per half-step.
 *
 * The chains of a CTA form two groups of one chain per warp.  In half-step h
 * the group g = h mod 2 takes its turn -- each warp applies the accept rule
 * to its group-g chain's proposal, scored in the previous half-step, then
 * draws and compiles the next proposal and publishes its program -- while
 * every warp, once its own turn is done, pulls evaluation tasks (a chain of
 * the other group and a range of its passes) from the CTA's shared pool,
 * longest programs first.  A barrier closes the half-step.  A warp whose
 * turn was short therefore evaluates more; the CTA waits once per half-step
 * for the last task instead of twice per step (after the proposals and after
 * the evaluation), and a chain's passes are spread over all warps, however
 * many there are.
 *
 * Every chain takes exactly the steps of MH_simple_kernel (main.cu:679-813)
 * in its own order, with the proposal, prior, likelihood and accept rule of
 * gpr_mh.cuh; only the schedule differs, so each chain's trajectory is the
 * one mh_block_kernel gives it, bit for bit.
 */
#ifndef GPR_PIPE_CUH
#define GPR_PIPE_CUH

#include "gpr_mh.cuh"

namespace gpr {

/* Chunk sums per chain kept on the CTA's shared-memory board; datasets with
 * more chunks keep them in p.part. */
#define GPR_PIPE_CHUNKS 64
/* Most tasks one chain's evaluation is split into. */
#define GPR_PIPE_TASKS 32

/* A chain's state between its warp's turns (shared memory; a turn reads the
 * fields into registers and lane 0 writes them back). */
struct PipeSlot {
    df cur_prior, cur_S, cur_cs;  /* the current state: prior, likelihood sum (scale 2^-e), Cauchy sum */
    df prior, cs;                 /* the proposal in flight: prior, Cauchy sum                           */
    df fw, bw;                    /* forward/backward terms (main.cu:702,723,761-775)                    */
    int chain;                    /* >= p.N: no chain in this slot                                       */
    int cur, ccur, pbuf, cbuf;    /* ops/program and constants buffers: current, proposal                */
    int ninstr, count, cur_ninstr, cur_count;
    float len, cur_len;
    uint32_t rs, rblk, rw0, rw1, rw2, rw3;   /* the chain's random stream                           */
    float rw_sd, log_sd;          /* random-walk scale and its adaptation state                         */
    int n_cmoves;
    int structural;               /* the proposal in flight is a structure move                          */
};

/* Per-warp dynamic shared memory: per slot the op, constant and program
 * buffers (current and proposal), then one region shared by the slots' turns
 * and the warp's evaluation tasks (value stack and transcendental scratch |
 * constant-move records | compiler scratch). */
__host__ __device__ __forceinline__ size_t pipe_slot_bytes(int PL, int max_instr) {
    const size_t plp = align16((size_t)PL);
    return 2 * plp + align16(2 * plp * 4) + align16(2 * (size_t)max_instr * sizeof(gpr_word));
}
__host__ __device__ __forceinline__ size_t pipe_warp_bytes(int PL, int max_instr, int levels, int K) {
    return 2 * pipe_slot_bytes(PL, max_instr) + shared_region_bytes(PL, levels, K);
}

/* The CTA's chunk-sum board, [2 groups][8 warps][GPR_PIPE_CHUNKS] floats, in
 * dynamic shared memory after the warps' regions.  It exists only when every
 * chain's chunks fit on it; larger datasets keep their chunk sums in p.part
 * (p.part_stride > 0) and leave that shared memory to more resident CTAs. */
__host__ __device__ __forceinline__ size_t pipe_board_bytes() { return (size_t)2 * 8 * GPR_PIPE_CHUNKS * 4; }

/* The WarpSmem view of slot g of a warp's region (no evaluation program:
 * the pipelined kernel interprets program and constants in place). */
template <int K>
__device__ __forceinline__ WarpSmem carve_pipe(uint8_t* base, int PL, int max_instr, int levels, int g) {
    WarpSmem w;
    const size_t plp = align16((size_t)PL);
    uint8_t* p = base + (size_t)g * pipe_slot_bytes(PL, max_instr);
    w.ops[0] = p; w.ops[1] = p + plp; p += 2 * plp;
    w.Cs[0] = (float*)p; w.Cs[1] = (float*)p + plp; p += align16(2 * plp * 4);
    w.prog[0] = (gpr_word*)p; w.prog[1] = (gpr_word*)p + max_instr;
    w.eprog = nullptr;
    uint8_t* r = base + 2 * pipe_slot_bytes(PL, max_instr);
    w.stk = (float*)r;
    w.scr = w.stk + (size_t)levels * K * 32;
    w.off = (int*)r;
    w.ndr = w.off + plp;
    w.fw = (float*)(w.ndr + plp);
    w.bw = w.fw + plp;
    return w;
}

template <int K, bool ONEPASS, int RNG, bool ROLLED, bool STREAM, int NV, bool BATCHED, bool PROF = false>
__global__ void __launch_bounds__(256, GPR_MIN_CTAS) mh_pipe_kernel(const __grid_constant__ KParams p) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    __shared__ unsigned long long s_ph[PROF ? 8 : 1][PROF ? GPR_PH_SLOTS : 1];
    long long ph_t = 0;
    if constexpr (PROF) {
        for (int i = threadIdx.x; i < 8 * GPR_PH_SLOTS; i += blockDim.x) (&s_ph[0][0])[i] = 0ull;
        __syncthreads();
        ph_t = ph_clock();
    }

    uint64_t* bar = (uint64_t*)smem;
    float* fx = (float*)(smem + GPR_STAGED_OFFSET);
    DataView dv = data_view(p, fx, STREAM);
    int staged_ds = -1;
    bool bar_live = false;
    uint8_t* wbase = smem + GPR_STAGED_OFFSET;
    if (!STREAM) {
        wbase += align16((size_t)data_arrays(p) * p.nd_pad * 4);
        if (!BATCHED && !stage_dataset(fx, bar, p, dv)) return;   /* timed out: flag set, the CTA leaves */
    }
    const int PL = p.PL;
    uint8_t* const mybase = wbase + (size_t)warp * pipe_warp_bytes(PL, p.max_instr, p.levels, K);
    /* the warp's value stack and transcendental scratch for its evaluation tasks */
    float* const my_stk = (float*)(mybase + 2 * pipe_slot_bytes(PL, p.max_instr));
    float* const my_scr = my_stk + (size_t)p.levels * K * 32;

    LaneData<K> ld;
    if (ONEPASS) {
        ld.valid = 0u;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int i = lane + 32 * k;
            const bool v = i < dv.nd;
            ld.x[k] = v ? data_at<STREAM>(dv, DA_X1, i) : 0.0f;
            ld.valid |= (v ? 1u : 0u) << k;
        }
    }
    /* Each lane's LCG jump maps (the same in every warp), read around each
     * proposal instead of held in registers. */
    __shared__ LaneJump s_lj[32];
    if (warp == 0) s_lj[lane] = make_lane_jump(p, lane);
    /* The block's counters (GPR_STAT_*), per warp in shared memory, added to
     * p.stats once when the warp leaves (the first claim's barrier orders
     * these stores before any use). */
    __shared__ unsigned long long s_st[8][GPR_NSTATS];
    for (int i = lane; i < GPR_NSTATS; i += 32) s_st[warp][i] = 0ull;
#define ST_ADD(i, v) do { if (lane == 0) s_st[warp][(i)] += (unsigned long long)(v); } while (0)

    __shared__ PipeSlot s_slot[2][8];
    __shared__ const gpr_word* s_pp[2][8];   /* published program ...          */
    __shared__ const float* s_pc[2][8];      /* ... and its constants          */
    __shared__ int s_cost[2][8];             /* its length (-1: none)          */
    __shared__ int s_cnt[2][8];              /* its node count                 */
    __shared__ int s_bad[2][8];              /* a point was invalid            */
    __shared__ int s_next[2];                /* next task of each pool         */
    __shared__ int s_group_base;

    /* the dataset's passes, chunks and task split */
    int npass = 0, nch = 0, ppt = 1, tpc = 1;
    float inv_tpc = 1.0f;
    auto split = [&](const DataView& v) {
        npass = ONEPASS ? 1 : (v.nd + 32 * K - 1) / (32 * K);
        nch = chunk_count(v.nd);
        tpc = min(npass, GPR_PIPE_TASKS);
        if (tpc < 1) tpc = 1;
        ppt = (npass + tpc - 1) / tpc;
        tpc = (npass + ppt - 1) / ppt;
        if (tpc < 1) tpc = 1;
        inv_tpc = __frcp_rn((float)tpc);
    };
    split(dv);
    /* chunk sums of (group, warp): the board, or this CTA's rows of p.part */
    float* const board = (float*)(wbase + (size_t)nwarps * pipe_warp_bytes(PL, p.max_instr, p.levels, K));
    auto part_row = [&](int g, int w) -> float* {
        if (p.part_stride > 0) return p.part + ((size_t)(blockIdx.x * 2 + g) * 8 + w) * p.part_stride;
        return board + ((size_t)g * 8 + w) * GPR_PIPE_CHUNKS;
    };

    GPR_PH(GPR_PH_CLAIM);

#pragma unroll 1
    for (;;) {
        /* claim two chains per warp: group 0 = base + warp, group 1 = base + nwarps + warp */
        __syncthreads();
        if (threadIdx.x == 0) {
            int b = atomicAdd(p.next_chain, 2 * nwarps);
            if (BATCHED && b < p.N) b = p.ds_order[b / p.chains_per_ds] * p.chains_per_ds + b % p.chains_per_ds;
            s_group_base = b;
        }
        __syncthreads();
        const int base = s_group_base;
        if (base >= p.N) break;
        if constexpr (BATCHED) {
            const int d = chain_dataset(p, base);   /* a group never straddles datasets */
            if (d != staged_ds) {
                dv = data_view(p, fx, STREAM, d);
                if (!STREAM && !stage_dataset(fx, bar, p, dv, d, bar_live)) break;
                bar_live = bar_live || dv.nd_pad > 0;
                staged_ds = d;
                split(dv);
            }
        }
        if (lane == 0) {
            s_slot[0][warp].chain = base + warp;
            s_slot[1][warp].chain = base + nwarps + warp;
        }
        __syncwarp();
        GPR_PH(GPR_PH_CLAIM);

#pragma unroll 1
        for (int h = 0; h < 2 * p.steps + 4; ++h) {
            const int g = h & 1;
            if (threadIdx.x == 0) s_next[g] = 0;   /* pool g is published now, evaluated next */

            /* ---- this warp's turn on its group-g chain ---- */
            {
                PipeSlot& SS = s_slot[g][warp];
                const int chain = SS.chain;
                const int step = (h - g) / 2 - 1;   /* the step proposed now: -1 the loaded state */
                const WarpSmem wg = carve_pipe<K>(mybase, PL, p.max_instr, p.levels, g);
                int publish = -1;
                int pbuf = 0, cbuf = 0, count = 0;
                if (chain < p.N) {
                    /* the chain's state, into registers */
                    df cur_prior = SS.cur_prior, cur_S = SS.cur_S, cur_cs = SS.cur_cs;
                    df prior = SS.prior, cs = SS.cs, fw = SS.fw, bw = SS.bw;
                    int cur = SS.cur, ccur = SS.ccur;
                    pbuf = SS.pbuf; cbuf = SS.cbuf;
                    int ninstr = SS.ninstr, cur_ninstr = SS.cur_ninstr, cur_count = SS.cur_count;
                    count = SS.count;
                    float len = SS.len, cur_len = SS.cur_len;
                    float rw_sd = SS.rw_sd, log_sd = SS.log_sd;
                    int n_cmoves = SS.n_cmoves;
                    bool structural = SS.structural != 0;
                    Rng r;
                    r.key0 = p.seed; r.key1 = (uint32_t)chain; r.drawn = 0;
                    r.s = SS.rs; r.blk = SS.rblk; r.w0 = SS.rw0; r.w1 = SS.rw1; r.w2 = SS.rw2; r.w3 = SS.rw3;
                    if (step >= 0) {
                        /* the accept rule for the proposal of step - 1 (the loaded state when step == 0) */
                        const bool init = step == 0;
                        df S;
                        if (s_bad[g][warp]) {
                            S = lik_invalid();
                        } else {
                            const float* pr = part_row(g, warp);
                            S = df_make(0.0f, 0.0f);
                            for (int c = 0; c < nch; ++c) S = df_add(S, df_make(pr[c], 0.0f));
                        }
                        GPR_PH(GPR_PH_COMBINE);
                        bool accept = true;
                        if (!init) {
                            float prob;
                            accept = mh_accept_u<RNG>(prior, S, cur_prior, cur_S, bw, fw, r, p, &prob);
                            if (!structural && p.adapt_target > 0.0f && p.const_mode == 1) {
                                log_sd = rm_update(log_sd, prob, p.adapt_target, n_cmoves++);
                                rw_sd = expf(log_sd);
                            }
                            if (structural) { ST_ADD(GPR_STAT_STRUCT_PROPOSED, 1); ST_ADD(GPR_STAT_STRUCT_ACCEPTED, accept); }
                            else { ST_ADD(GPR_STAT_CONST_PROPOSED, 1); ST_ADD(GPR_STAT_CONST_ACCEPTED, accept); }
                        }
                        ST_ADD(GPR_STAT_EVALS, 1); ST_ADD(GPR_STAT_EVAL_NODES, count);
                        if (accept) {
                            cur = pbuf; ccur = cbuf;
                            cur_len = len; cur_count = count; cur_ninstr = ninstr; cur_cs = cs;
                            cur_prior = prior; cur_S = S;
                        }
                        if (p.trace && !init && lane < p.trace_n && chain < p.trace_chains)
                            p.trace[((size_t)chain * p.steps + (step - 1)) * p.trace_n + lane] = wg.Cs[ccur][lane];
                        GPR_PH(GPR_PH_ACCEPT);
                    }
                    if (step < 0) {
                        /* load the chain (reference layout, main.cu:683-685) */
                        for (int i = lane; i < PL; i += 32) {
                            const int o = p.P[(size_t)i * p.N + chain];
                            wg.ops[0][i] = (uint8_t)((o >= 0 && o < OP_NALL) ? o : 255);
                            wg.Cs[0][i] = p.C[(size_t)i * p.N + chain];
                        }
                        __syncwarp();
                        r = rng_start<RNG>(p.seed, chain);
                        cur = ccur = pbuf = cbuf = 0;
                        cur_ninstr = cur_count = 0; cur_len = 0.0f;
                        cur_prior = cur_S = cur_cs = df_make(0.0f, 0.0f);
                        fw = bw = df_make(0.0f, 0.0f);
                        rw_sd = p.chain_scale ? p.chain_scale[chain] : p.rw_sd;
                        log_sd = logf(rw_sd);
                        n_cmoves = 0;
                        GPR_PH(GPR_PH_LOAD);
                    }
                    if (step < p.steps) {
                        const bool init = step < 0;
                        structural = !init && p.struct_every > 0 && (step % p.struct_every == 0);
                        bool need_compile = init;
                        if (structural) {
                            /* ---- structure move (main.cu:699-742) ---- */
                            fw = df_make(-p.logcount[cur_count], 0.0f);
                            const bool cur_invalid = !(isfinite(cur_prior.hi) && isfinite(cur_S.hi));
                            structure_move<RNG>(r, wg.ops[cur], wg.ops[cur ^ 1], cur_invalid, p, s_lj[lane], lane);
                            pbuf = cur ^ 1; cbuf = ccur;
                            need_compile = true;
                            GPR_PH(GPR_PH_STRUCT);
                        } else if (!init) {
                            /* ---- constant move (main.cu:743-806) ---- */
                            df fws, bws;
                            constant_move<RNG>(r, wg, wg.Cs[ccur], wg.Cs[ccur ^ 1], fws, bws, p, s_lj[lane], lane, rw_sd);
                            if (p.const_mode == 0) { fw = df_add(fw, fws); bw = df_add(bw, bws); }
                            pbuf = cur; cbuf = ccur ^ 1;
                            len = cur_len; count = cur_count; ninstr = cur_ninstr;
                            GPR_PH(GPR_PH_CONST);
                        }
                        __syncwarp();
                        if (need_compile) {
                            const CompileOut co = compile_parallel<NV>(wg.ops[pbuf], PL, wg.prog[pbuf],
                                                                   compile_scratch(wg.stk, PL), lane);
                            len = co.length; count = co.count; ninstr = co.ninstr;
                            __syncwarp();
                            GPR_PH(GPR_PH_COMPILE);
                        }
                        if (structural) {
                            bw = df_make(-p.logcount[count], 0.0f);
                            cs = cur_cs;
                        } else {
                            cs = cauchy_sum_u(wg.Cs[cbuf], p, lane);
                            GPR_PH(GPR_PH_CAUCHY);
                        }
                        prior = prior_u(len, cs, p);
                        publish = ninstr;
                    } else {
                        /* write back (main.cu:811-812 and the in-place P, C) */
                        for (int i = lane; i < PL; i += 32) {
                            const uint8_t o = wg.ops[cur][i];
                            if (o != 255) p.P[(size_t)i * p.N + chain] = (int32_t)o;
                            p.C[(size_t)i * p.N + chain] = wg.Cs[ccur][i];
                        }
                        if (lane == 0) {
                            p.prior[chain] = (double)cur_prior.hi + (double)cur_prior.lo;
                            p.lik[chain] = lik_of(cur_S, dv, p);
                            if (p.chain_scale && p.adapt_target > 0.0f && p.const_mode == 1) p.chain_scale[chain] = rw_sd;
                        }
                        GPR_PH(GPR_PH_STORE);
                    }
                    __syncwarp();
                    if (lane == 0) {
                        SS.cur_prior = cur_prior; SS.cur_S = cur_S; SS.cur_cs = cur_cs;
                        SS.prior = prior; SS.cs = cs; SS.fw = fw; SS.bw = bw;
                        SS.cur = cur; SS.ccur = ccur; SS.pbuf = pbuf; SS.cbuf = cbuf;
                        SS.ninstr = ninstr; SS.count = count; SS.cur_ninstr = cur_ninstr; SS.cur_count = cur_count;
                        SS.len = len; SS.cur_len = cur_len;
                        SS.rs = r.s; SS.rblk = r.blk; SS.rw0 = r.w0; SS.rw1 = r.w1; SS.rw2 = r.w2; SS.rw3 = r.w3;
                        SS.rw_sd = rw_sd; SS.log_sd = log_sd; SS.n_cmoves = n_cmoves;
                        SS.structural = structural ? 1 : 0;
                    }
                }
                __syncwarp();
                if (lane == 0) {
                    s_cost[g][warp] = publish;
                    s_cnt[g][warp] = count;
                    s_bad[g][warp] = 0;
                    s_pp[g][warp] = wg.prog[pbuf & 1];
                    s_pc[g][warp] = wg.Cs[cbuf & 1];
                }
                __syncwarp();
            }

            /* ---- evaluation tasks of the other group's proposals ---- */
            if (h >= 1) {
                const int e = g ^ 1;
                int my_rank = 64, nact = 0;
                {
                    const int cl = lane < nwarps ? s_cost[e][lane] : -1;
                    int rk = 0;
                    for (int j = 0; j < nwarps; ++j) {
                        const int cj = s_cost[e][j];
                        nact += cj >= 0;
                        rk += (cj > cl) || (cj == cl && j < lane);
                    }
                    if (cl >= 0) my_rank = rk;
                }
                const int ntasks = nact * tpc;
                GPR_PH(GPR_PH_RANK);
#pragma unroll 1
                for (;;) {
                    int t = 0;
                    if (lane == 0) t = atomicAdd(&s_next[e], 1);
                    t = __shfl_sync(FULLMASK, t, 0);
                    if (t >= ntasks) break;
                    /* task t: the chain of rank q (longest program first), passes of piece t - q tpc */
                    const int q = (int)__fmul_rz(__int2float_rn(t) + 0.5f, inv_tpc);
                    const int piece = t - q * tpc;
                    const int w = __ffs(__ballot_sync(FULLMASK, my_rank == q)) - 1;
                    if (s_bad[e][w]) continue;
                    const PCProg prog = {s_pp[e][w], s_pc[e][w]};
                    float* pr = part_row(e, w);
                    const int p0 = piece * ppt, p1 = min(npass, p0 + ppt);
                    int np = 0;
#pragma unroll 1
                    for (int pass = p0; pass < p1; ++pass) {
                        float csum[K / 4];
                        const bool bad = eval_pass_chunks<K, ONEPASS, ROLLED, NV, STREAM>(prog, my_stk, my_scr, ld,
                                                                                        dv, p, lane, pass, csum);
                        np += ONEPASS ? dv.nd : min(32 * K, dv.nd - pass * 32 * K);
                        if (lane == 0) {
#pragma unroll
                            for (int j = 0; j < K / 4; ++j)
                                if (pass * (K / 4) + j < nch) pr[pass * (K / 4) + j] = csum[j];
                            if (bad) s_bad[e][w] = 1;
                        }
                        GPR_PH_COUNT(GPR_PH_NPASSES, 1);
                        GPR_PH_COUNT(GPR_PH_NINSTR, s_cost[e][w]);
                        if (bad) break;
                    }
                    ST_ADD(GPR_STAT_EVAL_POINTS, np);
                    ST_ADD(GPR_STAT_EVAL_NODE_POINTS, (unsigned long long)(s_cnt[e][w] + 4) * (unsigned)np);
                }
                GPR_PH(GPR_PH_EVAL);
            }
            __syncthreads();
            GPR_PH(GPR_PH_BAR1);
        }
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

#endif /* GPR_PIPE_CUH */
