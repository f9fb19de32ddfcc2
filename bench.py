#!/usr/bin/env python
"""Benchmark: MH chain-steps/s and point-evals/s of the sampler on one GB300.

Workload (default "plain-mh-131k"): 131072 chains, PROGRAM_LENGTH 63 (max
postfix length 64), ops {+,-,*,/,exp,log,pow,x,const}, Gaussian random-walk
constant proposals sd 0.1, 250 float32 points of y = b1*exp(-b2*x)+b3 with
x ~ U[0,50] and noise N(0, 0.05 std(y)); blocks of 1000 MH steps, chains more
than 20 log-units below the block's MAP re-drawn from the prior between
blocks.  One bench "step" = one block (1000 MH steps of every chain).

value     : chain-steps/s of the device-resident block loop (kernel time from
            CUDA events on the library's stream, L2 flushed between blocks).
e2e       : the same through the C ABI with host buffers: each block uploads
            the state from pinned memory, runs, re-draws the chains below the
            MAP-delta cutoff on the device, and downloads state and scores
            (the reference's loop, main.cu:1156-1239, as the CLI runs it with
            --device-resample).
roofline  : the MH kernel against FP32 issue: (reachable nodes + 4) FP32
            ops per point evaluated over the kernel's time, against 152 SMs x
            128 lanes x the SM clock; roofline_hbm the same work's 12 bytes
            per point-eval against the measured HBM copy rate.
batched / streamed : short runs of the batched uneven workload (256 datasets)
            and of the large streamed three-variable workload (65,536
            points, random-walk and Hamiltonian constant moves, batched
            path), reported beside the headline.
cpu_baseline / --impl reference : the reference's own per-chain code
            (main.cu:679-813) compiled for the host cores, OpenMP over chains,
            on a bounded sample of the same chains.
ess       : ESS/s of constants, gradient moves (HMC, MALA) against
            random-walk MH, on 65536 chains of the rational function
            y = (b1 + b2 x + b3 x^2)/(1 + b4 x + b5 x^2) fitted to 1024 points
            (x ~ U[-3, 3], noise N(0, 0.02)), constants-only moves
            (see ess_comparison).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# where the nvidia-smi clock samples of the timed regions are written
CLOCKS_DIR = os.environ.get("GPR_CLOCKS_DIR", tempfile.gettempdir())
sys.path.insert(0, ROOT)

from tests import helpers as H  # noqa: E402  (seeded synthetic inputs)

WORKLOADS = {
    "plain-mh-131k": dict(N=131072, PL=63, nd=250, data="expdecay", ops="basic", rw_sd=0.1,
                          mh_steps=1000, map_delta=20.0, blocks=20),
    "plain-mh-1k": dict(N=1024, PL=31, nd=101, data="quad", ops="basic", rw_sd=0.1,
                        mh_steps=1000, map_delta=20.0, blocks=10),
    # three input variables, 65536 points read from device memory in every pass
    "streamed-3var-16k": dict(N=16384, PL=127, nd=65536, data="multivar", ops="multi", rw_sd=0.1,
                              mh_steps=20, map_delta=0.0, blocks=1),
    # 256 datasets of uneven size (log-uniform in [8, 4096] points), 512 chains
    # each, in one launch; blocks replayed from a captured graph
    "batched-256ds-131k": dict(N=131072, PL=47, nds=256, data="batched", ops="basic", rw_sd=0.1,
                               mh_steps=200, blocks=5),
    # the batched workload cut to 64 datasets x 128 chains, the streamed layout, no
    # comparison handles: the case ncu captures
    "batched-64ds-8k-profile": dict(N=8192, PL=47, nds=64, data="batched", ops="basic", rw_sd=0.1,
                                    mh_steps=50, blocks=1, stream=True, compare=False),
    # the streamed workload cut to 8192 chains x 5 steps: the case ncu captures
    "streamed-3var-8k-profile": dict(N=8192, PL=127, nd=65536, data="multivar", ops="multi", rw_sd=0.1,
                                     mh_steps=5, map_delta=0.0, blocks=1),
    # Hamiltonian moves on 8192 chains of the rational model: the case ncu captures
    "hmc-rational-8k-profile": dict(N=8192, PL=31, nd=1024, data="rational", ops="basic", rw_sd=0.0,
                                    mh_steps=20, map_delta=0.0, blocks=1),
    # the 131k workload cut to 8192 chains x 100 steps: the case ncu captures
    "plain-mh-8k-profile": dict(N=8192, PL=63, nd=250, data="expdecay", ops="basic", rw_sd=0.1,
                                mh_steps=100, map_delta=20.0, blocks=1),
}
METRIC = "MH chain-steps/s & point-evals/s (1 GB300); ESS/s gradient vs random-walk MH"
# DRAM bytes (read + write) of one mh_block_kernel launch of the plain-mh-131k workload, taken
# from an ncu capture of that launch (dram__bytes_read.sum + dram__bytes_write.sum), not measured
# in this run: the chain state read and written once; the dataset lives in shared memory.
MH_LAUNCH_DRAM_BYTES = 113.43e6
MH_LAUNCH_DRAM_SOURCE = "ncu capture of one launch (dram__bytes_read.sum + dram__bytes_write.sum), not this run"


def config_of(args, w):
    """The workload keys both arms report (the GPU arm adds its layout elsewhere)."""
    return {"workload": args.workload, **{k: w[k] for k in ("N", "PL", "nd", "mh_steps", "map_delta")},
            "ops": w["ops"], "const_proposal": "rw:%g" % w["rw_sd"], "rng": "lcg",
            "l2": "GPU arm: flushed between blocks (256 MB write); the CPU arm has no GPU cache"}


def fp32_roofline(node_points, seconds, nsm, peaks, sm_mhz=None, traffic=None):
    """Algorithmic FP32 ops ((reachable nodes + 4) per point-eval, a
    transcendental counting as one) per second against FP32 issue:
    SMs x 128 lanes x the maximum SM clock (nominal: no measured FP32 peak).
    traffic: DRAM bytes of one launch from an ncu capture, when there is one."""
    peak = nsm * 128 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    achieved = node_points / seconds / 1e12
    out = {"bound": "fp32-issue", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
           "frac": achieved / peak, "traffic": traffic,
           "traffic_source": MH_LAUNCH_DRAM_SOURCE if traffic else None,
           "peak_source": "nominal: SMs x 128 FP32 lanes x max SM clock (MEASURED_PEAKS.json has no FP32 figure)",
           "note": "algorithmic ops = (reachable non-pass-through nodes + 4) per point evaluated; exp, log, pow "
                   "and division count as one op but cost 10-70 FP32 instructions each"}
    if sm_mhz:
        out["frac_at_measured_clock"] = achieved / (nsm * 128 * sm_mhz * 1e6 / 1e12)
    return out


def dataset(w):
    if w["data"] == "expdecay":
        return H.expdecay_data(w["nd"], seed=2024)
    return H.quad_data(w["nd"], seed=2024)


def initial_state(w, seed=99):
    ops = H.OPSET_BASIC if w["ops"] == "basic" else None
    return H.random_programs(w["N"], w["PL"], ops=ops, seed=seed, shallow_frac=0.0)


def resample_host(P, C, prior, lik, delta, ops, rng):
    """Re-draw chains whose posterior is below max - delta from the prior-draw
    distribution of the reference's initialisation (main.cu:1133-1137)."""
    post = prior + lik
    fin = np.isfinite(post)
    if not fin.any():
        return 0
    cut = post[fin].max() - delta
    bad = np.where(post < cut)[0]
    if bad.size:
        opsa = np.asarray(ops)
        P[:, bad] = opsa[rng.integers(0, len(opsa) - 1, size=(P.shape[0], bad.size))]
        C[:, bad] = (10.0 ** rng.integers(-4, 4, size=(P.shape[0], bad.size)) *
                     rng.normal(size=(P.shape[0], bad.size))).astype(np.float32)
    return bad.size


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self, device_index=0):
        try:
            rows = [r.split(", ") for r in open(self.path).read().strip().splitlines()]
        except OSError:
            return None
        rows = [r for r in rows if len(r) >= 9 and r[0].strip() == str(device_index)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(rows[0][2]),
                "samples": len(rows), "reasons": sorted(reasons)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# constants-mixing comparison: 65536 chains of the rational function's own
# structure (five constants), 1024 points, constants-only moves
ESS_WORKLOAD = dict(N=65536, PL=31, nd=1024, traced=4096, rw_steps=3000)


class EssRig:
    """The constants-mixing setup: 65536 copies of the rational model's own
    structure (five constants, 1024 points), constants-only moves, burned in
    from the generating constants by an adapted random walk (4000 steps)."""

    def __init__(self, g, stream):
        w = ESS_WORKLOAD
        self.g, self.stream = g, stream
        self.N, self.PL = w["N"], w["PL"]
        b, _ = H.rational_coefficients(0)
        self.data = H.rational_data(w["nd"], seed=0)
        P, C = H.rational_program(self.N, b)
        self.used = H.used_constants(P)
        s = self.sampler("rw", sd=0.001)
        s.set_state(P, C)
        s.adapt_scales(0.234)
        for i in range(4):
            s.run_block(1000, 10 + i)
        self.state = s.get_state()[:2]
        s.close()

    def sampler(self, mode, **kw):
        g = self.g
        if mode == "rw":
            s = g.Sampler(self.N, program_length=self.PL, ops=H.OPSET_BASIC, const_proposal=g.CONST_RANDOM_WALK,
                          rw_sd=kw["sd"], stream=self.stream.cuda_stream)
            s.set_moves(0)
        else:
            s = g.Sampler(self.N, program_length=self.PL, ops=H.OPSET_BASIC, const_proposal=g.CONST_HMC,
                          stream=self.stream.cuda_stream)
            s.set_moves(0, kw["eps"], kw["L"])
        s.set_data(*self.data)
        return s

    def adapted_rw(self):
        """A random walk with per-chain sd adapted toward acceptance 0.234 (2000 steps)."""
        s = self.sampler("rw", sd=0.001)
        s.set_state(*self.state)
        s.adapt_scales(0.234)
        for i in range(2):
            s.run_block(1000, 20 + i)
        s.adapt_scales(0.0)
        return s

    def adapted_hmc(self, L, target, adapt_steps, len_jit=0.0):
        """Hamiltonian moves with L leapfrog steps (count jittered by len_jit),
        the CTA shape autotuned and per-chain steps adapted toward target."""
        s = self.sampler("hmc", eps=0.0005, L=L)
        s.set_state(*self.state)
        s.autotune(steps=10, seed=77)          # CTA shape against L1 for the gradient tapes
        s.set_hmc_jitter(0.0, len_jit)
        s.adapt_scales(target)
        for i in range(2):
            s.run_block(adapt_steps, 30 + i)
        s.adapt_scales(0.0)
        return s

    def timed(self, s, steps, seed):
        import torch
        s.set_state(*self.state)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.reset_stats()
        e0.record(self.stream)
        s.run_block(steps, seed)
        e1.record(self.stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, s.stats()

    def trace(self, s, steps, seed, chains):
        """The same trajectories as timed(s, steps, seed), constants recorded
        for the first `chains` chains."""
        s.set_state(*self.state)
        return s.run_block_traced(steps, seed, self.PL, chains=chains)

    def ess(self, tr):
        """(population ESS per chain, mean per-chain Geyer ESS) of a trace,
        min over the five constants."""
        from gpuropolis_gb300.diagnostics import chain_ess, population_ess
        n = tr.shape[0]
        return population_ess(tr, self.used[:, :n]), float(chain_ess(tr, self.used[:, :n]).mean())


def ess_comparison(g, stream, dev):
    """ESS/s of the constants under Gaussian random-walk MH (the configured sd
    0.1, and a per-chain adapted sd) and under gradient moves (HMC with 8 and
    32 leapfrog steps, each also with a jittered leapfrog count, and MALA),
    each from the same burned-in state, with per-chain step sizes
    adapted beforehand; gradient arms run for the random walk's wall time (at
    least 30 steps).  ESS per chain = min over the five constants of the
    population ESS (pooled autocorrelation of the traced chains, all
    stationary copies of one model), which stays accurate on runs only a few
    autocorrelation times long; the per-chain Geyer figure, which
    overestimates such runs, is kept beside it.  ESS/s = ESS per chain x N /
    seconds of the untraced block."""
    w = ESS_WORKLOAD
    rig = EssRig(g, stream)
    N, NT = rig.N, w["traced"]

    def arm(s, steps, seed, extra):
        dt, st = rig.timed(s, steps, seed)
        e_pop, e_geyer = rig.ess(rig.trace(s, steps, seed, NT))
        out = {"steps": steps, "seconds": dt, "chain_steps_per_s": N * steps / dt,
               "acceptance": st["const_accepted"] / max(1, st["const_proposed"]),
               "ess_per_chain": e_pop, "ess_per_s": e_pop * N / dt,
               "ess_per_chain_geyer": e_geyer, "ess_per_s_geyer": e_geyer * N / dt}
        out.update(extra)
        return out

    res = {}
    s = rig.sampler("rw", sd=0.1)
    res["rw_sd_0.1"] = arm(s, w["rw_steps"], 1, {"sd": 0.1})
    s.close()
    s = rig.adapted_rw()
    sc = s.chain_scales()
    res["rw_adapted"] = arm(s, w["rw_steps"], 2, {"sd_median": float(np.median(sc)), "target": 0.234})
    t_rw = res["rw_adapted"]["seconds"]
    s.close()
    # HMC with the workload's 8 leapfrog steps and with 32 (longer trajectories cross the
    # correlated posterior of the rational model's coefficients in fewer MH steps), each also
    # with the leapfrog count drawn per move from [1, 2L]; and MALA
    for name, L, tgt, adapt_steps, len_jit in (("hmc_L8", 8, 0.8, 150, 0.0), ("hmc_L8_jitter", 8, 0.8, 150, 1.0),
                                               ("hmc_L32", 32, 0.65, 100, 0.0),
                                               ("hmc_L32_jitter", 32, 0.65, 100, 1.0),
                                               ("mala", 1, 0.574, 600, 0.0)):
        s = rig.adapted_hmc(L, tgt, adapt_steps, len_jit)
        sc = s.chain_scales()
        dt, _ = rig.timed(s, 20, 5)
        steps = max(30, int(t_rw / (dt / 20)))
        res[name] = arm(s, steps, 3, {"leapfrog_steps": L, "leapfrog_count_jitter": len_jit,
                                      "eps_median": float(np.median(sc)), "target": tgt})
        s.close()
    # the configured move as the workload states it: step 0.01, 8 leapfrog steps, not adapted
    s = rig.sampler("hmc", eps=0.01, L=8)
    s.set_state(*rig.state)
    s.autotune(steps=10, seed=77)
    dt, _ = rig.timed(s, 20, 5)
    steps = max(30, int(t_rw / (dt / 20)))
    res["hmc_L8_eps0.01"] = arm(s, steps, 3, {"leapfrog_steps": 8, "eps": 0.01, "adapted": False})
    s.close()
    arms = ("hmc_L8", "hmc_L8_jitter", "hmc_L32", "hmc_L32_jitter", "mala")
    best_arm = max(arms, key=lambda a: res[a]["ess_per_s"])
    rw_ad = res["rw_adapted"]["ess_per_s"]
    rw_ad_g = res["rw_adapted"]["ess_per_s_geyer"]
    return {"workload": "rational-65k", "N": N, "PL": rig.PL, "nd": w["nd"], "constants": 5,
            "moves": "constants only (no structure moves)", "traced_chains": NT,
            "ratio_of_record": {"gradient_vs_adapted_rw": res[best_arm]["ess_per_s"] / rw_ad, "best_arm": best_arm,
                                "hmc_L8_adapted_vs_adapted_rw": res["hmc_L8"]["ess_per_s"] / rw_ad,
                                "hmc_L8_jitter_vs_adapted_rw": res["hmc_L8_jitter"]["ess_per_s"] / rw_ad,
                                "hmc_L8_configured_vs_adapted_rw": res["hmc_L8_eps0.01"]["ess_per_s"] / rw_ad,
                                "target": 3.0,
                                "met": bool(res[best_arm]["ess_per_s"] / rw_ad >= 3.0),
                                "estimator": "population ESS (pooled autocorrelation)"},
            "per_chain_geyer": {"gradient_vs_adapted_rw": max(res[a]["ess_per_s_geyer"] for a in arms) / rw_ad_g,
                                "hmc_L8_adapted_vs_adapted_rw": res["hmc_L8"]["ess_per_s_geyer"] / rw_ad_g,
                                "note": "each chain's own mean: overestimates runs only a few autocorrelation "
                                        "times long, the random walk's most of all"},
            **res,
            "footnote": {"gradient_vs_rw_sd_0.1": res[best_arm]["ess_per_s"] / max(res["rw_sd_0.1"]["ess_per_s"],
                                                                                   1e-300),
                         "note": "the configured sd 0.1 random walk accepts almost no proposal on this posterior; "
                                 "it is not a baseline worth beating"},
            "method": "population ESS: autocorrelation pooled over the traced chains (stationary copies of one "
                      "model) around the pooled mean, Geyer initial monotone sequence; min over the five "
                      "constants; every arm runs the adapted random walk's wall time from the same burned-in state"}


def ess_horizons(args):
    """How the two ESS estimators depend on the run length: the adapted random
    walk at 3000, 10000 and 30000 steps and HMC with 32 leapfrog steps (fixed
    and jittered count) at 30, 100 and 300 steps, 2048 traced chains each, one
    trajectory per arm cut at each horizon.  An estimator that is right gives
    the same ESS per step at every horizon."""
    import torch
    import gpuropolis_gb300 as g
    stream = torch.cuda.Stream(torch.device("cuda", 0))
    torch.cuda.set_stream(stream)
    rig = EssRig(g, stream)
    out = {"workload": "rational-65k", "traced_chains": 2048, "arms": {}}
    for name, mk, horizons in (("rw_adapted", lambda: rig.adapted_rw(), (3000, 10000, 30000)),
                               ("hmc_L32", lambda: rig.adapted_hmc(32, 0.65, 100), (30, 100, 300)),
                               ("hmc_L32_jitter", lambda: rig.adapted_hmc(32, 0.65, 100, 1.0), (30, 100, 300))):
        s = mk()
        tr = rig.trace(s, horizons[-1], 2, 2048)
        s.close()
        rows = []
        for T in horizons:
            e_pop, e_geyer = rig.ess(np.ascontiguousarray(tr[:, :T]))
            rows.append({"steps": T, "ess_population": e_pop, "ess_geyer": e_geyer,
                         "steps_per_ess_population": T / max(e_pop, 1e-300),
                         "steps_per_ess_geyer": T / max(e_geyer, 1e-300)})
        del tr
        out["arms"][name] = rows
    print(json.dumps(out), flush=True)


def run_hmc_profile(args):
    """Throughput of the Hamiltonian-move kernel alone: 8192 chains of the
    rational model, HMC with 8 leapfrog steps (step 0.001), constants only,
    blocks of 20 MH steps; the case ncu captures."""
    import torch
    import gpuropolis_gb300 as g
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    N, steps = 8192, 20
    b, _ = H.rational_coefficients(0)
    x, y, sd = H.rational_data(1024, seed=0)
    P, C = H.rational_program(N, b)
    s = g.Sampler(N, program_length=31, ops=H.OPSET_BASIC, const_proposal=g.CONST_HMC, stream=stream.cuda_stream)
    s.set_data(x, y, sd)
    s.set_moves(0, 0.001, 8)
    s.set_state(P, C)
    for i in range(args.warmup):
        s.run_block(steps, 1 + i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        s.run_block(steps, 100 + i)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    print(json.dumps({"metric": "HMC chain-steps/s (8 leapfrog steps, 1024 points)", "unit": "chain-steps/s",
                      "value": N * steps * args.steps / sec,
                      "gradient_evals_per_s": N * steps * args.steps * 8 / sec,
                      "config": {"workload": args.workload, "N": N, "PL": 31, "nd": 1024, "mh_steps": steps},
                      "launch": s.launch_geometry()}))


class _PortRunner:
    """The C restatement of the reference (oracle/gpr_oracle.c) with the
    reference oracle's run_kernel interface: the CPU baseline where the
    reference's own source could not be built."""

    def __init__(self, w):
        from oracle import port
        self.port = port
        ops = H.OPSET_BASIC if w["ops"] == "basic" else None
        self.cfg = port.cfg(PL=w["PL"], ops=ops, rng=0, const_mode=1 if w["rw_sd"] > 0 else 0,
                            rw_sd=w["rw_sd"], project_math=0)

    def run_kernel(self, P, C, x, y, sd, steps, seed, nthreads=0):
        return self.port.run_block(self.cfg, P, C, x, y, sd, steps, seed, nthreads=nthreads)


def cpu_runner(w):
    """(runner, kind): the reference's own code compiled for the host, or the
    restatement when the reference source is absent."""
    from oracle import ref as oref
    try:
        return oref.get(pl=w["PL"], opset=1 if w["ops"] == "basic" else 0, project_math=0,
                        rw_sd=w["rw_sd"]), "reference"
    except RuntimeError:
        return _PortRunner(w), "port"


def streamed_measure(args, w, steps_timed, warmup):
    """Large streamed data: 16384 chains, PROGRAM_LENGTH 127, 65536 points of
    three input variables (x1, x2, x3 ~ N(0, 1), y = sin(x1) x2 + exp(-x3^2)
    + N(0, 0.05)), op set {+,-,*,/,sin,cos,exp,x1,x2,x3,const}; the dataset is
    read from device memory (L2) in every pass (it cannot be staged per CTA).
    Two legs: random-walk constants (sd 0.1) with the reference's structure
    moves, on a single-dataset handle; then, as the workload specifies, the
    same chains on the batched path (the dataset behind gpr_set_batched_data,
    blocks replayed from a captured graph) with Hamiltonian constant moves (8
    leapfrog steps) beside the structure moves.  Data bytes per point-eval:
    20 (x1, x2, x3, y, w)."""
    import torch
    import gpuropolis_gb300 as g
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    N, PL, nd, steps = w["N"], w["PL"], w["nd"], w["mh_steps"]
    x1, x2, x3, y, sd = H.multivar_data(nd, seed=2024)
    P, C = g.host_init_chains(N, PL, 99, ops=H.OPSET_MULTI)
    peaks = measured_peaks()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count

    def timed(run, seed0, st_handle):
        for i in range(warmup):
            run(seed0 + i)
        torch.cuda.synchronize()
        st_handle.reset_stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps_timed):
            run(seed0 + 100 + i)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, st_handle.stats()

    def leg(sec, st, geo):
        pe = st["eval_points"] / sec
        return {"chain_steps_per_s": N * steps * steps_timed / sec, "point_evals_per_s": pe,
                "data_read_gbs": pe * 20 / 1e9,
                "roofline": fp32_roofline(st["eval_node_points"], sec, nsm, peaks),
                "roofline_hbm": hbm_roofline(st["eval_points"], sec, peaks, None, nbytes=20),
                "acceptance": {"structure": st["struct_accepted"] / max(1, st["struct_proposed"]),
                               "constant": st["const_accepted"] / max(1, st["const_proposed"])},
                "launch": geo}

    s = g.Sampler(N, program_length=PL, ops=H.OPSET_MULTI, n_vars=3, const_proposal=g.CONST_RANDOM_WALK,
                  rw_sd=0.1, stream=stream.cuda_stream)
    try:
        s.set_data3(x1, x2, x3, y, sd)
        s.set_state(P, C)
        sec, st = timed(lambda sd_: s.run_block(steps, sd_), 1, s)
        rw = leg(sec, st, s.launch_geometry())
        Pw, Cw, _, _ = s.get_state()
    finally:
        s.close()
    h = g.Sampler(N, program_length=PL, ops=H.OPSET_MULTI, n_vars=3, const_proposal=g.CONST_HMC,
                  stream=stream.cuda_stream)
    try:
        h.set_batched_data([(x1, x2, x3, y, sd)])
        h.set_moves(5, 0.001, 8)
        h.set_state(Pw, Cw)
        h.capture_blocks(1, steps)
        hsec, hst = timed(lambda sd_: h.run_captured([sd_]), 7, h)
        hmc = leg(hsec, hst, h.launch_geometry())
        hmc["likelihood_gradients_per_s"] = hst["evals"] / hsec
        hmc["path"] = "batched (gpr_set_batched_data, one dataset), captured graph of blocks"
    finally:
        h.close()
    return {"metric": "MH chain-steps/s, large streamed multivariate data", "unit": "chain-steps/s",
            "value": rw["chain_steps_per_s"], "steps": steps_timed, "warmup": warmup,
            "rw": rw, "hmc_batched": hmc,
            "note": "the 1.3 MB dataset stays in L2: data bandwidth is served on chip and can exceed the HBM peak",
            "config": {"workload": "streamed-3var-16k", "N": N, "PL": PL, "nd": nd, "n_vars": 3,
                       "mh_steps": steps, "ops": "{+,-,*,/,sin,cos,exp,x1,x2,x3,const}",
                       "hmc": {"leapfrog_steps": 8, "eps": 0.001, "struct_every": 5}}}


def run_streamed(args, w):
    out = streamed_measure(args, w, args.steps, args.warmup)
    out.update({"higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)"})
    print(json.dumps(out))


def hbm_roofline(point_evals, seconds, peaks, traffic, nbytes=12):
    """The MH kernel against the HBM roof: algorithmic bytes = 12 per
    point-eval (x, y and the weight of one point; 20 with three input
    variables), over the timed launches.  The kernel reads them from shared
    memory, registers or L2, not HBM (its DRAM traffic per launch is
    `traffic`, the chain state); the bound is FP32 issue (roofline)."""
    peak = peaks.get("hbm_gbs")
    achieved = point_evals * nbytes / seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if peak else None, "traffic": traffic,
            "traffic_source": MH_LAUNCH_DRAM_SOURCE if traffic else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if peak else None,
            "note": "12 algorithmic bytes per point-eval, served from shared memory (staged layout) or "
                    "L1/L2 (streamed layout), not HBM; DRAM traffic per launch (traffic) is the chain state. "
                    "The kernel is latency-bound, not HBM-bound."}


def batched_datasets(g, nds, seed=2024):
    """nds datasets: sizes log-uniform in [8, 4096], x ~ U[-5, 5], y = f(x) +
    N(0, 0.01 std f(x)) with f a program of 3-15 nodes drawn from the prior
    over the op set {+,-,*,/,exp,log,pow,x,const} (heap of 15 nodes, ops
    uniform, Cauchy(0, 1) constants), redrawn until it is finite and not
    constant on the dataset's x.  f is evaluated by the library's own
    evaluator.  Returns the datasets and the generating programs."""
    r = np.random.default_rng(seed)
    sizes = np.round(np.exp(r.uniform(np.log(8), np.log(4096), nds))).astype(int)
    M, PLg = 64, 15
    ev = g.Sampler(M, program_length=PLg, ops=H.OPSET_BASIC)
    out, gens = [], []
    try:
        for d in range(nds):
            x = r.uniform(-5, 5, sizes[d]).astype(np.float32)
            while True:
                P, _ = H.random_programs(M, PLg, ops=H.OPSET_BASIC, seed=int(r.integers(1 << 30)),
                                         shallow_frac=1.0)
                C = r.standard_cauchy((PLg, M)).astype(np.float32)
                ev.set_state(P, C)
                vals, _, count = ev.eval_values(x)
                with np.errstate(all="ignore"):
                    sdv = np.std(vals.astype(np.float64), axis=1)
                    ok = ((count >= 3) & (count <= 15) & np.all(np.isfinite(vals), axis=1)
                          & (np.max(np.abs(vals), axis=1) < 1e6) & (sdv > 1e-3))
                if ok.any():
                    c = int(np.argmax(ok))
                    break
            f = vals[c].astype(np.float64)
            noise = 0.01 * sdv[c]
            y = (f + r.normal(0, noise, sizes[d])).astype(np.float32)
            out.append((x, y, np.full(sizes[d], noise, np.float32)))
            gens.append((P[:, c].copy(), C[:, c].copy(), int(count[c])))
    finally:
        ev.close()
    return out, gens


def batched_measure(args, w, steps_timed, warmup, compare=True):
    """Batched uneven workload: 256 independent datasets (sizes log-uniform in
    [8, 4096] points), 512 chains each (131072 chains), PROGRAM_LENGTH 47, op
    set {+,-,*,/,exp,log,pow,x,const}, random-walk constants (sd 0.1) with the
    reference's structure moves; the layout picked by the autotuner; one
    timed step = one replay of a captured graph of 5 MH blocks of 200 steps
    (1000 MH steps per chain), then the device resampling per dataset
    (chains more than 20 log-units below their dataset's MAP re-drawn).
    Beside it, the same chains run as 256 separate handles (one launch per
    dataset per block)."""
    import torch
    import gpuropolis_gb300 as g
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    N, PL, nds, steps, nb = w["N"], w["PL"], w["nds"], w["mh_steps"], w["blocks"]
    cpd = N // nds
    sets, gens = batched_datasets(g, nds)
    sizes = np.array([len(d[0]) for d in sets])
    P0, C0 = H.random_programs(N, PL, ops=H.OPSET_BASIC, seed=99, shallow_frac=0.0)
    s = g.Sampler(N, program_length=PL, ops=H.OPSET_BASIC, rng=g.RNG_LCG, const_proposal=g.CONST_RANDOM_WALK,
                  rw_sd=w["rw_sd"], stream=stream.cuda_stream)
    s.set_batched_data(sets)
    if w.get("stream"):
        s.set_streaming(True)
    s.set_state(P0, C0)
    default_geo = s.launch_geometry()
    for i in range(warmup):
        s.run_block(steps, 11 + i)
    tuned = None if args.no_autotune else s.autotune(steps=50, seed=4242)
    geo = s.launch_geometry()
    s.capture_blocks(nb, steps)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    s.run_captured([5 + b for b in range(nb)])   # the first replay uploads the graph
    torch.cuda.synchronize()
    s.reset_stats()
    launches0 = s.launch_count()
    evs = []
    clk = ClockSampler(os.path.join(CLOCKS_DIR, "clocks_batched.csv"))
    with clk:
        for i in range(steps_timed):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run_captured([1000 * (i + 1) + b for b in range(nb)])
            s.lib.gpr_resample_datasets(s.h, 1, 20.0, 77 + i, None, None)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
    ms = float(sum(a.elapsed_time(b) for a, b in evs))
    st = s.stats()
    launches = s.launch_count() - launches0
    value = N * steps * nb * steps_timed / (ms / 1e3)

    # end to end through the C ABI: pinned host state in, replay, state out
    Ph = torch.empty((PL, N), dtype=torch.int32, pin_memory=True).numpy()
    Ch = torch.empty((PL, N), dtype=torch.float32, pin_memory=True).numpy()
    prh = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    lih = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    lib, ptr = s.lib, (lambda a: a.ctypes.data_as(g.ctypes.c_void_p))
    lib.gpr_get_state(s.h, ptr(Ph), ptr(Ch), ptr(prh), ptr(lih))
    seeds = np.arange(nb, dtype=np.int32) + 77
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(steps_timed, 2))
    for i in range(e2e_steps):
        lib.gpr_set_state(s.h, ptr(Ph), ptr(Ch))
        lib.gpr_run_captured(s.h, ptr(seeds + i))
        lib.gpr_resample_datasets(s.h, 1, 20.0, 99 + i, None, None)
        lib.gpr_get_state(s.h, ptr(Ph), ptr(Ch), ptr(prh), ptr(lih))
    e2e = N * steps * nb * e2e_steps / (time.perf_counter() - t0)
    Pw, Cw, _, _ = s.get_state()
    s.close()

    # the same chains as 256 separate handles, one block each, one launch per dataset
    hs = []
    sep = float("nan")
    try:
        for d in range(nds if (compare and w.get("compare", True)) else 0):
            h = g.Sampler(cpd, program_length=PL, ops=H.OPSET_BASIC, rng=g.RNG_LCG,
                          const_proposal=g.CONST_RANDOM_WALK, rw_sd=w["rw_sd"], stream=stream.cuda_stream)
            h.set_data(*sets[d])
            h.set_state(Pw[:, d * cpd:(d + 1) * cpd], Cw[:, d * cpd:(d + 1) * cpd])
            hs.append(h)
        if hs:
            for h in hs:
                h.run_block(steps, 3)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for h in hs:
                h.run_block(steps, 4)
            e1.record(stream)
            torch.cuda.synchronize()
            sep = N * steps / (e0.elapsed_time(e1) / 1e3)
    finally:
        for h in hs:
            h.close()

    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    return {
        "metric": "MH chain-steps/s, batched uneven datasets", "value": value, "unit": "chain-steps/s",
        "n_gpus": 1, "steps": steps_timed, "warmup": warmup, "ms_per_step": ms / steps_timed,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
        "point_evals_per_s": st["eval_points"] / (ms / 1e3),
        "separate_handles": {"chain_steps_per_s": sep, "launches_per_block": nds,
                             "batched_over_separate": value / sep} if sep == sep else None,
        "e2e": {"value": e2e, "unit": "chain-steps/s", "h2d_bytes_per_step": Ph.nbytes + Ch.nbytes,
                "d2h_bytes_per_step": Ph.nbytes + Ch.nbytes + prh.nbytes + lih.nbytes, "steps": e2e_steps},
        "gpu_launches": launches,
        "roofline": fp32_roofline(st["eval_node_points"], ms / 1e3, props.multi_processor_count, peaks),
        "roofline_hbm": hbm_roofline(st["eval_points"], ms / 1e3, peaks, None),
        "acceptance": {"structure": st["struct_accepted"] / max(1, st["struct_proposed"]),
                       "constant": st["const_accepted"] / max(1, st["const_proposed"])},
        "clocks": clk.summary(0),
        "config": {"workload": args.workload, "N": N, "PL": PL, "datasets": nds, "chains_per_dataset": cpd,
                   "points": {"total": int(sizes.sum()), "min": int(sizes.min()), "max": int(sizes.max()),
                              "median": float(np.median(sizes))},
                   "generator_nodes": {"min": min(c for _, _, c in gens), "max": max(c for _, _, c in gens)},
                   "mh_steps_per_block": steps, "blocks_per_replay": nb, "rng": "lcg",
                   "resample": "per dataset, map-delta 20, on the device after each replay",
                   "const_proposal": "rw:%g" % w["rw_sd"], "l2": "flushed between replays (256 MB write)",
                   "launch_default": default_geo, "launch": geo, "autotuned": tuned}}


def run_batched(args, w):
    print(json.dumps(batched_measure(args, w, args.steps, args.warmup)))


def cpu_reference_rate(w, P, C, x, y, sd, target_s=12.0, threads=0, chains=None):
    """chain-steps/s of the reference's own code (or its restatement) on the
    host cores, measured on chains [0, S) of the given state, S sized to
    about target_s seconds."""
    o, kind = cpu_runner(w)
    ncores = threads or os.cpu_count()
    steps = w["mh_steps"]
    if chains is None:
        S = min(w["N"], 4 * ncores)
        Ps, Cs = np.ascontiguousarray(P[:, :S]), np.ascontiguousarray(C[:, :S])
        t0 = time.perf_counter()
        o.run_kernel(Ps, Cs, x, y, sd, steps, 12345, nthreads=ncores)
        dt = max(time.perf_counter() - t0, 1e-3)
        chains = int(min(w["N"], max(S, S * target_s / dt)))
    Ps, Cs = np.ascontiguousarray(P[:, :chains]), np.ascontiguousarray(C[:, :chains])
    t0 = time.perf_counter()
    o.run_kernel(Ps, Cs, x, y, sd, steps, 12345, nthreads=ncores)
    dt = time.perf_counter() - t0
    return chains * steps / dt, ncores, chains, dt, kind


def run_reference(args, w):
    """--impl reference: the reference's CPU code on a bounded sample per step."""
    x, y, sd = dataset(w)
    P, C = initial_state(w)
    ncores = os.cpu_count()
    rates = []
    chains = None
    for i in range(args.warmup + args.steps):
        rate, cores, chains, dt, kind = cpu_reference_rate(w, P, C, x, y, sd, chains=chains)
        if i >= args.warmup:
            rates.append(rate)
    value = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "chain-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * w["N"] * w["mh_steps"] / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "point_evals_per_s": value * w["nd"],
        "config": config_of(args, w),
        "cpu_baseline": {"value": value, "unit": "chain-steps/s", "cores": ncores, "kind": kind,
                         "sample": "%d chains x %d MH steps per step, from the seeded initial state"
                                   % (chains, w["mh_steps"])},
        "e2e": {"value": value, "unit": "chain-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args, w):
    import torch
    import gpuropolis_gb300 as g

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)          # the library's stream; events are recorded on it
    torch.cuda.set_stream(stream)

    x, y, sd = dataset(w)
    P0, C0 = initial_state(w, seed=99 + rank)
    ops = H.OPSET_BASIC if w["ops"] == "basic" else list(range(27))
    s = g.Sampler(w["N"], program_length=w["PL"], ops=ops, rng=g.RNG_LCG,
                  const_proposal=g.CONST_RANDOM_WALK, rw_sd=w["rw_sd"], device=local,
                  stream=stream.cuda_stream)
    s.set_data(x, y, sd)
    s.set_state(P0, C0)
    hostrng = np.random.default_rng(7 + rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def block(i):
        s.run_block(w["mh_steps"], 1000003 * (i + 1) + rank)

    nres = [0]

    def resample():
        if world > 1:
            # one population over all ranks: the MAP-delta cutoff over every rank's chains
            # (one all_reduce), each rank re-drawing its own chains on its device
            from gpuropolis_gb300 import population
            nres[0] += 1
            population.resample_population(s, 1, w["map_delta"], 4242 + nres[0])
            return
        P, C, prior, lik = s.get_state()
        resample_host(P, C, prior, lik, w["map_delta"], ops, hostrng)
        s.set_state(P, C)

    # warm-up blocks (untimed), then the layout autotuner on the warmed state
    for i in range(args.warmup):
        block(i)
        resample()
    tuned = None if args.no_autotune else s.autotune(steps=100, seed=4242)
    torch.cuda.synchronize()
    s.reset_stats()
    launches0 = s.launch_count()

    # device-resident timed loop: per block CUDA events around the kernel
    evs = []
    clk = ClockSampler(os.path.join(CLOCKS_DIR, "clocks_bench.csv"))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with clk:
        for i in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            block(args.warmup + i)
            e1.record(stream)
            evs.append((e0, e1))
            resample()   # state stays resident; the re-draw is outside the events
        torch.cuda.synchronize()
    kernel_ms = float(sum(a.elapsed_time(b) for a, b in evs))
    launches = s.launch_count() - launches0
    st = s.stats()
    if world > 1:
        t = torch.tensor([kernel_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        kernel_ms = float(t.item())
    chain_steps = w["N"] * w["mh_steps"] * args.steps
    value = world * chain_steps / (kernel_ms / 1e3)

    # end-to-end through the C ABI with pinned host buffers
    Ph = torch.empty((w["PL"], w["N"]), dtype=torch.int32, pin_memory=True).numpy()
    Ch = torch.empty((w["PL"], w["N"]), dtype=torch.float32, pin_memory=True).numpy()
    prh = torch.empty(w["N"], dtype=torch.float64, pin_memory=True).numpy()
    lih = torch.empty(w["N"], dtype=torch.float64, pin_memory=True).numpy()
    lib = s.lib
    ptr = lambda a: a.ctypes.data_as(g.ctypes.c_void_p)  # noqa: E731
    lib.gpr_get_state(s.h, ptr(Ph), ptr(Ch), ptr(prh), ptr(lih))
    e2e_blocks = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # the drop-in's block loop through the C ABI, as the CLI runs it with --device-resample:
    # state in from pinned host buffers, the block, the MAP-delta resampling on the device,
    # state out to pinned host buffers (where samples.txt is written from)
    for i in range(e2e_blocks):
        lib.gpr_set_state(s.h, ptr(Ph), ptr(Ch))
        lib.gpr_run_block(s.h, w["mh_steps"], 7919 * (i + 1))
        lib.gpr_resample(s.h, 1, w["map_delta"], 31 * (i + 1), None, None)
        lib.gpr_get_state(s.h, ptr(Ph), ptr(Ch), ptr(prh), ptr(lih))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * w["N"] * w["mh_steps"] * e2e_blocks / e2e_s
    h2d = Ph.nbytes + Ch.nbytes
    d2h = Ph.nbytes + Ch.nbytes + prh.nbytes + lih.nbytes

    if rank != 0:
        return
    peaks = measured_peaks()
    clocks = clk.summary(local)
    props = torch.cuda.get_device_properties(dev)
    nsm = props.multi_processor_count
    geo = s.launch_geometry()

    ess = None if args.no_ess else ess_comparison(g, stream, dev)
    cpu = None
    err = None
    if not args.no_cpu_baseline:
        # scores of the final state (after the e2e loop's device resampling, the
        # re-drawn chains' scores are the next block's to compute: evaluate them)
        prw, liw = s.evaluate()
        Pw, Cw, _, _ = s.get_state()
        rate, cores, chains, dt, kind = cpu_reference_rate(w, Pw, Cw, x, y, sd)
        cpu = {"value": rate, "unit": "chain-steps/s", "cores": cores, "kind": kind,
               "sample": "%d chains x %d MH steps of the warmed-up state (%.1f s)"
                         % (chains, w["mh_steps"], dt)}
        err = loglik_error_vs_fp64(Pw, Cw, liw, x, y, sd)
    phases = None
    if args.phase_profile:
        # one block of the same layout through its phase-timed build (untimed; same chains)
        ph = s.phase_profile(w["mh_steps"], 4711)
        cs = w["N"] * w["mh_steps"]
        tot = sum(ph["cycles"].values())
        phases = {"cycles_per_chain_step": {k: round(v / cs, 1) for k, v in ph["cycles"].items()},
                  "share": {k: round(v / tot, 4) for k, v in ph["cycles"].items()},
                  "passes_per_chain_step": ph["passes"] / cs,
                  "instructions_per_pass": ph["instructions"] / max(1, ph["passes"]),
                  "layout": s.launch_geometry(),
                  "note": "clock64 cycles of each warp between phase boundaries, summed over warps, per chain-step"}
    side = {}
    if not args.no_side:
        side["batched"] = batched_measure(args, WORKLOADS["batched-256ds-131k"], 2, 1, compare=False)
        side["streamed"] = streamed_measure(args, WORKLOADS["streamed-3var-16k"], 2, 1)
    line = {
        "metric": METRIC, "value": value, "unit": "chain-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "point_evals_per_s": value * w["nd"],
        "config": config_of(args, w),
        "parallelism": "one population over %d GPUs (resampling cutoff exchanged per block, outside the "
                       "timed region)" % world if world > 1 else "1 GPU",
        "layout": {"launch": geo, "autotuned": tuned},
        "e2e": {"value": e2e_value, "unit": "chain-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "blocks": e2e_blocks,
                "loop": "gpr_set_state (pinned host), gpr_run_block, gpr_resample (device, map-delta), "
                        "gpr_get_state (pinned host)"},
        "gpu_launches": launches,
        "roofline": fp32_roofline(st["eval_node_points"], kernel_ms / 1e3, nsm, peaks,
                                  (clocks or {}).get("sm_mhz"),
                                  MH_LAUNCH_DRAM_BYTES if args.workload == "plain-mh-131k" else None),
        "roofline_hbm": hbm_roofline(st["eval_points"], kernel_ms / 1e3, peaks,
                                     MH_LAUNCH_DRAM_BYTES if args.workload == "plain-mh-131k" else None),
        "loglik_err_vs_fp64": err,
        "precision": {"evaluation": "FP32",
                      "likelihood": "FP32 sums of 128-point chunks (<= 9 roundings), double-float across "
                                    "chunks; <= 10 u = 6.0e-7 relative to the exact sum of the FP32 terms",
                      "acceptance_ratio": "double-float from the prior difference and the difference of the "
                                          "likelihood sums (the normalising sum cancels); carries the two "
                                          "likelihoods' 10 u each",
                      "range": "weights scaled by 2^-e chosen from the data: no overflow, no posterior floor",
                      "fp64": "only when a block writes its scores"},
        "stats": st,
        "acceptance": {"structure": st["struct_accepted"] / max(1, st["struct_proposed"]),
                       "constant": st["const_accepted"] / max(1, st["const_proposed"])},
        "clocks": clocks,
        "cpu_baseline": cpu,
        "ess": ess,
        "phases": phases,
        **side,
    }
    print(json.dumps(line))


def loglik_error_vs_fp64(P, C, lik, x, y, sd, n=2048):
    """The device log-likelihoods of n chains spread over the final state
    against the oracle's FP64 evaluation of the same programs (checker only),
    on the chains whose FP32 evaluation is determined to 1e-6 (the oracle's
    FP32 restatement within 1e-6 of its FP64 one)."""
    from oracle import port
    idx = np.linspace(0, P.shape[1] - 1, n).astype(int)
    f64 = np.array([port.likelihood(P, C, int(i), x, y, sd, f64=True) for i in idx])
    f32 = np.array([port.likelihood(P, C, int(i), x, y, sd, f64=False) for i in idx])
    with np.errstate(all="ignore"):
        cond = np.abs(f32 - f64) / np.maximum(np.abs(f64), 1.0)
        e = np.abs(lik[idx] - f64) / np.maximum(np.abs(f64), 1.0)
    ok = np.isfinite(f64) & np.isfinite(lik[idx]) & (cond <= 1e-6)
    if not ok.any():
        return None
    return {"median": float(np.median(e[ok])), "max": float(e[ok].max()), "n": int(ok.sum()),
            "sampled": int(n), "invalid_agree": bool(np.all(np.isfinite(f64) | ~np.isfinite(lik[idx]) |
                                                           (cond > 1e-6)))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="plain-mh-131k", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ess", action="store_true", help="skip the constants-mixing (ESS/s) comparison")
    ap.add_argument("--ess-horizons", action="store_true",
                    help="only: the ESS estimators against run length (random walk and HMC, one JSON line)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default layout (fixed launch sequence, for profilers)")
    ap.add_argument("--phase-profile", action="store_true",
                    help="add a per-phase cycle table of one more block, from the kernel's phase-timed build")
    ap.add_argument("--no-side", action="store_true",
                    help="skip the short batched and streamed workloads reported beside the headline")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.ess_horizons:
        ess_horizons(args)
        return
    if args.workload == "hmc-rational-8k-profile":
        run_hmc_profile(args)
        return
    if args.workload in ("streamed-3var-16k", "streamed-3var-8k-profile"):
        run_streamed(args, w)
        return
    if args.workload in ("batched-256ds-131k", "batched-64ds-8k-profile"):
        run_batched(args, w)
        return
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args, w)
    else:
        run_gpu(args, w)


if __name__ == "__main__":
    main()
