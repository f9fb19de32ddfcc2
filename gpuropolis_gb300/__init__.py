"""gpuropolis_gb300 -- GB300-native Metropolis-Hastings sampler over arithmetic
expressions (the sampling loop of GPUropolis's main.cu, re-built for sm_103a).

The product is the C ABI in include/gpuropolis.h, implemented by
_lib/libgpuropolis.so (CUDA kernels + host library), and the `gpuropolis`
command-line tool beside it.  This module is a thin ctypes binding used by the
tests and bench.py.  It fails loudly when the library has not been built:
there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgpuropolis.so")
CLI_PATH = os.path.join(_HERE, "_lib", "gpuropolis")

# op codes, reference numbering (main.cu:53)
(ONE, CONST, INV, A, B, PLUS, MINUS, RMINUS, CPLUS, TIMES, CTIMES, DIV, RDIV, LOG, EXP, POW,
 CPOW, RPOW, CRPOW, SQRT, SIN, ASIN, COS, ACOS, TAN, ATAN, ABS) = range(27)
X1, X2, X3 = 27, 28, 29          # input variables of multivariate data (no reference counterpart)
NOPS_REFERENCE = 27
PROGRAM_CODE = "1CIab+-_#*@/|LE^pVPRSsCcTtAXYZ"   # main.cu:55, then the variable leaves

OPSET_REFERENCE = list(range(27))
# {+, -, *, /, exp, log, pow, x, const}: x reached through the A/B pass-throughs
OPSET_BASIC = [CONST, A, B, PLUS, MINUS, TIMES, DIV, LOG, EXP, POW]

RNG_LCG, RNG_PHILOX = 0, 1
CONST_REFERENCE, CONST_RANDOM_WALK, CONST_HMC = 0, 1, 2

GPR_OK = 0
ERRORS = {1: "GPR_ERR_ARG", 2: "GPR_ERR_CUDA", 3: "GPR_ERR_STATE", 4: "GPR_ERR_DEVICE",
          5: "GPR_ERR_NOMEM"}


class GprError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("program_length", ctypes.c_int), ("n_ops", ctypes.c_int),
                ("ops", ctypes.c_int * 32), ("rng", ctypes.c_int),
                ("const_proposal", ctypes.c_int), ("rw_sd", ctypes.c_float),
                ("device", ctypes.c_int), ("stream", ctypes.c_void_p),
                ("n_vars", ctypes.c_int), ("reserved", ctypes.c_int * 7)]


_lib = None


def library():
    """Load libgpuropolis.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libgpuropolis.so is not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    vp, ip, fp, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
    P = ctypes.POINTER
    lib.gpr_default_config.argtypes = [P(Config)]
    lib.gpr_default_config.restype = None
    lib.gpr_create.argtypes = [P(Config), ip, P(vp)]
    lib.gpr_destroy.argtypes = [vp]
    lib.gpr_set_data.argtypes = [vp, vp, vp, vp, ip]
    lib.gpr_set_data3.argtypes = [vp, vp, vp, vp, vp, vp, ip]
    lib.gpr_set_state.argtypes = [vp, vp, vp]
    lib.gpr_get_state.argtypes = [vp, vp, vp, vp, vp]
    lib.gpr_run_block.argtypes = [vp, ip, ip]
    lib.gpr_evaluate.argtypes = [vp]
    lib.gpr_sync.argtypes = [vp]
    lib.gpr_device_state.argtypes = [vp, vp, vp, vp, vp]
    lib.gpr_launch_count.argtypes = [vp]
    lib.gpr_launch_count.restype = ctypes.c_int64
    lib.gpr_last_error.argtypes = [vp]
    lib.gpr_last_error.restype = ctypes.c_char_p
    lib.gpr_version.restype = ctypes.c_char_p
    lib.gpr_debug_eval_values.argtypes = [vp, vp, ip, vp, vp, vp]
    lib.gpr_launch_geometry.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.gpr_stream.argtypes = [vp]
    lib.gpr_stream.restype = vp
    lib.gpr_debug_math.argtypes = [vp, ip, vp, vp, vp, ip]
    lib.gpr_debug_phase_profile.argtypes = [vp, ip, ip, vp, ip]
    lib.gpr_debug_stage_wait.argtypes = [vp, ip]
    lib.gpr_debug_fp_issue.argtypes = [ip, ip, vp, vp, vp]
    lib.gpr_autotune.argtypes = [vp, ip, ip, vp, vp, vp, vp]
    lib.gpr_set_layout.argtypes = [vp, ip, ip, ip]
    lib.gpr_layout_rolled.argtypes = [vp]
    lib.gpr_layout_lockstep.argtypes = [vp]
    lib.gpr_set_layout2.argtypes = [vp, ip, ip, ip, ip, ip]
    lib.gpr_set_layout3.argtypes = [vp, ip, ip, ip, ip, ip, ip]
    lib.gpr_layout_pipelined.argtypes = [vp]
    lib.gpr_get_stats.argtypes = [vp, vp, ip]
    lib.gpr_reset_stats.argtypes = [vp]
    lib.gpr_set_scores.argtypes = [vp, vp, vp]
    lib.gpr_set_moves.argtypes = [vp, ip, fp, ip]
    lib.gpr_set_hmc_jitter.argtypes = [vp, fp, fp]
    lib.gpr_run_block_traced_first.argtypes = [vp, ip, ip, ip, ip, vp]
    lib.gpr_set_hmc_layout.argtypes = [vp, ip, ip]
    lib.gpr_set_streaming.argtypes = [vp, ip]
    lib.gpr_layout_streamed.argtypes = [vp]
    lib.gpr_adapt_scales.argtypes = [vp, fp]
    lib.gpr_chain_scales.argtypes = [vp, vp]
    lib.gpr_loglik_grad.argtypes = [vp, vp, vp]
    lib.gpr_run_block_traced.argtypes = [vp, ip, ip, ip, vp]
    lib.gpr_set_batched_data.argtypes = [vp, ip, vp, vp, vp, vp, vp, vp]
    lib.gpr_resample_datasets.argtypes = [vp, ip, dp, ctypes.c_uint32, vp, vp]
    lib.gpr_resample_below.argtypes = [vp, dp, ctypes.c_uint32, ip, vp]
    lib.gpr_capture_blocks.argtypes = [vp, ip, ip]
    lib.gpr_run_captured.argtypes = [vp, vp]
    lib.gpr_resample.argtypes = [vp, ip, dp, ctypes.c_uint32, vp, vp]
    lib.gpr_top_chains.argtypes = [vp, ip, dp, vp, ip, vp, vp]
    lib.gpr_map_chain.argtypes = [vp, vp, vp]
    # host side (include/gpuropolis_host.h)
    lib.gpr_load_data_file.argtypes = [ctypes.c_char_p, fp, ip, ip, P(vp), P(vp), P(vp), P(ip)]
    lib.gpr_load_data_file3.argtypes = [ctypes.c_char_p, fp, ip, ip, P(vp), P(vp), P(vp), P(vp), P(vp), P(ip)]
    lib.gpr_free.argtypes = [vp]
    lib.gpr_host_last_error.restype = ctypes.c_char_p
    lib.gpr_format_expression.argtypes = [vp, vp, ip, ip, ip, ctypes.c_char_p, ip, ctypes.c_char_p, ip]
    lib.gpr_program_length_of.argtypes = [vp, vp, ip, ip, ip]
    lib.gpr_program_length_of.restype = fp
    lib.gpr_polynomial_degree.argtypes = [vp, vp, ip, ip, ip]
    lib.gpr_polynomial_degree.restype = fp
    lib.gpr_format_samples.argtypes = [vp, vp, vp, vp, ip, ip, ip, ip, ip, P(vp)]
    lib.gpr_format_samples.restype = ctypes.c_int64
    lib.gpr_host_srand.argtypes = [ctypes.c_uint]
    lib.gpr_host_init_chains.argtypes = [vp, vp, ip, ip, vp, ip]
    lib.gpr_host_resample.argtypes = [vp, vp, vp, vp, ip, ip, vp, ip, ip, ctypes.c_double]
    lib.gpr_tops_new.argtypes = [ip]
    lib.gpr_tops_new.restype = vp
    lib.gpr_tops_free.argtypes = [vp]
    lib.gpr_tops_add_text.argtypes = [vp, ctypes.c_char_p, ctypes.c_int64]
    lib.gpr_tops_add_lines.argtypes = [vp, ctypes.c_char_p, ctypes.c_int64, vp, ip]
    lib.gpr_tops_write.argtypes = [vp, ctypes.c_char_p]
    lib.gpr_tops_write.restype = ctypes.c_int64
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def fp_issue_times(device=0, iters=4096):
    """(ms FP64 adds on all lanes, ms FP64 adds on one lane per warp, ms FP32
    adds on all lanes) of the same work on the device."""
    lib = library()
    v = [ctypes.c_float() for _ in range(3)]
    rc = lib.gpr_debug_fp_issue(device, iters, *[ctypes.byref(a) for a in v])
    if rc != GPR_OK:
        raise GprError(rc, lib.gpr_last_error(None).decode())
    return tuple(a.value for a in v)


def make_config(program_length=31, ops=None, rng=RNG_LCG, const_proposal=CONST_REFERENCE,
                rw_sd=0.1, device=0, stream=None, n_vars=1):
    lib = library()
    cfg = Config()
    lib.gpr_default_config(ctypes.byref(cfg))
    cfg.program_length = program_length
    ops = OPSET_REFERENCE if ops is None else list(ops)
    cfg.n_ops = len(ops)
    for i, o in enumerate(ops):
        cfg.ops[i] = o
    cfg.rng = rng
    cfg.const_proposal = const_proposal
    cfg.rw_sd = rw_sd
    cfg.device = device
    cfg.stream = stream
    cfg.n_vars = n_vars
    return cfg


class Sampler:
    """One handle of the C ABI: N chains of programs with program_length heap nodes."""

    def __init__(self, n_chains, **cfg_kwargs):
        self.lib = library()
        self.cfg = make_config(**cfg_kwargs)
        self.N = n_chains
        self.PL = self.cfg.program_length
        h = ctypes.c_void_p()
        rc = self.lib.gpr_create(ctypes.byref(self.cfg), n_chains, ctypes.byref(h))
        if rc != GPR_OK:
            raise GprError(rc, self.lib.gpr_last_error(None).decode())
        self.h = h

    def _check(self, rc):
        if rc != GPR_OK:
            raise GprError(rc, self.lib.gpr_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.gpr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_data(self, x, y, sd):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        sd = np.ascontiguousarray(sd, np.float32)
        self._check(self.lib.gpr_set_data(self.h, _ptr(x), _ptr(y), _ptr(sd), len(x)))

    def set_data3(self, x1, x2, x3, y, sd):
        a = [np.ascontiguousarray(v, np.float32) for v in (x1, x2, x3, y, sd)]
        self._check(self.lib.gpr_set_data3(self.h, *[_ptr(v) for v in a], len(a[0])))

    def set_batched_data(self, datasets):
        """datasets: a list of (x, y, sd) or, for three variables, of
        (x1, x2, x3, y, sd); chain c fits dataset c // (N // len(datasets))."""
        sizes = np.array([len(d[0]) for d in datasets], np.int32)
        ncol = 5 if self.cfg.n_vars == 3 else 3
        cat = [np.ascontiguousarray(np.concatenate([np.asarray(d[i], np.float32) for d in datasets])
                                    if datasets else np.zeros(0), np.float32) for i in range(ncol)]
        x1, x2, x3, y, sd = cat if ncol == 5 else (cat[0], None, None, cat[1], cat[2])
        self._check(self.lib.gpr_set_batched_data(self.h, len(datasets), _ptr(sizes), _ptr(x1), _ptr(x2),
                                                  _ptr(x3), _ptr(y), _ptr(sd)))

    def capture_blocks(self, n_blocks, steps):
        self._check(self.lib.gpr_capture_blocks(self.h, int(n_blocks), int(steps)))
        self._captured = int(n_blocks)

    def run_captured(self, seeds):
        seeds = np.ascontiguousarray(seeds, np.int32)
        if len(seeds) != getattr(self, "_captured", len(seeds)):
            raise GprError(1, f"{len(seeds)} seeds for {self._captured} captured blocks")
        self._check(self.lib.gpr_run_captured(self.h, _ptr(seeds)))

    def set_state(self, P, C):
        P = np.ascontiguousarray(P, np.int32).reshape(self.PL, self.N)
        C = np.ascontiguousarray(C, np.float32).reshape(self.PL, self.N)
        self._check(self.lib.gpr_set_state(self.h, _ptr(P), _ptr(C)))

    def get_scores(self):
        """(prior, likelihood) of every chain, without the programs."""
        prior = np.empty(self.N, np.float64)
        lik = np.empty(self.N, np.float64)
        self._check(self.lib.gpr_get_state(self.h, None, None, _ptr(prior), _ptr(lik)))
        return prior, lik

    def get_state(self):
        P = np.empty((self.PL, self.N), np.int32)
        C = np.empty((self.PL, self.N), np.float32)
        prior = np.empty(self.N, np.float64)
        lik = np.empty(self.N, np.float64)
        self._check(self.lib.gpr_get_state(self.h, _ptr(P), _ptr(C), _ptr(prior), _ptr(lik)))
        return P, C, prior, lik

    def run_block(self, steps, seed):
        self._check(self.lib.gpr_run_block(self.h, int(steps), int(seed)))

    def evaluate(self):
        self._check(self.lib.gpr_evaluate(self.h))
        _, _, prior, lik = self.get_state()
        return prior, lik

    def sync(self):
        self._check(self.lib.gpr_sync(self.h))

    def eval_values(self, xs):
        """Program values at points xs: shape (nx,), or (3, nx) for three variables."""
        xs = np.ascontiguousarray(xs, np.float32)
        nx = xs.shape[-1]
        out = np.empty((self.N, nx), np.float32)
        length = np.empty(self.N, np.float32)
        count = np.empty(self.N, np.int32)
        self._check(self.lib.gpr_debug_eval_values(self.h, _ptr(xs), nx, _ptr(out),
                                                   _ptr(length), _ptr(count)))
        return out, length, count

    def math(self, op, a, b=None):
        """The evaluator's exp ('exp'), log ('log') or pow ('pow') on the GPU."""
        code = {"exp": 0, "log": 1, "pow": 2}[op]
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(a if b is None else b, np.float32)
        out = np.empty_like(a)
        self._check(self.lib.gpr_debug_math(self.h, code, _ptr(a), _ptr(b), _ptr(out), len(a)))
        return out

    PHASE_NAMES = ("claim", "load", "step_barrier", "structure_proposal", "constant_proposal", "compile",
                   "cauchy_prior", "eval_program", "barrier1", "rank", "evaluation", "barrier2", "combine",
                   "accept", "store")

    def phase_profile(self, steps, seed):
        """One block of MH steps through the phase-timed build of the current
        layout (same results as run_block): clock64 cycles per phase summed
        over warps, plus the evaluation passes and program instructions
        interpreted."""
        out = np.zeros(len(self.PHASE_NAMES) + 2, np.uint64)
        self._check(self.lib.gpr_debug_phase_profile(self.h, int(steps), int(seed), _ptr(out), len(out)))
        d = {n: int(v) for n, v in zip(self.PHASE_NAMES, out)}
        return {"cycles": d, "passes": int(out[-2]), "instructions": int(out[-1])}

    def set_stage_wait(self, polls):
        """Polls of the staging barrier before a kernel gives up (testing)."""
        self._check(self.lib.gpr_debug_stage_wait(self.h, int(polls)))

    def autotune(self, steps=50, seed=1):
        """Pick the fastest evaluation layout on the current state and data."""
        k, op, ro = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = ctypes.c_float()
        self._check(self.lib.gpr_autotune(self.h, steps, seed, ctypes.byref(k), ctypes.byref(op),
                                          ctypes.byref(ro), ctypes.byref(ms)))
        return dict(K=k.value, onepass=op.value, rolled=ro.value, ms=ms.value)

    def set_layout(self, K, onepass, rolled, lockstep=1, warps_per_cta=8, pipe=0):
        """pipe=1: the pipelined kernel (two chains per warp); otherwise the
        lockstep kernel with CTA barriers every `lockstep` steps (0: none)."""
        self._check(self.lib.gpr_set_layout3(self.h, K, int(onepass), int(rolled), lockstep, warps_per_cta,
                                             int(pipe)))

    def launch_geometry(self):
        v = [ctypes.c_int() for _ in range(4)] + [ctypes.c_int64()]
        self._check(self.lib.gpr_launch_geometry(self.h, *[ctypes.byref(a) for a in v]))
        return dict(K=v[0].value, onepass=v[1].value, warps_per_cta=v[2].value,
                    ctas=v[3].value, smem_bytes=v[4].value, rolled=int(self.lib.gpr_layout_rolled(self.h)),
                    lockstep=int(self.lib.gpr_layout_lockstep(self.h)),
                    pipe=int(self.lib.gpr_layout_pipelined(self.h)),
                    stream=int(self.lib.gpr_layout_streamed(self.h)))

    STAT_NAMES = ("evals", "eval_nodes", "eval_points", "eval_node_points", "struct_proposed",
                  "struct_accepted", "const_proposed", "const_accepted")

    def stats(self):
        out = np.zeros(8, np.uint64)
        self._check(self.lib.gpr_get_stats(self.h, _ptr(out), 8))
        return dict(zip(self.STAT_NAMES, (int(v) for v in out)))

    def reset_stats(self):
        self._check(self.lib.gpr_reset_stats(self.h))

    def set_moves(self, struct_every=5, hmc_eps=0.01, hmc_steps=8):
        self._check(self.lib.gpr_set_moves(self.h, int(struct_every), float(hmc_eps), int(hmc_steps)))

    def set_hmc_jitter(self, eps_frac=0.0, len_frac=0.0):
        """Per-move jitter of the Hamiltonian trajectories: step x U(1 -
        eps_frac, 1 + eps_frac), leapfrog count uniform in [L(1 - len_frac),
        L(1 + len_frac)]."""
        self._check(self.lib.gpr_set_hmc_jitter(self.h, float(eps_frac), float(len_frac)))

    def set_streaming(self, always=True):
        self._check(self.lib.gpr_set_streaming(self.h, int(bool(always))))

    def set_hmc_layout(self, warps_per_cta=4, ctas_per_sm=0):
        self._check(self.lib.gpr_set_hmc_layout(self.h, int(warps_per_cta), int(ctas_per_sm)))

    def adapt_scales(self, target_accept):
        self._check(self.lib.gpr_adapt_scales(self.h, float(target_accept)))

    def chain_scales(self):
        out = np.empty(self.N, np.float32)
        self._check(self.lib.gpr_chain_scales(self.h, _ptr(out)))
        return out

    def loglik_grad(self):
        """(grad (PL, N) float64, likelihood (N,) float64) of the current state."""
        grad = np.empty((self.PL, self.N), np.float64)
        lik = np.empty(self.N, np.float64)
        self._check(self.lib.gpr_loglik_grad(self.h, _ptr(grad), _ptr(lik)))
        return grad, lik

    def run_block_traced(self, steps, seed, trace_n, chains=None):
        """run_block, returning the first trace_n constants after every step:
        an array (chains, steps, trace_n) of the first `chains` chains (all
        N by default; every chain steps either way)."""
        n = self.N if chains is None else int(chains)
        tr = np.empty((n, steps, trace_n), np.float32)
        self._check(self.lib.gpr_run_block_traced_first(self.h, int(steps), int(seed), int(trace_n), n, _ptr(tr)))
        return tr

    def set_scores(self, prior, lik):
        prior = np.ascontiguousarray(prior, np.float64)
        lik = np.ascontiguousarray(lik, np.float64)
        assert prior.shape == (self.N,) and lik.shape == (self.N,)
        self._check(self.lib.gpr_set_scores(self.h, _ptr(prior), _ptr(lik)))

    def resample(self, mode=0, param=0.5, seed=1):
        """Device resampling (gpr_resample): returns (chains re-drawn, cutoff)."""
        n, cut = ctypes.c_int(), ctypes.c_double()
        self._check(self.lib.gpr_resample(self.h, int(mode), float(param), int(seed) & 0xffffffff,
                                          ctypes.byref(n), ctypes.byref(cut)))
        return n.value, cut.value

    def resample_below(self, cutoff, seed=1, chain_offset=0):
        """Re-draw the chains below an explicit cutoff (gpr_resample_below);
        returns the number re-drawn."""
        n = ctypes.c_int()
        self._check(self.lib.gpr_resample_below(self.h, float(cutoff), int(seed) & 0xffffffff, int(chain_offset),
                                                ctypes.byref(n)))
        return n.value

    def resample_datasets(self, n_datasets, mode=0, param=0.5, seed=1):
        """Per-dataset device resampling (gpr_resample_datasets): returns
        (chains re-drawn, cutoffs, one per dataset)."""
        n = ctypes.c_int()
        cuts = np.zeros(max(1, int(n_datasets)), np.float64)
        self._check(self.lib.gpr_resample_datasets(self.h, int(mode), float(param), int(seed) & 0xffffffff,
                                                   ctypes.byref(n), _ptr(cuts)))
        return n.value, cuts

    def top_chains(self, k, margin=0.0, capacity=None):
        """Candidate chains for the k best (gpr_top_chains): (chains, count, threshold)."""
        capacity = self.N if capacity is None else capacity
        out = np.empty(max(capacity, 1), np.int32)
        n, t = ctypes.c_int(), ctypes.c_double()
        self._check(self.lib.gpr_top_chains(self.h, int(k), float(margin), _ptr(out), capacity,
                                            ctypes.byref(n), ctypes.byref(t)))
        return out[:min(n.value, capacity)].copy(), n.value, t.value

    def map_chain(self):
        """(MAP chain index, its posterior) (gpr_map_chain)."""
        c, v = ctypes.c_int(), ctypes.c_double()
        self._check(self.lib.gpr_map_chain(self.h, ctypes.byref(c), ctypes.byref(v)))
        return c.value, v.value

    def launch_count(self):
        return int(self.lib.gpr_launch_count(self.h))

    def stream(self):
        return self.lib.gpr_stream(self.h)


# ---- host-side helpers (CPU only; no GPU needed) ---------------------------

def load_data_file(path, sdscale=1.0, first_half=False, even_half=False):
    """The reference's data loader (main.cu:319-363); raises on errors."""
    lib = library()
    px, py, ps = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    n = ctypes.c_int()
    rc = lib.gpr_load_data_file(path.encode(), sdscale, int(first_half), int(even_half),
                                ctypes.byref(px), ctypes.byref(py), ctypes.byref(ps), ctypes.byref(n))
    if rc != 0:
        raise GprError(rc, lib.gpr_host_last_error().decode(errors="replace"))
    out = []
    for p in (px, py, ps):
        a = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)), shape=(max(n.value, 1),))
        out.append(a[:n.value].copy())
        lib.gpr_free(p)
    return tuple(out)



def load_data_file3(path, sdscale=1.0, first_half=False, even_half=False):
    """Data with three input variables, lines "x1 x2 x3 y sd" (the reference's
    loader rules, main.cu:319-363); returns (x1, x2, x3, y, sd)."""
    lib = library()
    ptrs = [ctypes.c_void_p() for _ in range(5)]
    n = ctypes.c_int()
    rc = lib.gpr_load_data_file3(path.encode(), sdscale, int(first_half), int(even_half),
                                 *[ctypes.byref(p) for p in ptrs], ctypes.byref(n))
    if rc != 0:
        raise GprError(rc, lib.gpr_host_last_error().decode(errors="replace"))
    out = []
    for p in ptrs:
        a = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)), shape=(max(n.value, 1),))
        out.append(a[:n.value].copy())
        lib.gpr_free(p)
    return tuple(out)

def format_expression(P, C, idx, cfmt="C", latex=False):
    lib = library()
    P = np.ascontiguousarray(P, np.int32)
    C = np.ascontiguousarray(C, np.float32)
    PL, N = P.shape
    n = lib.gpr_format_expression(_ptr(P), _ptr(C), N, PL, idx, cfmt.encode(), int(latex), None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    lib.gpr_format_expression(_ptr(P), _ptr(C), N, PL, idx, cfmt.encode(), int(latex), buf, n + 1)
    return buf.value.decode("latin-1")


def program_length_of(P, C, idx):
    P = np.ascontiguousarray(P, np.int32)
    C = np.ascontiguousarray(C, np.float32)
    return library().gpr_program_length_of(_ptr(P), _ptr(C), P.shape[1], P.shape[0], idx)


def polynomial_degree(P, C, idx):
    P = np.ascontiguousarray(P, np.int32)
    C = np.ascontiguousarray(C, np.float32)
    return library().gpr_polynomial_degree(_ptr(P), _ptr(C), P.shape[1], P.shape[0], idx)


def format_samples(P, C, prior, lik, block, show_constants=False, nthreads=0):
    lib = library()
    P = np.ascontiguousarray(P, np.int32)
    C = np.ascontiguousarray(C, np.float32)
    prior = np.ascontiguousarray(prior, np.float64)
    lik = np.ascontiguousarray(lik, np.float64)
    out = ctypes.c_void_p()
    n = lib.gpr_format_samples(_ptr(P), _ptr(C), _ptr(prior), _ptr(lik), P.shape[1], P.shape[0],
                               block, int(show_constants), nthreads, ctypes.byref(out))
    if n < 0:
        raise GprError(1, "gpr_format_samples failed")
    s = ctypes.string_at(out, n).decode("latin-1")
    lib.gpr_free(out)
    return s


def host_init_chains(N, PL, seed, ops=None):
    """srand(seed) then the reference's initial state (main.cu:1107,1133-1137)."""
    lib = library()
    ops = np.ascontiguousarray(OPSET_REFERENCE if ops is None else ops, np.int32)
    P = np.empty((PL, N), np.int32)
    C = np.empty((PL, N), np.float32)
    lib.gpr_host_srand(seed)
    lib.gpr_host_init_chains(_ptr(P), _ptr(C), N, PL, _ptr(ops), len(ops))
    return P, C


def host_resample(P, C, prior, lik, ops=None, mode=0, param=0.5):
    """In-place resampling (main.cu:1216-1231); continues the current rand() stream."""
    lib = library()
    ops = np.ascontiguousarray(OPSET_REFERENCE if ops is None else ops, np.int32)
    prior = np.ascontiguousarray(prior, np.float64)
    lik = np.ascontiguousarray(lik, np.float64)
    return lib.gpr_host_resample(_ptr(P), _ptr(C), _ptr(prior), _ptr(lik), P.shape[1], P.shape[0],
                                 _ptr(ops), len(ops), mode, param)


class Tops:
    """The k lines `LC_ALL=C sort -g -k3 | tail -n k` keeps (gpr_tops_*)."""

    def __init__(self, k):
        self.lib = library()
        self.t = self.lib.gpr_tops_new(int(k))
        if not self.t:
            raise GprError(1, "k must be >= 1")

    def add_text(self, text):
        b = text.encode("latin-1") if isinstance(text, str) else text
        if self.lib.gpr_tops_add_text(self.t, b, len(b)) != 0:
            raise GprError(1, "gpr_tops_add_text failed")

    def add_lines(self, text, lines):
        b = text.encode("latin-1") if isinstance(text, str) else text
        lines = np.ascontiguousarray(lines, np.int32)
        if self.lib.gpr_tops_add_lines(self.t, b, len(b), _ptr(lines), len(lines)) != 0:
            raise GprError(1, "gpr_tops_add_lines failed")

    def write(self, path):
        n = self.lib.gpr_tops_write(self.t, path.encode())
        if n < 0:
            raise GprError(1, "gpr_tops_write failed")
        return n

    def close(self):
        if self.t:
            self.lib.gpr_tops_free(self.t)
            self.t = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
