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
NOPS_REFERENCE = 27
PROGRAM_CODE = "1CIab+-_#*@/|LE^pVPRSsCcTtA"   # main.cu:55

OPSET_REFERENCE = list(range(27))
# {+, -, *, /, exp, log, pow, x, const}: x reached through the A/B pass-throughs
OPSET_BASIC = [CONST, A, B, PLUS, MINUS, TIMES, DIV, LOG, EXP, POW]

RNG_LCG, RNG_PHILOX = 0, 1
CONST_REFERENCE, CONST_RANDOM_WALK = 0, 1

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
                ("reserved", ctypes.c_int * 8)]


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
    lib.gpr_get_stats.argtypes = [vp, vp, ip]
    lib.gpr_reset_stats.argtypes = [vp]
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def make_config(program_length=31, ops=None, rng=RNG_LCG, const_proposal=CONST_REFERENCE,
                rw_sd=0.1, device=0, stream=None):
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

    def set_state(self, P, C):
        P = np.ascontiguousarray(P, np.int32).reshape(self.PL, self.N)
        C = np.ascontiguousarray(C, np.float32).reshape(self.PL, self.N)
        self._check(self.lib.gpr_set_state(self.h, _ptr(P), _ptr(C)))

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
        xs = np.ascontiguousarray(xs, np.float32)
        out = np.empty((self.N, len(xs)), np.float32)
        length = np.empty(self.N, np.float32)
        count = np.empty(self.N, np.int32)
        self._check(self.lib.gpr_debug_eval_values(self.h, _ptr(xs), len(xs), _ptr(out),
                                                   _ptr(length), _ptr(count)))
        return out, length, count

    def launch_geometry(self):
        v = [ctypes.c_int() for _ in range(4)] + [ctypes.c_int64()]
        self._check(self.lib.gpr_launch_geometry(self.h, *[ctypes.byref(a) for a in v]))
        return dict(K=v[0].value, onepass=v[1].value, warps_per_cta=v[2].value,
                    ctas=v[3].value, smem_bytes=v[4].value)

    STAT_NAMES = ("evals", "eval_nodes", "eval_points", "eval_node_points", "struct_proposed",
                  "struct_accepted", "const_proposed", "const_accepted")

    def stats(self):
        out = np.zeros(8, np.uint64)
        self._check(self.lib.gpr_get_stats(self.h, _ptr(out), 8))
        return dict(zip(self.STAT_NAMES, (int(v) for v in out)))

    def reset_stats(self):
        self._check(self.lib.gpr_reset_stats(self.h))

    def launch_count(self):
        return int(self.lib.gpr_launch_count(self.h))

    def stream(self):
        return self.lib.gpr_stream(self.h)
