"""ctypes view of the C restatement oracle (oracle/gpr_oracle.c).
TEST INFRASTRUCTURE ONLY."""
import ctypes

import numpy as np

from . import build_port


class PortCfg(ctypes.Structure):
    _fields_ = [("program_length", ctypes.c_int), ("n_ops", ctypes.c_int), ("ops", ctypes.c_int * 32),
                ("rng", ctypes.c_int), ("const_mode", ctypes.c_int), ("rw_sd", ctypes.c_float),
                ("project_math", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build_port.build())
        vp, ip, fp, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
        L.gpr_port_eval.argtypes = [vp, vp, ip, ip, ip, fp]
        L.gpr_port_eval.restype = fp
        L.gpr_port_eval_f64.argtypes = [vp, vp, ip, ip, ip, dp]
        L.gpr_port_eval_f64.restype = dp
        L.gpr_port_eval_f64_perturbed.argtypes = [vp, vp, ip, ip, ip, dp, ctypes.c_uint, dp]
        L.gpr_port_eval_f64_perturbed.restype = dp
        L.gpr_port_length.argtypes = [vp, ip, ip, ip]
        L.gpr_port_length.restype = fp
        L.gpr_port_count.argtypes = [vp, ip, ip, ip]
        L.gpr_port_prior.argtypes = [vp, vp, ip, ip, ip, ip]
        L.gpr_port_prior.restype = dp
        L.gpr_port_likelihood.argtypes = [vp, vp, ip, ip, ip, vp, ip]
        L.gpr_port_likelihood.restype = dp
        L.gpr_port_likelihood_f64.argtypes = [vp, vp, ip, ip, ip, vp, ip]
        L.gpr_port_likelihood_f64.restype = dp
        L.gpr_port_run_block.argtypes = [ctypes.POINTER(PortCfg), ip, ip, ip, vp, vp, vp, ip, ip, vp, vp, ip, ip]
        L.gpr_port_run_block_trace.argtypes = [ctypes.POINTER(PortCfg), ip, vp, vp, vp, ip, ip, vp, vp, ip, vp, ip]
        L.gpr_port_loglik_f64d.argtypes = [vp, ip, ip, ip, vp, vp, ip]
        L.gpr_port_loglik_f64d.restype = dp
        L.gpr_port_loglik_grad_f64.argtypes = [vp, ip, ip, ip, vp, vp, ip, vp, vp]
        L.gpr_port_loglik_grad_f64.restype = dp
        L.gpr_port_loglik_grad_f64p.argtypes = [vp, ip, ip, ip, vp, vp, ip, vp, ctypes.c_uint, dp]
        L.gpr_port_loglik_grad_f64p.restype = dp
        L.gpr_port_call_nv.argtypes = [vp, vp, ip, ip, ip, fp, fp, fp]
        L.gpr_port_call_nv.restype = fp
        L.gpr_port_likelihood_nv.argtypes = [vp, vp, ip, ip, ip, vp, ip, ip]
        L.gpr_port_likelihood_nv.restype = dp
        L.gpr_port_loglik_grad_f64_nv.argtypes = [vp, ip, ip, ip, vp, vp, ip, vp, vp]
        L.gpr_port_loglik_grad_f64_nv.restype = dp
        L.gpr_port_resample.argtypes = [ctypes.POINTER(PortCfg), ip, vp, vp, vp, vp, ip, dp, ctypes.c_uint, vp]
        L.gpr_port_resample_segments.argtypes = [ctypes.POINTER(PortCfg), ip, ip, vp, vp, vp, vp, ip, dp,
                                                 ctypes.c_uint, vp]
        assert L.gpr_port_sizeof_cfg() == ctypes.sizeof(PortCfg)
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def pack(x, y, sd):
    d = np.empty((len(x), 3), np.float32)
    d[:, 0], d[:, 1], d[:, 2] = x, y, sd
    return np.ascontiguousarray(d)


def cfg(PL=31, ops=None, rng=0, const_mode=0, rw_sd=0.1, project_math=1):
    c = PortCfg()
    c.program_length = PL
    ops = list(range(27)) if ops is None else list(ops)
    c.n_ops = len(ops)
    for i, o in enumerate(ops):
        c.ops[i] = o
    c.rng, c.const_mode, c.rw_sd, c.project_math = rng, const_mode, rw_sd, project_math
    return c


def run_block(c, P, C, x, y, sd, steps, seed, nthreads=0, chains=None):
    PL, N = P.shape
    assert P.dtype == np.int32 and C.dtype == np.float32 and P.flags.c_contiguous and C.flags.c_contiguous
    D = pack(x, y, sd)
    prior = np.zeros(N)
    lik = np.zeros(N)
    c0, c1 = chains if chains else (0, N)
    lib().gpr_port_run_block(ctypes.byref(c), N, c0, c1, _p(P), _p(C), _p(D), len(x), steps, _p(prior),
                             _p(lik), int(seed), nthreads)
    return prior, lik


def run_block_trace(c, P, C, x, y, sd, steps, seed, nthreads=0):
    """run_block over all chains, also returning trace[N, steps, 8] =
    (proposal posterior, current posterior, acceptance, uniform or -1, accepted,
    conditioning of the proposal's and of the current FP32 log-likelihood)."""
    PL, N = P.shape
    D = pack(x, y, sd)
    prior = np.zeros(N)
    lik = np.zeros(N)
    tr = np.zeros((N, max(steps, 1), 8))
    lib().gpr_port_run_block_trace(ctypes.byref(c), N, _p(P), _p(C), _p(D), len(x), steps, _p(prior), _p(lik),
                                   int(seed), _p(tr), nthreads)
    return prior, lik, tr


def call(P, C, idx, x):
    return lib().gpr_port_eval(_p(P), _p(C), P.shape[1], P.shape[0], idx, float(x))


def call_f64(P, C, idx, x):
    return lib().gpr_port_eval_f64(_p(P), _p(C), P.shape[1], P.shape[0], idx, float(x))


def sensitivity(P, C, idx, x, rel=2.0 ** -22, trials=6):
    """max |f_perturbed - f| over `trials` FP64 evaluations with every node's
    result jittered by up to `rel` (relative): the FP32 noise floor of this
    program at x.  inf when a perturbation changes finiteness."""
    base = call_f64(P, C, idx, x)
    worst = 0.0
    for t in range(trials):
        v = lib().gpr_port_eval_f64_perturbed(_p(P), _p(C), P.shape[1], P.shape[0], idx, float(x), 977 * t + 1, rel)
        if np.isfinite(v) != np.isfinite(base):
            return np.inf
        if np.isfinite(v):
            worst = max(worst, abs(v - base))
    return worst


def length(P, idx):
    return lib().gpr_port_length(_p(P), P.shape[1], P.shape[0], idx)


def count(P, idx):
    return lib().gpr_port_count(_p(P), P.shape[1], P.shape[0], idx)


def prior(P, C, idx, n_ops):
    return lib().gpr_port_prior(_p(P), _p(C), P.shape[1], P.shape[0], idx, n_ops)


def likelihood(P, C, idx, x, y, sd, f64=False):
    D = pack(x, y, sd)
    f = lib().gpr_port_likelihood_f64 if f64 else lib().gpr_port_likelihood
    return f(_p(P), _p(C), P.shape[1], P.shape[0], idx, _p(D), len(x))


def resample(c, P, C, prior, lik, mode, param, seed):
    """In-place re-draw of the chains below the cutoff with the device's
    random stream; returns (number re-drawn, cutoff)."""
    PL, N = P.shape
    assert P.dtype == np.int32 and C.dtype == np.float32 and P.flags.c_contiguous and C.flags.c_contiguous
    prior = np.ascontiguousarray(prior, np.float64)
    lik = np.ascontiguousarray(lik, np.float64)
    cut = ctypes.c_double()
    n = lib().gpr_port_resample(ctypes.byref(c), N, _p(P), _p(C), _p(prior), _p(lik), mode, param, seed,
                                ctypes.byref(cut))
    return n, cut.value


def resample_segments(c, P, C, prior, lik, nseg, mode, param, seed):
    """resample per dataset of a batched handle: chains [d*N/nseg, (d+1)*N/nseg)
    against their own cutoff; returns (number re-drawn, cutoffs)."""
    PL, N = P.shape
    assert P.dtype == np.int32 and C.dtype == np.float32 and P.flags.c_contiguous and C.flags.c_contiguous
    prior = np.ascontiguousarray(prior, np.float64)
    lik = np.ascontiguousarray(lik, np.float64)
    cuts = np.zeros(nseg, np.float64)
    n = lib().gpr_port_resample_segments(ctypes.byref(c), N, nseg, _p(P), _p(C), _p(prior), _p(lik), mode,
                                         param, seed, _p(cuts))
    return n, cuts


def loglik_f64(P, idx, Cd, x, y, sd):
    """FP64 log-likelihood of chain idx with constants Cd (PL doubles)."""
    PL, N = P.shape
    D = pack(x, y, sd)
    Cd = np.ascontiguousarray(Cd, np.float64)
    return lib().gpr_port_loglik_f64d(_p(P), N, PL, idx, _p(Cd), _p(D), len(x))


def loglik_grad_f64(P, idx, Cd, x, y, sd):
    """(FP64 log-likelihood, d loglik / d Cd, sum of |per-point terms|) of chain idx."""
    PL, N = P.shape
    D = pack(x, y, sd)
    Cd = np.ascontiguousarray(Cd, np.float64)
    g = np.zeros(PL)
    ga = np.zeros(PL)
    ll = lib().gpr_port_loglik_grad_f64(_p(P), N, PL, idx, _p(Cd), _p(D), len(x), _p(g), _p(ga))
    return ll, g, ga


def grad_sensitivity(P, idx, Cd, x, y, sd, rel=2.0 ** -22, trials=4):
    """max over trials of |g_perturbed - g| per constant: the FP32 noise floor
    of the log-likelihood gradient (inf where a jitter changes finiteness)."""
    PL, N = P.shape
    D = pack(x, y, sd)
    Cd = np.ascontiguousarray(Cd, np.float64)
    _, g0, _ = loglik_grad_f64(P, idx, Cd, x, y, sd)
    worst = np.zeros(PL)
    for t in range(trials):
        g = np.zeros(PL)
        lib().gpr_port_loglik_grad_f64p(_p(P), N, PL, idx, _p(Cd), _p(D), len(x), _p(g), 977 * t + 1, rel)
        with np.errstate(invalid="ignore"):
            d = np.where(np.isfinite(g) == np.isfinite(g0), np.abs(g - g0), np.inf)
        worst = np.maximum(worst, np.nan_to_num(d, nan=np.inf))
    return worst


def pack5(x1, x2, x3, y, sd):
    d = np.empty((len(x1), 5), np.float32)
    d[:, 0], d[:, 1], d[:, 2], d[:, 3], d[:, 4] = x1, x2, x3, y, sd
    return np.ascontiguousarray(d)


def call_nv(P, C, idx, x1, x2, x3):
    """FP32 value of chain idx at one multivariate point."""
    return lib().gpr_port_call_nv(_p(P), _p(C), P.shape[1], P.shape[0], idx, x1, x2, x3)


def likelihood_nv(P, C, idx, x1, x2, x3, y, sd, f64=False):
    D = pack5(x1, x2, x3, y, sd)
    return lib().gpr_port_likelihood_nv(_p(P), _p(C), P.shape[1], P.shape[0], idx, _p(D), len(x1), int(f64))


def loglik_grad_f64_nv(P, idx, Cd, x1, x2, x3, y, sd):
    """(FP64 log-likelihood, d loglik / d Cd, sum of |per-point terms|), multivariate."""
    PL, N = P.shape
    D = pack5(x1, x2, x3, y, sd)
    Cd = np.ascontiguousarray(Cd, np.float64)
    g = np.zeros(PL)
    ga = np.zeros(PL)
    ll = lib().gpr_port_loglik_grad_f64_nv(_p(P), N, PL, idx, _p(Cd), _p(D), len(x1), _p(g), _p(ga))
    return ll, g, ga
