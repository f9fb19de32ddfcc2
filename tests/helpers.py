"""Seeded synthetic inputs shared by the tests and bench.py.

Datasets follow the workload descriptions the sampler is measured on (no
public dataset is involved): a noisy quadratic, an exponential decay, a
rational function and a 3-variable sin/exp surface, all float32.
"""
import numpy as np

OPSET_BASIC = [1, 3, 4, 5, 6, 9, 11, 13, 14, 15]   # CONST A B + - * / log exp pow


def quad_data(n=101, seed=0):
    """x ~ U[0,10], y = 2.5x^2 - 1.3x + 0.7 + N(0, 0.1), sd = 0.1."""
    r = np.random.default_rng(seed)
    x = r.uniform(0, 10, n).astype(np.float32)
    y = (2.5 * x.astype(np.float64) ** 2 - 1.3 * x + 0.7 + r.normal(0, 0.1, n)).astype(np.float32)
    sd = np.full(n, 0.1, np.float32)
    return x, y, sd


def expdecay_data(n=250, seed=0):
    """x ~ U[0,50], y = b1 exp(-b2 x) + b3, b1~U(50,150), b2~U(.01,.2),
    b3~U(-5,5), noise N(0, 0.05 std(y)); sd = the noise sd."""
    r = np.random.default_rng(seed)
    x = r.uniform(0, 50, n)
    b1, b2, b3 = r.uniform(50, 150), r.uniform(0.01, 0.2), r.uniform(-5, 5)
    y0 = b1 * np.exp(-b2 * x) + b3
    s = 0.05 * np.std(y0)
    y = y0 + r.normal(0, s, n)
    return x.astype(np.float32), y.astype(np.float32), np.full(n, s, np.float32)


def random_programs(N, PL, ops=None, seed=0, shallow_frac=0.5):
    """Chains in the reference layout (PL, N).  Ops are drawn like the
    reference's initialisation (op index < n_ops-1, main.cu:1133); a fraction
    of chains is cut to a random depth with CONST/A/B below it so that many
    programs are small and finite.  Constants are 10^U{-4..3} * N(0,1)
    (main.cu:1134-1137)."""
    r = np.random.default_rng(seed)
    ops = np.arange(27) if ops is None else np.asarray(ops)
    P = ops[r.integers(0, max(1, len(ops) - 1), size=(PL, N))].astype(np.int32)
    depth = np.floor(np.log2(np.arange(1, PL + 1))).astype(int)
    nshallow = int(N * shallow_frac)
    for c in range(nshallow):
        d0 = r.integers(1, 4)
        leafy = np.array([1, 3, 4], np.int32)
        sel = depth >= d0
        P[sel, c] = leafy[r.integers(0, 3, size=sel.sum())]
    C = (10.0 ** r.integers(-4, 4, size=(PL, N)) * r.normal(size=(PL, N))).astype(np.float32)
    return np.ascontiguousarray(P), np.ascontiguousarray(C)


def rel_err(a, b, floor=1.0):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def same_class(a, b):
    """Both finite, or both the same non-finite value class (nan / +inf / -inf)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    both_nan = np.isnan(a) & np.isnan(b)
    same_inf = (~fa) & (~fb) & (a == b)
    return (fa & fb) | both_nan | same_inf


def mixed_scores(N, seed, nan=0.05, ninf=0.05, ties=True):
    """(prior, likelihood) per chain whose sums cover the cases the
    resampling comparator orders specially: NaN, -inf, ties, signed zeros."""
    r = np.random.default_rng(seed)
    post = -np.abs(r.normal(0, 1e3, N)) * 10.0 ** r.integers(-3, 4, N)
    if ties:
        post[r.integers(0, N, N // 10)] = -12.5
        post[r.integers(0, N, 3)] = 0.0
        post[r.integers(0, N, 3)] = -0.0
    post[r.random(N) < ninf] = -np.inf
    prior = np.zeros(N)
    prior[r.random(N) < nan] = np.nan
    return prior, post.copy()
