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


def rational_coefficients(seed=0):
    """b_i ~ N(0, 1), redrawn until 1 + b4 x + b5 x^2 stays above 0.2 on [-3, 3]."""
    r = np.random.default_rng(seed)
    grid = np.linspace(-3, 3, 601)
    while True:
        b = r.normal(0, 1, 5)
        if np.min(1 + b[3] * grid + b[4] * grid ** 2) > 0.2:
            return b, r


def rational_data(n=1024, seed=0):
    """x ~ U[-3, 3], y = (b1 + b2 x + b3 x^2) / (1 + b4 x + b5 x^2) + N(0, 0.02)
    with b from rational_coefficients(seed); sd = 0.02."""
    b, r = rational_coefficients(seed)
    x = r.uniform(-3, 3, n)
    y = (b[0] + b[1] * x + b[2] * x ** 2) / (1 + b[3] * x + b[4] * x ** 2) + r.normal(0, 0.02, n)
    return x.astype(np.float32), y.astype(np.float32), np.full(n, 0.02, np.float32)


# heap nodes (1-based) of the constants of rational_program, in b order
RATIONAL_NODES = (2, 9, 18, 15, 30)


def rational_program(N, b, PL=31):
    """N copies of (b1 + x (b2 + b3 x)) / (1 + x (b4 + b5 x)) as heap programs:
    node 1 DIV(2, 3); 2 CPLUS b1 over 4 TIMES(8, 9), 8 A -> 16 A -> x,
    9 CPLUS b2 over 18 CTIMES b3 over x; 3 PLUS(6, 7), 6 ONE, 7 TIMES(14, 15),
    14 A -> 28 A -> x, 15 CPLUS b4 over 30 CTIMES b5 over x.  Unreachable nodes
    are ONE with constant 0."""
    assert PL == 31
    P = np.zeros((PL, N), np.int32)
    C = np.zeros((PL, N), np.float32)
    ops = {1: 11, 2: 8, 4: 9, 8: 3, 16: 3, 9: 8, 18: 10, 3: 5, 6: 0, 7: 9, 14: 3, 28: 3, 15: 8, 30: 10}
    for j, o in ops.items():
        P[j - 1] = o
    for j, v in zip(RATIONAL_NODES, b):
        C[j - 1] = v
    return P, C


def used_constants(P):
    """Mask (PL, N): the constants each program reads -- CONST leaves and the
    constant ops (+C, *C, ^C, C^), reachable from the root through the A/B
    pass-throughs."""
    PL, N = P.shape
    used = np.zeros((PL, N), bool)
    reach = np.zeros((PL + 1, N), bool)
    reach[1] = True
    for j in range(1, PL + 1):
        o = P[j - 1]
        r = reach[j]
        used[j - 1] = r & np.isin(o, (1, 8, 10, 16, 18))
        unary = np.isin(o, (2, 8, 10, 13, 14, 16, 18, 19, 20, 21, 22, 23, 24, 25, 26))
        binary = np.isin(o, (5, 6, 7, 9, 11, 12, 15, 17))
        for child, m in ((2 * j, np.isin(o, (3,)) | unary | binary), (2 * j + 1, np.isin(o, (4,)) | binary)):
            if child <= PL:
                reach[child] |= r & m
    return used


# {+, -, *, /, sin, cos, exp, const, x1, x2, x3} and the A/B pass-throughs
OPSET_MULTI = [1, 3, 4, 5, 6, 9, 11, 20, 22, 27, 28, 29, 14]


def multivar_data(n=65536, seed=0):
    """x1, x2, x3 ~ N(0, 1); y = sin(x1) x2 + exp(-x3^2) + N(0, 0.05); sd 0.05."""
    r = np.random.default_rng(seed)
    x1, x2, x3 = r.normal(0, 1, (3, n))
    y = np.sin(x1) * x2 + np.exp(-x3 ** 2) + r.normal(0, 0.05, n)
    f = lambda a: a.astype(np.float32)  # noqa: E731
    return f(x1), f(x2), f(x3), f(y), np.full(n, 0.05, np.float32)
