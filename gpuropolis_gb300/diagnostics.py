"""Mixing diagnostics for traces of chain constants (host-side NumPy).

ess_geyer: effective sample size of each series by Geyer's initial monotone
sequence estimator (Geyer, "Practical Markov chain Monte Carlo", Statistical
Science 7, 1992): autocorrelations from an FFT, summed in adjacent pairs
Gamma_m = rho_2m + rho_2m+1 up to the first non-positive pair, each pair
capped by the one before it; tau = -1 + 2 sum Gamma_m, ESS = T / tau.  tau is
floored at 1 (ESS at most T), so anti-correlated chains are not credited
beyond independent draws.  A series that never moves has ESS 0.

ess_population: the effective sample size per chain of a population of
independent chains that all start at stationarity and share one target (as
after a burn-in of copies of one model): the autocorrelation at lag k is the
mean over chains and time of (x_t - mu)(x_t+k - mu) / sigma^2, with mu and
sigma^2 the pooled mean and variance of all draws and each lag normalised by
its own number of pairs, then Geyer's initial monotone sequence as above.
Centering on the pooled mean instead of each chain's own keeps a run that is
short against the autocorrelation time from being credited with more
independent draws than it holds: per chain, the chain's own mean soaks up its
slow drift and ess_geyer then overestimates (on AR(1) series of length 1.5
tau it reports about 4x the true ESS; this estimator stays within 10%).
"""
import numpy as np


def ess_geyer(X):
    """ESS of each row of X (n_series, T)."""
    X = np.asarray(X, np.float64)
    n, T = X.shape
    Xc = X - X.mean(axis=1, keepdims=True)
    var = (Xc ** 2).mean(axis=1)
    f = np.fft.rfft(Xc, n=2 * T, axis=1)
    acov = np.fft.irfft(f * np.conj(f), n=2 * T, axis=1)[:, :T] / T
    rho = acov / np.maximum(acov[:, :1], 1e-300)
    m = T // 2
    gam = rho[:, 0:2 * m:2] + rho[:, 1:2 * m:2]
    pos = gam > 0
    first = np.where(pos.all(axis=1), m, np.argmin(pos, axis=1))
    keep = np.arange(m)[None, :] < first[:, None]
    mono = np.minimum.accumulate(np.where(keep, gam, 0.0), axis=1)
    tau = -1.0 + 2.0 * np.sum(np.where(keep, mono, 0.0), axis=1)
    ess = T / np.maximum(tau, 1.0)
    ess[var <= 0] = 0.0
    return ess


def chain_ess(trace, used):
    """Per chain, the smallest ESS over the constants it reads.
    trace: (N, T, n) constants after each step; used: (n, N) bool."""
    N, T, n = trace.shape
    out = np.zeros(N)
    for c0 in range(0, N, 1024):
        c1 = min(N, c0 + 1024)
        X = np.ascontiguousarray(trace[c0:c1].transpose(0, 2, 1)).reshape(-1, T)
        e = ess_geyer(X).reshape(c1 - c0, n)
        e = np.where(used[:, c0:c1].T, e, np.inf)
        m = e.min(axis=1)
        out[c0:c1] = np.where(np.isfinite(m), m, 0.0)
    return out


def _geyer_tau(rho):
    """tau = -1 + 2 sum of Geyer's initial monotone pair sums of rho (1-D),
    floored at 1."""
    m = len(rho) // 2
    gam = rho[0:2 * m:2] + rho[1:2 * m:2]
    pos = gam > 0
    first = m if pos.all() else int(np.argmin(pos))
    mono = np.minimum.accumulate(gam[:first]) if first > 0 else np.zeros(0)
    return max(1.0, -1.0 + 2.0 * float(mono.sum()))


def ess_population(X):
    """ESS per chain of X (m_chains, T), chains independent and stationary
    with one target: T / tau, tau from the pooled autocorrelation.  0 if no
    chain moves; the sum behind tau spans at most the run, so a population
    that barely moves reads about 0.5, the estimator's resolution."""
    X = np.asarray(X, np.float64)
    m, T = X.shape
    if m < 2 or T < 4:
        raise ValueError("need at least 2 chains of 4 draws")
    mu = X.mean()
    var = X.var()
    if not var > 0 or not np.any(X != X[:, :1]):
        return 0.0
    Xc = X - mu
    acc = np.zeros(T)
    for c0 in range(0, m, 512):                      # bounded FFT memory
        f = np.fft.rfft(Xc[c0:c0 + 512], n=2 * T, axis=1)
        acc += np.fft.irfft(f * np.conj(f), n=2 * T, axis=1)[:, :T].sum(axis=0)
    rho = acc / (m * (T - np.arange(T)) * var)
    return T / _geyer_tau(rho)


def population_ess(trace, used):
    """The smallest population ESS per chain over the constants that every
    traced chain reads (trace: (N, T, n); used: (n, N) bool)."""
    N, T, n = trace.shape
    cols = [i for i in range(n) if used[i, :N].all()]
    if not cols:
        return 0.0
    return min(ess_population(np.ascontiguousarray(trace[:, :, i])) for i in cols)
