"""Mixing diagnostics for traces of chain constants (host-side NumPy).

ess_geyer: effective sample size of each series by Geyer's initial monotone
sequence estimator (Geyer, "Practical Markov chain Monte Carlo", Statistical
Science 7, 1992): autocorrelations from an FFT, summed in adjacent pairs
Gamma_m = rho_2m + rho_2m+1 up to the first non-positive pair, each pair
capped by the one before it; tau = -1 + 2 sum Gamma_m, ESS = T / tau.  tau is
floored at 1 (ESS at most T), so anti-correlated chains are not credited
beyond independent draws.  A series that never moves has ESS 0.
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
