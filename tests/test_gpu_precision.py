"""Precision of the device log-likelihood and acceptance ratio, stage by stage.

The evaluation is FP32; the likelihood's per-point terms (f - y)^2 w are
summed in FP32 within a 128-point chunk (four fused multiply-adds per lane,
then a five-level butterfly: at most nine roundings, every term >= 0, so the
chunk sum is within 9 u = 9 * 2^-24 of its exact value, relatively); the
chunk sums are added as double-floats in chunk order (error about 2^-47 of
the running sum per chunk: 4e-12 relative at 512 chunks); the weight
w = 2^-e/(2 sd^2) is the float nearest to the exact one (one more u).  So
against the reference's double sum of the same FP32 residuals
(main.cu:454-468) the quadratic part of the likelihood is within 10 u = 6.0e-7
relative, whatever the number of points.  The prior and the acceptance ratio
((proposal - current) + backward) - forward (main.cu:728, 790) are
double-floats formed from the prior difference and the difference of the two
likelihood sums (the normalising sum cancels), so the ratio carries the two
likelihoods' 10 u each and nothing measurable besides; FP64 -- on GB300 one
warp-wide FP64 add costs about 64 FP32 adds of issue time -- is used only
when a block writes its scores.  The weight's scale 2^-e is chosen from the
data so that no sum can overflow: posteriors are valid over the reference's
whole range (there is no floor at -6e57)."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
port = pytest.importorskip("oracle.port")

U = 2.0 ** -24
CHUNK_BOUND = 10 * U          # chunk sums (9 u) + the weight's rounding (1 u)


def _const_programs(N, PL, values):
    """Chains whose program is the single constant C[0] (op CONST at the root)."""
    P = np.full((PL, N), 1, np.int32)          # CONST everywhere; only the root is reachable
    C = np.zeros((PL, N), np.float32)
    C[0] = values
    return P, C


def _exact_quadratic(values, y, sd):
    """sum_d q_d / (2 sd_d^2) with q_d = fl32(fl32(c - y_d)^2), the reference's
    FP32 residual squared, summed exactly (math.fsum of the double terms)."""
    import math
    out = []
    y32, sd64 = y.astype(np.float32), sd.astype(np.float64)
    for c in values:
        r = (np.float32(c) - y32).astype(np.float32)
        q = (r * r).astype(np.float32).astype(np.float64)
        out.append(math.fsum(q / (2.0 * sd64 * sd64)))
    return np.array(out)


@pytest.mark.parametrize("nd", [250, 65536])
def test_accumulation_stage_within_its_bound(nd):
    """Constant programs evaluate exactly, so the whole difference from the
    exact sum is the accumulation: within CHUNK_BOUND relative at 250 points
    (cfg1's size) and at 65,536 (512 chunks)."""
    N, PL = 64, 31
    r = np.random.default_rng(nd)
    x = r.uniform(0, 50, nd).astype(np.float32)
    y = (100 * np.exp(-0.05 * x) + r.normal(0, 1, nd)).astype(np.float32)
    sd = r.uniform(0.5, 2.0, nd).astype(np.float32)
    values = np.concatenate([[0.0], r.uniform(-20, 120, N - 1)]).astype(np.float32)
    P, C = _const_programs(N, PL, values)
    s = g.Sampler(N, program_length=PL)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        _, lik = s.evaluate()
    finally:
        s.close()
    ns = float(np.sum(0.5 * (np.float64(np.log(np.float32(2 * 3.141592653589))) +
                             2.0 * np.log(sd).astype(np.float32).astype(np.float64))))
    quad_dev = -(lik + ns)            # the device's quadratic part (ns is exact to ~1e-16)
    quad = _exact_quadratic(values, y, sd)
    rel = np.abs(quad_dev - quad) / quad
    assert rel.max() <= CHUNK_BOUND * (1 + 1e-6) + 1e-12, (rel.max(), CHUNK_BOUND)
    print("nd %d: accumulation error median %.2e max %.2e (bound %.2e)" % (nd, np.median(rel), rel.max(),
                                                                            CHUNK_BOUND))


def test_loglik_error_vs_fp64_at_65536_points():
    """Whole programs on 65,536 points: within 1e-5 relative of the FP64
    evaluation wherever the program's own FP32 evaluation is determined to
    1e-6 (the FP32 restatement within 1e-6 of FP64)."""
    N, PL = 256, 31
    r = np.random.default_rng(8)
    n = 65536
    x = r.uniform(0, 50, n).astype(np.float32)
    y = (80 * np.exp(-0.07 * x) + 3 + r.normal(0, 0.5, n)).astype(np.float32)
    sd = np.full(n, 0.5, np.float32)
    P, C = H.random_programs(N, PL, ops=H.OPSET_BASIC, seed=12)
    s = g.Sampler(N, program_length=PL, ops=H.OPSET_BASIC)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        _, lik = s.evaluate()
    finally:
        s.close()
    f64 = np.array([port.likelihood(P, C, i, x, y, sd, f64=True) for i in range(N)])
    f32 = np.array([port.likelihood(P, C, i, x, y, sd, f64=False) for i in range(N)])
    with np.errstate(all="ignore"):
        cond = np.abs(f32 - f64) / np.maximum(np.abs(f64), 1.0)
        err = np.abs(lik - f64) / np.maximum(np.abs(f64), 1.0)
    ok = np.isfinite(f64) & (cond <= 1e-6)
    assert ok.sum() >= 20, ok.sum()
    assert np.all(np.isfinite(lik[ok]))
    assert err[ok].max() <= 1e-5, err[ok].max()
    print("65536 points: loglik error vs FP64 (%d chains): median %.2e max %.2e"
          % (ok.sum(), np.median(err[ok]), err[ok].max()))


def test_posterior_has_no_floor():
    """sd = 1e-30: every term -(r^2)/(2 sd^2) with |r| >= 1 is beyond 5e59 in
    the reference's double (main.cu:300), so every likelihood is beyond the
    -6e57 a fixed 2^-64 scale could hold; the device keeps them valid and
    equal to the FP64 value within 1e-5."""
    N, PL = 256, 31
    x, y, _ = H.quad_data(101, seed=2)
    sd = np.full(x.size, 1e-30, np.float32)
    P, C = H.random_programs(N, PL, ops=H.OPSET_BASIC, seed=5, shallow_frac=1.0)
    s = g.Sampler(N, program_length=PL, ops=H.OPSET_BASIC)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        _, lik = s.evaluate()
    finally:
        s.close()
    f64 = np.array([port.likelihood(P, C, i, x, y, sd, f64=True) for i in range(N)])
    f32 = np.array([port.likelihood(P, C, i, x, y, sd, f64=False) for i in range(N)])
    with np.errstate(all="ignore"):
        cond = np.abs(f32 - f64) / np.abs(f64)
        err = np.abs(lik - f64) / np.abs(f64)
    big = np.isfinite(f64) & (np.abs(f64) > 1e58) & (cond <= 1e-6)
    assert big.sum() >= 10, big.sum()
    assert np.all(np.isfinite(lik[big]))
    assert err[big].max() <= 1e-5, err[big].max()
