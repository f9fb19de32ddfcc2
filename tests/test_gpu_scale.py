"""Parity at the benchmarked configuration: 131,072 chains, PROGRAM_LENGTH 63,
250 points of the exponential-decay data, ops {+,-,*,/,exp,log,pow,x,const},
random-walk constants (sd 0.1), one block of 1000 MH steps through the layout
the autotuner picks -- the run bench.py times.

  * the final states of 4,096 chains spread over the population are scored by
    the reference's own compute_prior / compute_likelihood (main.cu:529-544,
    454-468, compiled for the host) and by an FP64 restatement: 1e-5 relative,
    judged wherever the program's FP32 evaluation is determined to 1e-6;
  * the final log-posteriors and node counts of 1,024 chains agree in
    distribution with the reference's own MH code run from the same states
    with another seed (two-sample Kolmogorov-Smirnov, p > 1e-3)."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
oref = pytest.importorskip("oracle.ref")
port = pytest.importorskip("oracle.port")

N, PL, ND, STEPS = 131072, 63, 250, 1000


def _need_ref():
    if not oref.available():
        pytest.skip("reference oracle source not available")


@pytest.fixture(scope="module")
def cfg1_run():
    x, y, sd = H.expdecay_data(ND, seed=2024)
    P0, C0 = H.random_programs(N, PL, ops=H.OPSET_BASIC, seed=99, shallow_frac=0.0)
    s = g.Sampler(N, program_length=PL, ops=H.OPSET_BASIC, rng=g.RNG_LCG, const_proposal=g.CONST_RANDOM_WALK,
                  rw_sd=0.1)
    try:
        s.set_data(x, y, sd)
        s.set_state(P0, C0)
        s.run_block(200, 7)                     # move off the initial state before tuning
        tuned = s.autotune(steps=50, seed=4242)
        geo = s.launch_geometry()
        s.run_block(STEPS, 12345)
        P, C, prior, lik = s.get_state()
    finally:
        s.close()
    return dict(x=x, y=y, sd=sd, P=P, C=C, prior=prior, lik=lik, geo=geo, tuned=tuned)


def test_scores_at_scale_match_reference_and_fp64(cfg1_run):
    _need_ref()
    r = cfg1_run
    P, C, x, y, sd = r["P"], r["C"], r["x"], r["y"], r["sd"]
    idx = np.linspace(0, N - 1, 4096).astype(int)
    o = oref.get(pl=PL, opset=1, project_math=1, rw_sd=0.1)
    rprior = np.array([o.prior(P, C, int(i)) for i in idx])
    rlik = np.array([o.likelihood(P, C, int(i), x, y, sd) for i in idx])
    f64 = np.array([port.likelihood(P, C, int(i), x, y, sd, f64=True) for i in idx])
    prior, lik = r["prior"][idx], r["lik"][idx]
    assert np.all(H.same_class(prior, rprior))
    fin = np.isfinite(rprior)
    assert H.rel_err(prior[fin], rprior[fin]).max() <= 1e-5
    with np.errstate(all="ignore"):
        cond = np.abs(rlik - f64) / np.maximum(np.abs(f64), 1.0)
        err_ref = np.abs(lik - rlik) / np.maximum(np.abs(rlik), 1.0)
        err64 = np.abs(lik - f64) / np.maximum(np.abs(f64), 1.0)
    judged = np.isfinite(f64) & np.isfinite(rlik) & (cond <= 1e-6)
    assert judged.sum() > 1000, judged.sum()
    assert np.all(np.isfinite(lik[judged]))
    assert err_ref[judged].max() <= 1e-5, err_ref[judged].max()
    assert err64[judged].max() <= 1e-5, err64[judged].max()
    # validity agrees wherever FP32 rounding cannot decide it
    edge = ~np.isfinite(f64) | (cond > 1e-6)
    assert np.all(H.same_class(lik, rlik) | edge)
    print("cfg1 at scale (%s): %d chains judged; loglik error vs FP64 median %.2e max %.2e"
          % (r["geo"], judged.sum(), np.median(err64[judged]), err64[judged].max()))


def test_posterior_distribution_at_pl63_matches_reference(cfg1_run):
    """KS agreement after 1000 further steps from the same 1,024 states
    (spread over the population), the device and the reference's code with
    different seeds."""
    _need_ref()
    from scipy import stats
    r = cfg1_run
    x, y, sd = r["x"], r["y"], r["sd"]
    idx = np.linspace(0, N - 1, 1024).astype(int)
    P, C = np.ascontiguousarray(r["P"][:, idx]), np.ascontiguousarray(r["C"][:, idx])
    M = len(idx)
    s = g.Sampler(M, program_length=PL, ops=H.OPSET_BASIC, rng=g.RNG_LCG, const_proposal=g.CONST_RANDOM_WALK,
                  rw_sd=0.1)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        s.run_block(STEPS, 2468)
        Pg, Cg, prior_g, lik_g = s.get_state()
        _, _, count_g = s.eval_values(x[:1])
    finally:
        s.close()
    o = oref.get(pl=PL, opset=1, project_math=1, rw_sd=0.1)
    Pr, Cr = P.copy(), C.copy()
    prior_r, lik_r = o.run_kernel(Pr, Cr, x, y, sd, STEPS, 1357)
    count_r = np.array([o.count_nodes(Pr, Cr, i) for i in range(M)])
    post_g, post_r = prior_g + lik_g, prior_r + lik_r
    fin_g, fin_r = post_g[np.isfinite(post_g)], post_r[np.isfinite(post_r)]
    assert len(fin_g) > M // 4 and len(fin_r) > M // 4, (len(fin_g), len(fin_r))
    ks = stats.ks_2samp(fin_g, fin_r)
    assert ks.pvalue > 1e-3, (ks, np.median(fin_g), np.median(fin_r))
    kc = stats.ks_2samp(count_g, count_r)
    assert kc.pvalue > 1e-3, kc
