"""Multivariate data (three input variables x1, x2, x3 and the leaf ops that
read them; no reference counterpart) against the oracle's restatement
(oracle/gpr_oracle.c): program values, prior and likelihood, gradients; the
staged and streamed layouts agree exactly; a 65,536-point three-variable
dataset samples."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
port = pytest.importorskip("oracle.port")

KW = dict(n_vars=3, ops=H.OPSET_MULTI)


def _programs(N, PL, seed):
    P, C = H.random_programs(N, PL, ops=H.OPSET_MULTI, seed=seed)
    return P, C


def test_values_match_oracle():
    N, PL = 1024, 31
    P, C = _programs(N, PL, 1)
    x1, x2, x3, y, sd = H.multivar_data(64, seed=2)
    s = g.Sampler(N, program_length=PL, **KW)
    try:
        s.set_state(P, C)
        out, length, count = s.eval_values(np.stack([x1, x2, x3]))
    finally:
        s.close()
    agree = total = 0
    for idx in range(N):
        assert length[idx] == port.length(P, idx) or (np.isnan(length[idx]) and np.isnan(port.length(P, idx)))
        assert count[idx] == port.count(P, idx)
        for i in range(0, 64, 4):
            ref = port.call_nv(P, C, idx, x1[i], x2[i], x3[i])
            v = out[idx, i]
            total += 1
            if (np.isnan(ref) and np.isnan(v)) or v == ref or \
                    (np.isfinite(ref) and abs(v - ref) <= 1e-5 * max(abs(ref), 1e-3)):
                agree += 1
    assert agree >= 0.99 * total, (agree, total)


def test_prior_likelihood_match_oracle():
    N, PL = 2048, 31
    P, C = _programs(N, PL, 3)
    x1, x2, x3, y, sd = H.multivar_data(500, seed=4)
    s = g.Sampler(N, program_length=PL, **KW)
    try:
        s.set_data3(x1, x2, x3, y, sd)
        s.set_state(P, C)
        prior, lik = s.evaluate()
    finally:
        s.close()
    n_ops = len(H.OPSET_MULTI)
    good = finite = 0
    for idx in range(N):
        pr = port.prior(P, C, idx, n_ops)
        assert (np.isnan(pr) and np.isnan(prior[idx])) or abs(prior[idx] - pr) <= 1e-6 * max(1.0, abs(pr))
        l64 = port.likelihood_nv(P, C, idx, x1, x2, x3, y, sd, f64=True)
        if np.isfinite(l64):
            finite += 1
            good += bool(abs(lik[idx] - l64) <= 1e-5 * abs(l64))
    assert finite > 100 and good >= 0.95 * finite, (good, finite)


def test_gradient_matches_fp64():
    N, PL = 512, 31
    P, C = _programs(N, PL, 5)
    x1, x2, x3, y, sd = H.multivar_data(300, seed=6)
    s = g.Sampler(N, program_length=PL, **KW)
    try:
        s.set_data3(x1, x2, x3, y, sd)
        s.set_state(P, C)
        grad, lik = s.loglik_grad()
    finally:
        s.close()
    used = H.used_constants(P)
    ok = bad = 0
    for idx in range(N):
        if not np.isfinite(lik[idx]) or not used[:, idx].any():
            continue
        ll64, g64, gabs = port.loglik_grad_f64_nv(P, idx, C[:, idx].astype(np.float64), x1, x2, x3, y, sd)
        if not np.isfinite(ll64) or abs(lik[idx] - ll64) > 1e-6 * abs(ll64):
            continue
        for k in np.where(used[:, idx])[0]:
            if not (np.isfinite(g64[k]) and np.isfinite(grad[k, idx])):
                continue
            if abs(grad[k, idx] - g64[k]) <= 1e-4 * abs(g64[k]) + 2e-5 * gabs[k] + 1e-18:
                ok += 1
            else:
                bad += 1
    assert ok > 50 and bad <= 0.02 * ok, (ok, bad)


@pytest.mark.parametrize("mode", ["rw", "hmc"])
def test_streamed_equals_staged_and_large_data_samples(mode):
    N, PL = 1024, 31
    x1, x2, x3, y, sd = H.multivar_data(700, seed=8)
    P, C = g.host_init_chains(N, PL, 9, ops=H.OPSET_MULTI)
    cp = g.CONST_RANDOM_WALK if mode == "rw" else g.CONST_HMC
    res = []
    for stream in (False, True):
        s = g.Sampler(N, program_length=PL, const_proposal=cp, rw_sd=0.1, **KW)
        try:
            s.set_data3(x1, x2, x3, y, sd)
            if stream:
                s.set_streaming(True)
            if mode == "hmc":
                s.set_moves(5, 0.002, 4)
            s.set_state(P, C)
            s.run_block(25, 5)
            res.append(s.get_state())
        finally:
            s.close()
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))
    # 65,536 points only fit the streamed layout
    x1, x2, x3, y, sd = H.multivar_data(65536, seed=10)
    s = g.Sampler(256, program_length=PL, const_proposal=cp, rw_sd=0.1, **KW)
    try:
        s.set_data3(x1, x2, x3, y, sd)
        assert s.launch_geometry()["stream"] == 1
        s.set_state(*g.host_init_chains(256, PL, 11, ops=H.OPSET_MULTI))
        s.run_block(10, 1)
        st = s.stats()
        _, _, prior, lik = s.get_state()
    finally:
        s.close()
    assert st["struct_accepted"] > 0 and np.isfinite(lik).sum() > 0
