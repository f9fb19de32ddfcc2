"""The C restatement oracle (oracle/gpr_oracle.c) pinned against the
reference's own code compiled for the host (oracle/_ref): evaluator values,
description length, node count, prior, likelihood and whole MH blocks must be
bit-identical.  CPU only."""
import numpy as np
import pytest

from tests import helpers as H

oref = pytest.importorskip("oracle.ref")
from oracle import port  # noqa: E402


def _need_ref():
    if not oref.available():
        pytest.skip("reference oracle source not available")


@pytest.mark.parametrize("PL", [1, 31, 63, 255])
def test_port_folds_match_reference(PL):
    _need_ref()
    P, C = H.random_programs(300, PL, seed=21)
    o = oref.get(pl=PL, project_math=1)
    xs = np.float32([-2.5, 0.0, 0.5, 3.0, 11.0])
    for i in range(P.shape[1]):
        assert port.length(P, i) == o.length(P, C, i)
        assert port.count(P, i) == o.count_nodes(P, C, i)
        for xv in xs:
            a, b = port.call(P, C, i, xv), o.call(P, C, i, xv)
            assert (a == b) or (np.isnan(a) and np.isnan(b)), (i, xv, a, b)


@pytest.mark.parametrize("data", ["quad", "expdecay"])
def test_port_prior_likelihood_match_reference(data):
    _need_ref()
    x, y, sd = H.quad_data() if data == "quad" else H.expdecay_data()
    P, C = H.random_programs(500, 31, seed=22)
    o = oref.get(pl=31, project_math=1)
    for i in range(P.shape[1]):
        a, b = port.prior(P, C, i, 27), o.prior(P, C, i)
        assert a == b or (np.isnan(a) and np.isnan(b)), (i, a, b)
        a, b = port.likelihood(P, C, i, x, y, sd), o.likelihood(P, C, i, x, y, sd)
        assert a == b or (np.isnan(a) and np.isnan(b)), (i, a, b)


MH_CASES = [
    dict(PL=31, opset=0, rng=0, rw=0.0, pm=1),
    dict(PL=31, opset=0, rng=0, rw=0.0, pm=0),
    dict(PL=31, opset=0, rng=1, rw=0.0, pm=1),
    dict(PL=31, opset=1, rng=0, rw=0.1, pm=1),
    dict(PL=63, opset=1, rng=1, rw=0.1, pm=1),
    # program-length edges, and an empty dataset
    dict(PL=1, opset=0, rng=0, rw=0.0, pm=1),
    dict(PL=255, opset=1, rng=0, rw=0.1, pm=1),
    dict(PL=31, opset=1, rng=0, rw=0.1, pm=1, data="empty"),
]


@pytest.mark.parametrize("case", MH_CASES,
                         ids=lambda c: "pl%(PL)d-o%(opset)d-r%(rng)d-rw%(rw)g-m%(pm)d" % c + c.get("data", ""))
def test_port_mh_block_matches_reference(case):
    _need_ref()
    ops = H.OPSET_BASIC if case["opset"] else None
    if case.get("data") == "empty":
        x = y = sd = np.zeros(0, np.float32)
    else:
        x, y, sd = H.quad_data() if case["PL"] in (1, 31) else H.expdecay_data()
    P, C = H.random_programs(256, case["PL"], ops=ops, seed=23)
    o = oref.get(pl=case["PL"], opset=case["opset"], philox=case["rng"], project_math=case["pm"],
                 rw_sd=case["rw"])
    Pr, Cr = P.copy(), C.copy()
    pr_r, lk_r = o.run_kernel(Pr, Cr, x, y, sd, 40, 4242)
    c = port.cfg(case["PL"], ops=o.ops, rng=case["rng"], const_mode=1 if case["rw"] else 0,
                 rw_sd=case["rw"], project_math=case["pm"])
    Pp, Cp = P.copy(), C.copy()
    pr_p, lk_p = port.run_block(c, Pp, Cp, x, y, sd, 40, 4242)
    np.testing.assert_array_equal(Pp, Pr)
    np.testing.assert_array_equal(Cp.view(np.int32), Cr.view(np.int32))
    np.testing.assert_array_equal(pr_p, pr_r)
    np.testing.assert_array_equal(lk_p, lk_r)


@pytest.mark.parametrize("N", [1, 7, 1000, 4097])
@pytest.mark.parametrize("map_delta", [0.0, 20.0])
def test_port_resample_cutoff_matches_reference(N, map_delta):
    """The restated resampling picks the reference's cutoff and chains
    (main.cu:1215-1223, the reference's own cmp), NaN and ties included; its
    re-draws follow the Philox stream instead of rand()."""
    _need_ref()
    o = oref.get(pl=31, project_math=1, map_delta=map_delta)
    prior, lik = H.mixed_scores(N, seed=N)
    cut_ref, flags = o.resample_cutoff(prior, lik)
    P0, C0 = H.random_programs(N, 31, seed=N + 3)
    P, C = P0.copy(), C0.copy()
    mode, param = (1, map_delta) if map_delta > 0 else (0, 0.5)
    n, cut = port.resample(port.cfg(PL=31), P, C, prior, lik, mode, param, 77)
    assert (np.isnan(cut) and np.isnan(cut_ref)) or cut == cut_ref
    changed = np.any(P != P0, axis=0) | np.any(C.view(np.uint32) != C0.view(np.uint32), axis=0)
    assert n == int(flags.sum()) and np.array_equal(changed, flags)
    # re-drawn ops come from the op set minus its last op (random_int(n_ops - 1))
    assert np.all(P[:, flags] < 26)


@pytest.mark.parametrize("seed", [0, 1])
def test_port_gradient_matches_finite_differences(seed):
    """The oracle's FP64 reverse-mode gradient of the log-likelihood in the
    constants agrees with central FP64 finite differences (h = 1e-6) to 1e-4
    relative, wherever the difference quotient itself is stable."""
    x, y, sd = H.rational_data(200, seed=seed)
    P, C = H.random_programs(300, 15, seed=seed)
    used = H.used_constants(P)
    h = 1e-6
    checked = absorbed = 0
    for idx in range(P.shape[1]):
        Cd = C[:, idx].astype(np.float64)
        ll, g, _ = port.loglik_grad_f64(P, idx, Cd, x, y, sd)
        if not np.isfinite(ll):
            continue
        for k in np.where(used[:, idx])[0]:
            def fd(step):
                a, b = Cd.copy(), Cd.copy()
                a[k] += step
                b[k] -= step
                return (port.loglik_f64(P, idx, a, x, y, sd) - port.loglik_f64(P, idx, b, x, y, sd)) / (2 * step)
            f1, f2 = fd(h), fd(h / 2)
            if not (np.isfinite(f1) and np.isfinite(f2)):
                continue
            if abs(f1 - f2) > 1e-5 * max(abs(f1), 1e-6 * (abs(ll) + 1)):
                continue                      # the difference quotient is not stable here
            if np.isnan(g[k]):
                # a finite value computed through a NaN subexpression (pow(NaN, 0) = 1)
                # has no derivative through it; the chain rule yields NaN there
                absorbed += 1
                continue
            assert abs(g[k] - f1) <= 1e-4 * max(abs(f1), 1e-6 * (abs(ll) + 1)), (idx, k, g[k], f1)
            checked += 1
    assert checked >= 50 and absorbed <= 0.05 * checked, (checked, absorbed)


def test_rational_program_reads_its_five_constants():
    b, _ = H.rational_coefficients(0)
    x, y, sd = H.rational_data(200, seed=0)
    P, C = H.rational_program(1, b)
    assert sorted(np.where(H.used_constants(P)[:, 0])[0] + 1) == sorted(H.RATIONAL_NODES)
    f = np.array([port.call_f64(P, C, 0, v) for v in x])
    want = (b[0] + b[1] * x + b[2] * x ** 2) / (1 + b[3] * x + b[4] * x ** 2)
    assert np.allclose(f, want, rtol=1e-5, atol=1e-6)


def test_resample_segments_restates_resample_per_dataset():
    """The per-dataset restatement: one segment is the plain resample; with
    several, each segment's cutoff is the rank rule over its own chains and
    only its own chains below it are re-drawn (streams keyed by the global
    chain index)."""
    N, PL, nseg = 400, 31, 4
    P, C = H.random_programs(N, PL, ops=H.OPSET_BASIC, seed=1)
    prior, lik = H.mixed_scores(N, seed=3)
    c = port.cfg(PL=PL, ops=H.OPSET_BASIC)
    P1, C1 = P.copy(), C.copy()
    n1, cut1 = port.resample(c, P1, C1, prior, lik, 0, 0.5, 9)
    P2, C2 = P.copy(), C.copy()
    n2, cuts2 = port.resample_segments(c, P2, C2, prior, lik, 1, 0, 0.5, 9)
    assert n1 == n2 and cut1 == cuts2[0] and np.array_equal(P1, P2) and np.array_equal(C1, C2)
    for mode, param in ((0, 0.3), (1, 5.0)):
        P3, C3 = P.copy(), C.copy()
        n3, cuts3 = port.resample_segments(c, P3, C3, prior, lik, nseg, mode, param, 9)
        seg = N // nseg
        post = prior + lik
        total = 0
        for d in range(nseg):
            s = post[d * seg:(d + 1) * seg]
            srt = np.concatenate([s[np.isnan(s)], np.sort(s[~np.isnan(s)])])
            want = srt[-1] - param if mode == 1 else srt[int(seg * param)]
            assert (np.isnan(want) and np.isnan(cuts3[d])) or want == cuts3[d]
            below = s < cuts3[d]
            total += int(below.sum())
            changed = ~np.all(P3[:, d * seg:(d + 1) * seg] == P[:, d * seg:(d + 1) * seg], axis=0)
            assert not (changed & ~below).any()
        assert n3 == total
