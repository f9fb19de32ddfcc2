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


@pytest.mark.parametrize("PL", [31, 63])
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
]


@pytest.mark.parametrize("case", MH_CASES, ids=lambda c: "pl%(PL)d-o%(opset)d-r%(rng)d-rw%(rw)g-m%(pm)d" % c)
def test_port_mh_block_matches_reference(case):
    _need_ref()
    ops = H.OPSET_BASIC if case["opset"] else None
    x, y, sd = H.quad_data() if case["PL"] == 31 else H.expdecay_data()
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
