"""Device-side selection over chain posteriors (gpr_resample.cu) against the
oracle: the resampling cutoff of main.cu:1215-1219 under the reference's
comparator (NaN lowest, main.cu:987-995), the re-draw of the chains below it
(main.cu:1221-1229) with the device's Philox stream -- programs and constants
bit-exact against the C restatement (oracle/gpr_oracle.c) -- the top-k
candidates behind tops.txt and the MAP chain."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
port = pytest.importorskip("oracle.port")


def _sorted_ref(post):
    """The reference comparator's ascending order: NaN first."""
    return np.concatenate([post[np.isnan(post)], np.sort(post[~np.isnan(post)])])


@pytest.mark.parametrize("N", [1, 2, 7, 1000, 65537])
@pytest.mark.parametrize("mode,param", [(0, 0.5), (0, 0.0), (0, 0.9), (1, 20.0), (1, 0.0)])
def test_resample_matches_oracle(N, mode, param):
    PL = 31
    P0, C0 = H.random_programs(N, PL, seed=N)
    prior, lik = H.mixed_scores(N, seed=N + 1)
    s = g.Sampler(N, program_length=PL)
    try:
        s.set_state(P0, C0)
        s.set_scores(prior, lik)
        n_dev, cut_dev = s.resample(mode, param, seed=12345 + N)
        P1, C1, _, _ = s.get_state()
    finally:
        s.close()
    P2, C2 = P0.copy(), C0.copy()
    n_ref, cut_ref = port.resample(port.cfg(PL=PL), P2, C2, prior, lik, mode, param, 12345 + N)
    assert (np.isnan(cut_dev) and np.isnan(cut_ref)) or cut_dev == cut_ref, (cut_dev, cut_ref)
    post = prior + lik
    expect = _sorted_ref(post)[N - 1] - param if mode == 1 else _sorted_ref(post)[int(N * param)]
    assert (np.isnan(expect) and np.isnan(cut_dev)) or expect == cut_dev
    assert n_dev == n_ref == int(np.sum(post < cut_ref))
    assert np.array_equal(P1, P2)
    assert np.array_equal(C1.view(np.uint32), C2.view(np.uint32))
    # untouched chains keep their state
    keep = ~(post < cut_ref)
    assert np.array_equal(P1[:, keep], P0[:, keep]) and np.array_equal(C1[:, keep], C0[:, keep])


def test_resample_after_mh_block_matches_oracle():
    """On a state the device scored itself: one MH block, then the device
    resample equals the oracle's resample of the same scores."""
    N, PL = 4096, 31
    x, y, sd = H.quad_data(101, seed=0)
    ops = H.OPSET_BASIC
    P0, C0 = g.host_init_chains(N, PL, 7, ops=ops)
    s = g.Sampler(N, program_length=PL, ops=ops, const_proposal=g.CONST_RANDOM_WALK, rw_sd=0.1)
    try:
        s.set_data(x, y, sd)
        s.set_state(P0, C0)
        s.run_block(50, 99)
        P, C, prior, lik = s.get_state()
        n_dev, cut_dev = s.resample(1, 20.0, seed=4321)
        P1, C1, _, _ = s.get_state()
    finally:
        s.close()
    n_ref, cut_ref = port.resample(port.cfg(PL=PL, ops=ops), P, C, prior, lik, 1, 20.0, 4321)
    assert n_dev == n_ref and cut_dev == cut_ref and n_dev > 0
    assert np.array_equal(P1, P) and np.array_equal(C1.view(np.uint32), C.view(np.uint32))


@pytest.mark.parametrize("k,margin", [(1, 0.0), (10, 0.0), (100, 0.002), (999, 0.5), (1000, 0.0)])
def test_top_chains_and_map(k, margin):
    N = 1000
    prior, lik = H.mixed_scores(N, seed=5)
    s = g.Sampler(N, program_length=31)
    try:
        s.set_scores(prior, lik)
        chains, n, t = s.top_chains(k, margin)
        mc, mv = s.map_chain()
    finally:
        s.close()
    post = prior + lik
    t_ref = _sorted_ref(post)[N - k]
    assert (np.isnan(t) and np.isnan(t_ref)) or t == t_ref
    finite = ~np.isnan(post)
    want = np.where(finite & (post >= t_ref - margin))[0] if not np.isnan(t_ref) else np.where(finite)[0]
    assert n == len(want) and np.array_equal(chains, want)
    best = np.nanmax(post)
    assert mv == best and mc == int(np.where(post == best)[0][0])


def test_selection_rejects_bad_arguments():
    s = g.Sampler(16, program_length=31)
    try:
        for bad in (lambda: s.resample(0, 1.0), lambda: s.resample(0, -0.1), lambda: s.resample(2, 0.5),
                    lambda: s.top_chains(0), lambda: s.top_chains(17)):
            with pytest.raises(g.GprError):
                bad()
    finally:
        s.close()
    s = g.Sampler(16, program_length=31, ops=[g.CONST])
    try:
        with pytest.raises(g.GprError, match="at least 2 ops"):
            s.resample(0, 0.5)
    finally:
        s.close()


@pytest.mark.parametrize("mode,param", [(0, 0.5), (1, 20.0), (0, 0.0)])
def test_population_split_over_handles_equals_one_handle(mode, param):
    """One population of 4096 chains held by two handles (chains [0, 2048)
    and [2048, 4096)): the cutoff over both halves (population.py) and each
    half's re-draw below it with its chain offset (gpr_resample_below) give,
    bit for bit, the programs and constants of one handle holding every chain
    and resampling with gpr_resample.  This is the exchange a population
    spread over several GPUs makes once per block."""
    from gpuropolis_gb300 import population as pop
    N, PL, half = 4096, 31, 2048
    P0, C0 = H.random_programs(N, PL, seed=3)
    prior, lik = H.mixed_scores(N, seed=4)
    full = g.Sampler(N, program_length=PL)
    parts = [g.Sampler(half, program_length=PL) for _ in range(2)]
    try:
        full.set_state(P0, C0)
        full.set_scores(prior, lik)
        n_full, cut_full = full.resample(mode, param, seed=777)
        Pf, Cf, _, _ = full.get_state()
        cut = pop.population_cutoff(prior + lik, mode, param)
        assert (np.isnan(cut) and np.isnan(cut_full)) or cut == cut_full
        n_parts = 0
        Ps, Cs = [], []
        for k, s in enumerate(parts):
            sl = slice(k * half, (k + 1) * half)
            s.set_state(np.ascontiguousarray(P0[:, sl]), np.ascontiguousarray(C0[:, sl]))
            s.set_scores(prior[sl], lik[sl])
            pr, li = s.get_scores()
            assert np.array_equal(pr, prior[sl], equal_nan=True) and np.array_equal(li, lik[sl], equal_nan=True)
            n_parts += s.resample_below(cut, seed=777, chain_offset=k * half)
            P, C, _, _ = s.get_state()
            Ps.append(P)
            Cs.append(C)
    finally:
        full.close()
        for s in parts:
            s.close()
    assert n_parts == n_full
    assert np.array_equal(np.concatenate(Ps, axis=1), Pf)
    assert np.array_equal(np.concatenate(Cs, axis=1).view(np.uint32), Cf.view(np.uint32))


def test_resample_below_rejects_bad_arguments():
    s = g.Sampler(16, program_length=31)
    try:
        with pytest.raises(g.GprError):
            s.resample_below(0.0, 1, -1)
    finally:
        s.close()
