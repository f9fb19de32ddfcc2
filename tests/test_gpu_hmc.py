"""Hamiltonian (HMC / MALA) constant moves of the MH kernel (gpr_hmc.cuh), the
constants-only schedule and per-chain scale adaptation, checked
statistically: chains started from the exact posterior of a one-constant
model must stay distributed as that posterior.  The posterior -- Gaussian
likelihood (main.cu:454-468) times the Cauchy(0, 1) prior on constants
(main.cu:537-540) -- is computed by quadrature.  Also checks the per-step
constant trace."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
stats = pytest.importorskip("scipy.stats")

PL = 7


def _const_model(N, seed):
    """Data y ~ N(2, 0.5) at 20 points; program f = C[0] (root CONST; the
    other heap nodes are unreachable).  Initial C[0] from the exact posterior,
    the other constants from their Cauchy prior."""
    r = np.random.default_rng(seed)
    x = np.linspace(0, 1, 20).astype(np.float32)
    y = (2.0 + 0.5 * r.normal(size=20)).astype(np.float32)
    sd = np.full(20, 0.5, np.float32)
    grid = np.linspace(-3.0, 7.0, 400001)
    coarse = grid[::100]
    logp = np.array([-np.sum((y.astype(np.float64) - c) ** 2) / (2 * 0.25) for c in coarse])
    logp = np.interp(grid, coarse, logp) - np.log1p(grid ** 2)
    pdf = np.exp(logp - logp.max())
    cdf = np.cumsum(pdf)
    cdf /= cdf[-1]
    P = np.full((PL, N), g.ONE, np.int32)
    P[0] = g.CONST
    C = r.standard_cauchy((PL, N)).astype(np.float32)
    C[0] = np.interp(r.random(N), cdf, grid).astype(np.float32)
    return x, y, sd, P, C, grid, cdf


@pytest.mark.parametrize("mode,eps,L", [("hmc", 0.03, 8), ("hmc_jitter", 0.03, 8), ("mala", 0.05, 1),
                                        ("rw", 0.1, 0)])
def test_constant_moves_keep_the_posterior(mode, eps, L):
    """hmc_jitter draws each move's step from 0.03 x U(0.7, 1.3) and its
    leapfrog count from [1, 16]."""
    N, steps = 8192, 60
    x, y, sd, P, C, grid, cdf = _const_model(N, seed=3)
    if mode == "rw":
        s = g.Sampler(N, program_length=PL, const_proposal=g.CONST_RANDOM_WALK, rw_sd=eps)
        s.set_moves(0)
    else:
        s = g.Sampler(N, program_length=PL, const_proposal=g.CONST_HMC)
        s.set_moves(0, eps, L)
        if mode == "hmc_jitter":
            s.set_hmc_jitter(0.3, 1.0)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        tr = s.run_block_traced(steps, 12345, 2)
        P1, C1, prior, lik = s.get_state()
        st = s.stats()
    finally:
        s.close()
    assert np.array_equal(P1, P)                                   # no structure moves
    assert np.array_equal(tr[:, -1, :], C1[:2].T)                  # trace ends at the final state
    assert st["struct_proposed"] == 0 and st["const_proposed"] == N * steps
    acc = st["const_accepted"] / st["const_proposed"]
    assert acc > 0.3, acc
    cdf_f = lambda v: np.interp(v, grid, cdf)  # noqa: E731
    for samples in (C1[0].astype(np.float64), tr[:, steps // 2, 0].astype(np.float64)):
        ks = stats.kstest(samples, cdf_f)
        assert ks.pvalue > 1e-3, (mode, ks)
    assert np.mean(np.abs(C1[0] - C[0])) > 0.02                    # the chains moved


@pytest.mark.parametrize("mode,target", [("rw", 0.3), ("hmc", 0.7), ("mala", 0.6)])
def test_adapted_scales_reach_the_target_acceptance(mode, target):
    """Per-chain scale adaptation (Robbins-Monro for the random walk, dual
    averaging for HMC/MALA): after adapting blocks and freezing, the constant
    moves of a block are accepted at about the target rate; the frozen scales
    still leave the posterior invariant (KS against the quadrature)."""
    N = 8192
    x, y, sd, P, C, grid, cdf = _const_model(N, seed=5)
    if mode == "rw":
        s = g.Sampler(N, program_length=PL, const_proposal=g.CONST_RANDOM_WALK, rw_sd=1.0)
        s.set_moves(0)
    else:
        s = g.Sampler(N, program_length=PL, const_proposal=g.CONST_HMC)
        s.set_moves(0, 0.5, 8 if mode == "hmc" else 1)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        s.adapt_scales(target)
        for b in range(4):
            s.run_block(100, 100 + b)
        s.adapt_scales(0.0)
        sc = s.chain_scales()
        s.reset_stats()
        s.run_block(100, 999)
        st = s.stats()
        C1 = s.get_state()[1]
    finally:
        s.close()
    acc = st["const_accepted"] / st["const_proposed"]
    if mode == "hmc":
        # the averaged step of dual averaging errs on the small side where the
        # acceptance curve is flat: at least the target, and well adapted
        # from the far too large initial step
        assert target - 0.12 < acc < 0.98, (mode, acc, np.median(sc))
    else:
        assert abs(acc - target) < 0.12, (mode, acc, np.median(sc))
    assert np.all(np.isfinite(sc)) and np.all(sc > 0)
    ks = stats.kstest(C1[0].astype(np.float64), lambda v: np.interp(v, grid, cdf))
    assert ks.pvalue > 1e-3, (mode, ks)


def test_traced_first_chains_match_the_full_trace():
    """gpr_run_block_traced_first records the first chains' constants exactly
    as the full trace does, and every chain still steps."""
    N, steps = 512, 12
    x, y, sd, P, C, grid, cdf = _const_model(N, seed=4)
    s = g.Sampler(N, program_length=PL, const_proposal=g.CONST_HMC)
    try:
        s.set_moves(0, 0.03, 4)
        s.set_hmc_jitter(0.2, 0.5)
        s.set_data(x, y, sd)
        s.set_state(P, C)
        full = s.run_block_traced(steps, 77, 3)
        Cf = s.get_state()[1]
        s.set_state(P, C)
        part = s.run_block_traced(steps, 77, 3, chains=100)
        Cp = s.get_state()[1]
        with pytest.raises(g.GprError):
            s.run_block_traced(steps, 77, 3, chains=N + 1)
    finally:
        s.close()
    assert part.shape == (100, steps, 3)
    assert np.array_equal(part.view(np.uint32), full[:100].view(np.uint32))
    assert np.array_equal(Cp.view(np.uint32), Cf.view(np.uint32))
