"""GPU parity of the CUDA path (through the C ABI) against the reference's own
code compiled for host cores (oracle/ref.py).

  * evaluator: f(x) of compiled programs vs the reference's call()
    (main.cu:446-448), description length and node count exactly;
  * prior and log-likelihood of whole chains vs compute_prior /
    compute_likelihood (main.cu:529-544, 454-468), <= 1e-5 relative;
  * MH blocks: after a block of steps from the same state and seed, chains are
    bit-identical to MH_simple_kernel (main.cu:679-813) run by the oracle with
    the same random stream (LCG and Philox; reference and random-walk constant
    proposals; the reference op set and the {+,-,*,/,exp,log,pow} set).
"""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu

g = pytest.importorskip("gpuropolis_gb300")
oref = pytest.importorskip("oracle.ref")


def _need_ref():
    if not oref.available():
        pytest.skip("reference oracle source not available")


@pytest.fixture(scope="module")
def lib():
    return g.library()


@pytest.mark.parametrize("PL", [31, 63])
def test_eval_values_match_reference(lib, PL):
    _need_ref()
    N = 1024
    P, C = H.random_programs(N, PL, seed=PL)
    xs = np.linspace(-3.0, 12.0, 48).astype(np.float32)
    s = g.Sampler(N, program_length=PL)
    s.set_data(xs[:4], xs[:4], np.ones(4, np.float32))
    s.set_state(P, C)
    out, length, count = s.eval_values(xs)
    o = oref.get(pl=PL, project_math=1)
    ref = np.array([[o.call(P, C, i, xv) for xv in xs] for i in range(N)], np.float32)
    rlen = np.array([o.length(P, C, i) for i in range(N)], np.float32)
    rcnt = np.array([o.count_nodes(P, C, i) for i in range(N)], np.int32)
    np.testing.assert_array_equal(length, rlen)
    np.testing.assert_array_equal(count, rcnt)
    cls = H.same_class(out, ref)
    assert cls.mean() > 0.995, "finite/non-finite class differs on %.4f of points" % (1 - cls.mean())
    both = np.isfinite(out) & np.isfinite(ref)
    rel = H.rel_err(out[both], ref[both], floor=1e-30)
    assert np.mean(rel <= 1e-5) > 0.995, np.sort(rel)[-10:]
    s.close()


@pytest.mark.parametrize("data", ["quad", "expdecay"])
def test_prior_likelihood_match_reference(lib, data):
    _need_ref()
    N, PL = 2048, 31
    x, y, sd = H.quad_data() if data == "quad" else H.expdecay_data()
    P, C = H.random_programs(N, PL, seed=7)
    s = g.Sampler(N, program_length=PL)
    s.set_data(x, y, sd)
    s.set_state(P, C)
    prior, lik = s.evaluate()
    o = oref.get(pl=PL, project_math=1)
    rprior = np.array([o.prior(P, C, i) for i in range(N)])
    rlik = np.array([o.likelihood(P, C, i, x, y, sd) for i in range(N)])
    assert np.all(H.same_class(prior, rprior))
    fin = np.isfinite(rprior)
    assert H.rel_err(prior[fin], rprior[fin]).max() <= 1e-5
    assert H.same_class(lik, rlik).mean() > 0.995
    fin = np.isfinite(lik) & np.isfinite(rlik)
    assert fin.sum() > N // 10
    rel = H.rel_err(lik[fin], rlik[fin])
    assert np.mean(rel <= 1e-5) > 0.99, np.sort(rel)[-10:]
    s.close()


CASES = [
    # (PL, opset, rng, const mode, rw_sd, data)
    (31, None, g.RNG_LCG, g.CONST_REFERENCE, 0.0, "quad"),
    (31, None, g.RNG_PHILOX, g.CONST_REFERENCE, 0.0, "quad"),
    (31, H.OPSET_BASIC, g.RNG_LCG, g.CONST_RANDOM_WALK, 0.1, "quad"),
    (63, H.OPSET_BASIC, g.RNG_LCG, g.CONST_RANDOM_WALK, 0.1, "expdecay"),
    (63, None, g.RNG_PHILOX, g.CONST_REFERENCE, 0.0, "expdecay"),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "pl%d-%s-%s-%s" % (
    c[0], "basic" if c[1] else "ref", "philox" if c[2] else "lcg", "rw" if c[3] else "indep"))
def test_mh_block_matches_reference(lib, case):
    _need_ref()
    PL, ops, rng, cmode, rw_sd, data = case
    N, steps, seed = 1024, 25, 987654
    x, y, sd = H.quad_data() if data == "quad" else H.expdecay_data()
    P, C = H.random_programs(N, PL, ops=ops, seed=11)
    s = g.Sampler(N, program_length=PL, ops=ops, rng=rng, const_proposal=cmode, rw_sd=rw_sd)
    s.set_data(x, y, sd)
    s.set_state(P, C)
    s.run_block(steps, seed)
    Pg, Cg, prior_g, lik_g = s.get_state()
    o = oref.get(pl=PL, opset=1 if ops else 0, philox=int(rng == g.RNG_PHILOX), project_math=1,
                 rw_sd=rw_sd)
    Pr, Cr = P.copy(), C.copy()
    prior_r, lik_r = o.run_kernel(Pr, Cr, x, y, sd, steps, seed)
    same = np.all(Pg == Pr, axis=0) & np.all(Cg.view(np.int32) == Cr.view(np.int32), axis=0)
    assert same.mean() >= 0.98, "bit-identical chains: %.4f" % same.mean()
    ok = same & np.isfinite(lik_r) & np.isfinite(prior_r)
    assert H.rel_err(prior_g[ok], prior_r[ok]).max() <= 1e-5
    rel = H.rel_err(lik_g[ok], lik_r[ok])
    assert np.mean(rel <= 1e-5) > 0.99
    s.close()
