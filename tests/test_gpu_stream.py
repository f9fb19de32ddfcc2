"""Datasets read from device memory in every pass (the layout for data too
large to stage in shared memory) give exactly the results of the staged
layout -- same arithmetic in the same order -- for the MH kernel, the
Hamiltonian-move kernel and the gradient; a 65,536-point dataset, which only
the streamed layout can take, is scored like the oracle's likelihood
(main.cu:454-468) within the parity tolerance."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
port = pytest.importorskip("oracle.port")


def _pair(N, kw, x, y, sd, P, C):
    out = []
    for stream in (False, True):
        s = g.Sampler(N, **kw)
        s.set_data(x, y, sd)
        if stream:
            s.set_streaming(True)
        s.set_state(P, C)
        out.append(s)
    assert out[0].launch_geometry()["stream"] == 0 and out[1].launch_geometry()["stream"] == 1
    return out


@pytest.mark.parametrize("mode", ["rw", "ref", "hmc"])
def test_streamed_equals_staged(mode):
    N, PL = 2048, 31
    x, y, sd = H.expdecay_data(250, seed=9)
    kw = dict(program_length=PL, ops=H.OPSET_BASIC)
    if mode == "rw":
        kw.update(const_proposal=g.CONST_RANDOM_WALK, rw_sd=0.1)
    elif mode == "hmc":
        kw.update(const_proposal=g.CONST_HMC)
    P, C = g.host_init_chains(N, PL, 31, ops=H.OPSET_BASIC)
    a, b = _pair(N, kw, x, y, sd, P, C)
    try:
        for s in (a, b):
            if mode == "hmc":
                s.set_moves(5, 0.002, 4)
            s.run_block(30, 77)
        ra, rb = a.get_state(), b.get_state()
        assert np.array_equal(ra[0], rb[0])
        assert np.array_equal(ra[1].view(np.uint32), rb[1].view(np.uint32))
        assert np.array_equal(ra[2], rb[2]) and np.array_equal(ra[3], rb[3])
        if mode == "hmc":
            ga, la = a.loglik_grad()
            gb, lb = b.loglik_grad()
            assert np.array_equal(ga, gb, equal_nan=True) and np.array_equal(la, lb, equal_nan=True)
    finally:
        a.close()
        b.close()


def test_large_dataset_streams_and_matches_oracle():
    N, PL = 256, 31
    r = np.random.default_rng(4)
    n = 65536
    x = r.normal(0, 1, n).astype(np.float32)
    y = (np.sin(x) * x + np.exp(-x.astype(np.float64) ** 2) + r.normal(0, 0.05, n)).astype(np.float32)
    sd = np.full(n, 0.05, np.float32)
    P, C = H.random_programs(N, PL, ops=H.OPSET_BASIC, seed=6)
    s = g.Sampler(N, program_length=PL, ops=H.OPSET_BASIC, const_proposal=g.CONST_RANDOM_WALK, rw_sd=0.1)
    try:
        s.set_data(x, y, sd)
        assert s.launch_geometry()["stream"] == 1
        s.set_state(P, C)
        prior, lik = s.evaluate()
        s.run_block(5, 3)
        P1, C1, pr1, lk1 = s.get_state()
    finally:
        s.close()
    checked = 0
    for idx in range(N):
        ll64 = port.likelihood(P, C, idx, x, y, sd, f64=True)
        if not np.isfinite(ll64):
            assert not np.isfinite(lik[idx]) or abs(lik[idx]) > 1e30
            continue
        if abs(lik[idx] - ll64) <= 1e-5 * abs(ll64):
            checked += 1
    finite = np.isfinite(lik).sum()
    assert checked >= 0.95 * finite and finite > 20, (checked, finite)
    assert np.all(np.isfinite(lk1) | np.isinf(lk1))
