"""The reverse-mode adjoint of the device evaluator (gpr_loglik_grad,
gpr_hmc.cuh) against the oracle's FP64 gradient (oracle/gpr_oracle.c), which
is itself pinned to FP64 central finite differences (test_oracle_port.py), and
through a torch.autograd.Function in the test harness, against FP64 finite
differences with h = 1e-6.

Tolerance: 1e-4 relative, plus the FP32 rounding of the per-point sum, bounded
by 2e-5 times the sum of the absolute per-point terms (a gradient near an
optimum is a sum of terms that cancel), plus 1e-18 absolute: per-point terms
below the FP32 range at the 2^-64 bookkeeping scale (about 1e-26) vanish.
Beyond that, only where the gradient's own FP32 noise floor is larger: four
times its spread over FP64 evaluations with every operation jittered by
2^-22 (the method the value parity tests use).  Where an intermediate of the
FP32 sweep leaves the FP32 range the gradient comes out non-finite (a
Hamiltonian move then rejects); that must stay rare, and every finite
gradient must meet the tolerance."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")
port = pytest.importorskip("oracle.port")

REL, CANCEL, FLOOR = 1e-4, 2e-5, 1e-18


@pytest.mark.parametrize("PL,ops", [(15, None), (15, H.OPSET_BASIC), (31, H.OPSET_BASIC)])
def test_adjoint_matches_fp64_gradient(PL, ops):
    x, y, sd = H.rational_data(1024, seed=PL)
    N = 2048
    P, C = H.random_programs(N, PL, ops=ops, seed=PL + 1)
    s = g.Sampler(N, program_length=PL)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        grad, lik = s.loglik_grad()
        _, lik_ev = s.evaluate()
    finally:
        s.close()
    used = H.used_constants(P)
    n_ok = n_bad = n_chk = n_nonfinite = 0
    for idx in range(N):
        if not np.isfinite(lik[idx]) or not used[:, idx].any():
            continue
        ll64, g64, gabs = port.loglik_grad_f64(P, idx, C[:, idx].astype(np.float64), x, y, sd)
        # FP32-conditioned programs: the likelihood itself is off by more than 1e-5
        if not np.isfinite(ll64) or abs(lik[idx] - ll64) > 1e-5 * abs(ll64):
            continue
        assert abs(lik[idx] - lik_ev[idx]) <= 1e-6 * abs(lik_ev[idx])
        sens = None
        for k in np.where(used[:, idx])[0]:
            if not np.isfinite(g64[k]):
                continue
            n_chk += 1
            if not np.isfinite(grad[k, idx]):
                n_nonfinite += 1        # an FP32 intermediate left the range: flagged, not wrong
                continue
            tol = REL * abs(g64[k]) + CANCEL * gabs[k] + FLOOR
            if abs(grad[k, idx] - g64[k]) <= tol:
                n_ok += 1
                continue
            # beyond it only where the gradient's own FP32 noise floor is larger
            if sens is None:
                sens = port.grad_sensitivity(P, idx, C[:, idx].astype(np.float64), x, y, sd)
            if not abs(grad[k, idx] - g64[k]) <= tol + 4 * sens[k]:
                n_bad += 1
        assert np.all(grad[~used[:, idx], idx] == 0)
    assert n_chk > 200, n_chk
    assert n_bad == 0, (n_bad, n_chk)
    assert n_nonfinite <= 0.01 * n_chk, (n_nonfinite, n_chk)


def test_adjoint_on_the_rational_model():
    """The five constants of the generating rational function, at the truth
    and away from it: every gradient within 1e-4 of the FP64 one."""
    b, _ = H.rational_coefficients(3)
    x, y, sd = H.rational_data(1024, seed=3)
    N = 64
    P, C = H.rational_program(N, b)
    r = np.random.default_rng(0)
    nodes = np.array(H.RATIONAL_NODES) - 1
    C[nodes, 1:] += (r.normal(0, 0.05, (5, N - 1))).astype(np.float32)
    s = g.Sampler(N, program_length=31)
    try:
        s.set_data(x, y, sd)
        s.set_state(P, C)
        grad, lik = s.loglik_grad()
    finally:
        s.close()
    for idx in range(N):
        ll64, g64, gabs = port.loglik_grad_f64(P, idx, C[:, idx].astype(np.float64), x, y, sd)
        for k in nodes:
            assert abs(grad[k, idx] - g64[k]) <= REL * abs(g64[k]) + CANCEL * gabs[k] + FLOOR, (idx, k)


def _linear_program(PL=7):
    """f(x) = C[1] * x + C[0]: node 1 CPLUS (C[0]), node 2 CTIMES (C[1]),
    node 4 A -> x."""
    P = np.zeros((PL, 1), np.int32)
    P[0, 0], P[1, 0], P[3, 0] = g.CPLUS, g.CTIMES, g.A
    return P


def test_adjoint_through_torch_autograd():
    """d loglik / d C as a torch.autograd.Function over gpr_loglik_grad, checked
    against FP64 central differences (h = 1e-6) of the oracle's likelihood."""
    torch = pytest.importorskip("torch")
    x, y, sd = H.quad_data(101, seed=4)
    PL = 7
    P = _linear_program(PL)
    s = g.Sampler(1, program_length=PL)
    s.set_data(x, y, sd)

    class LogLik(torch.autograd.Function):
        @staticmethod
        def forward(ctx, c):
            C = c.detach().cpu().numpy().astype(np.float32).reshape(PL, 1)
            s.set_state(P, C)
            grad, lik = s.loglik_grad()
            ctx.save_for_backward(torch.from_numpy(grad[:, 0].copy()))
            return c.new_tensor(lik[0])

        @staticmethod
        def backward(ctx, go):
            (gr,) = ctx.saved_tensors
            return go * gr.to(go.dtype)

    try:
        for c0 in ([0.7, 20.0], [-1.3, 24.5], [3.0, 18.0]):
            c = torch.zeros(PL, dtype=torch.float64)
            c[0], c[1] = c0[0], c0[1]
            c.requires_grad_(True)
            LogLik.apply(c).backward()
            Cd = c.detach().numpy().astype(np.float32).astype(np.float64)
            _, g64, gabs = port.loglik_grad_f64(P, 0, Cd, x, y, sd)
            for k in (0, 1):
                a, b = Cd.copy(), Cd.copy()
                a[k] += 1e-6
                b[k] -= 1e-6
                fd = (port.loglik_f64(P, 0, a, x, y, sd) - port.loglik_f64(P, 0, b, x, y, sd)) / 2e-6
                assert abs(c.grad[k].item() - fd) <= REL * abs(fd) + CANCEL * gabs[k], (c0, k, c.grad[k].item(), fd)
            assert np.all(c.grad[2:].numpy() == 0)
    finally:
        s.close()
