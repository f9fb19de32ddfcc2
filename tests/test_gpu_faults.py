"""A kernel that gives up on a bounded wait reports it and leaves the GPU usable.

The dataset is staged into each CTA's shared memory by a bulk copy whose
arrival the kernel polls a bounded number of times.  Setting that bound to
zero makes every staged launch give up at once: the kernel sets its error
flag, waits (bounded again) for its own copy to land, and returns without
touching the chains; gpr_sync reports GPR_ERR_DEVICE.  Nothing faults, and
the next block on the same handle runs normally.  The lockstep, pipelined
and Hamiltonian kernels all take this path."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")

GPR_ERR_DEVICE = 4


@pytest.mark.parametrize("kernel", ["lockstep", "pipelined", "hmc"])
def test_staging_timeout_reports_and_recovers(kernel):
    N, PL = 256, 31
    x, y, sd = H.quad_data(101, seed=3)
    kw = dict(program_length=PL, ops=H.OPSET_BASIC)
    if kernel == "hmc":
        kw.update(const_proposal=g.CONST_HMC)
    s = g.Sampler(N, **kw)
    try:
        s.set_data(x, y, sd)
        if kernel == "hmc":
            s.set_hmc_layout(4, 0)
            s.set_moves(5, 0.001, 4)
        else:
            s.set_layout(4, 0, 0, 1, 8, 1 if kernel == "pipelined" else 0)
        assert s.launch_geometry()["stream"] == 0          # the dataset is staged
        P, C = g.host_init_chains(N, PL, 5, ops=H.OPSET_BASIC)
        s.set_state(P, C)
        s.set_stage_wait(0)
        s.run_block(10, 1)
        with pytest.raises(g.GprError) as ei:
            s.sync()
        assert ei.value.code == GPR_ERR_DEVICE and "staging" in str(ei.value)
        # the chains were left as they were
        P1, C1, _, _ = s.get_state()
        assert np.array_equal(P1, P) and np.array_equal(C1.view(np.uint32), C.view(np.uint32))
        # the default bound again: the handle and the GPU are fine
        s.set_stage_wait(1 << 22)
        s.run_block(10, 1)
        s.sync()
        _, _, prior, lik = s.get_state()
        assert np.isfinite(prior).any() and np.isfinite(lik).any()
    finally:
        s.close()
