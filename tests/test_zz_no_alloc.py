"""gpr_run_block_noalloc: the MH block on chain state in the caller's device
memory, with the dataset, the Hastings-term table and the kernel's counters in
one fixed scratch array per device instead of allocations.  It must give the
chains that gpr_create + gpr_set_data + gpr_set_state + gpr_run_block give,
call after call, and refuse datasets larger than its scratch.

This file is collected last so that the scratch is exercised after every other
test has used the library, and it passes on its own as well."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests import helpers as H

g = pytest.importorskip("gpuropolis_gb300")

_HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gpuropolis.h")
MAX_POINTS = 4096
# Both paths run the same kernel on the same inputs: programs and constants
# must be bit-identical, prior and likelihood equal to this relative tolerance.
RTOL = 1e-6


def _entry():
    f = g.library().gpr_run_block_noalloc
    vp, ip = ctypes.c_void_p, ctypes.c_int
    f.argtypes = [ctypes.POINTER(g.Config), ip, vp, vp, vp, vp, vp, vp, vp, ip, ip, ip]
    f.restype = ip
    return f


def _call(cfg, n, dev, x, y, sd, steps, seed):
    x, y, sd = (np.ascontiguousarray(a, np.float32) for a in (x, y, sd))
    rc = _entry()(ctypes.byref(cfg), n, dev[0], dev[1], dev[2], dev[3],
                  g._ptr(x), g._ptr(y), g._ptr(sd), len(x), steps, seed)
    return rc, g.library().gpr_last_error(None).decode()


def test_header_states_the_limit():
    text = open(_HEADER).read()
    m = re.search(r"#define\s+GPR_NOALLOC_MAX_POINTS\s+(\d+)", text)
    assert m and int(m.group(1)) == MAX_POINTS
    assert "int gpr_run_block_noalloc(" in text


def test_rejects_dataset_larger_than_scratch():
    """Rejected with GPR_ERR_ARG and a message naming the limit, before any
    device work (so this runs without a GPU; the state pointers are never
    dereferenced)."""
    cfg = g.make_config()
    n = MAX_POINTS + 1
    x = np.zeros(n, np.float32)
    sd = np.ones(n, np.float32)
    dummy = np.zeros(64 * 31, np.float64)
    p = g._ptr(dummy)
    rc, msg = _call(cfg, 64, (p, p, p, p), x, x, sd, 1, 1)
    assert rc == 1 and str(MAX_POINTS) in msg and "gpr_set_data" in msg, (rc, msg)
    rc, msg = _call(cfg, 64, (None, None, None, None), x[:10], x[:10], sd[:10], 1, 1)
    assert rc == 1 and "device pointers" in msg, (rc, msg)


def test_rejects_three_variable_config():
    """The entry point runs one input variable only: a configuration asking
    for three (or an invalid count) is refused, not run as univariate."""
    x = np.zeros(8, np.float32)
    sd = np.ones(8, np.float32)
    dummy = np.zeros(64 * 31, np.float64)
    p = g._ptr(dummy)
    for nv in (2, 3):
        cfg = g.make_config()
        cfg.n_vars = nv
        rc, msg = _call(cfg, 64, (p, p, p, p), x, x, sd, 1, 1)
        assert rc == 1 and "n_vars" in msg, (nv, rc, msg)


def _device_state(s):
    ptrs = [ctypes.c_void_p() for _ in range(4)]
    s._check(s.lib.gpr_device_state(s.h, *[ctypes.byref(p) for p in ptrs]))
    return tuple(p.value for p in ptrs)


def _same(a, b):
    Pa, Ca, pra, lia = a
    Pb, Cb, prb, lib_ = b
    assert np.array_equal(Pa, Pb)
    assert np.array_equal(Ca.view(np.uint32), Cb.view(np.uint32))
    np.testing.assert_allclose(prb, pra, rtol=RTOL, equal_nan=True)
    np.testing.assert_allclose(lib_, lia, rtol=RTOL, equal_nan=True)


CASES = {
    "ref-lcg": (dict(program_length=31), H.quad_data(60, seed=3), 1024),
    "basic-philox-rw": (dict(program_length=63, ops=H.OPSET_BASIC, rng=g.RNG_PHILOX,
                             const_proposal=g.CONST_RANDOM_WALK, rw_sd=0.1),
                        H.expdecay_data(250, seed=5), 512),
    "max-points": (dict(program_length=31), H.quad_data(MAX_POINTS, seed=7), 256),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_matches_handle_path_on_consecutive_calls(case):
    """Two blocks in a row: after each, the chains updated in place by the
    no-allocation call equal the handle path's."""
    kw, (x, y, sd), N = CASES[case]
    PL = kw["program_length"]
    P0, C0 = g.host_init_chains(N, PL, 4242, ops=kw.get("ops"))
    ref = g.Sampler(N, **kw)       # the handle path
    ref.set_data(x, y, sd)
    ref.set_state(P0, C0)
    own = g.Sampler(N, **kw)       # only its device arrays are used, as caller-owned memory
    own.set_state(P0, C0)
    dev = _device_state(own)
    cfg = g.make_config(**kw)
    try:
        for steps, seed in ((20, 11), (15, 987654)):
            ref.run_block(steps, seed)
            want = ref.get_state()
            rc, msg = _call(cfg, N, dev, x, y, sd, steps, seed)
            assert rc == 0, msg
            _same(want, own.get_state())
    finally:
        ref.close()
        own.close()
