"""Golden vectors produced by the reference's own code (tests/golden/,
generated by tests/golden/make_golden.py).  The C restatement oracle and the
host formatter must reproduce them exactly; these tests need neither the
reference checkout nor a GPU."""
import glob
import json
import os

import numpy as np
import pytest

from oracle import port

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(glob.glob(os.path.join(GOLD, "*.npz")))


def _load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}, json.loads(str(z["meta"]))


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-4] for p in CASES])
def test_port_reproduces_golden(path):
    g, m = _load(path)
    P0, C0 = g["P0"], g["C0"]
    N = P0.shape[1]
    for i in range(N):
        assert port.length(P0, i) == g["length0"][i]
        assert port.count(P0, i) == g["count0"][i]
        assert port.prior(P0, C0, i, len(g["ops"])) == g["prior0"][i]
        a, b = port.likelihood(P0, C0, i, g["x"], g["y"], g["sd"]), g["lik0"][i]
        assert a == b or (np.isnan(a) and np.isnan(b))
        for j, xv in enumerate(g["xs"]):
            a, b = port.call(P0, C0, i, xv), g["fx0"][i, j]
            assert a == b or (np.isnan(a) and np.isnan(b))
    c = port.cfg(m["PL"], ops=g["ops"], rng=m["philox"], const_mode=1 if m["rw"] else 0, rw_sd=m["rw"],
                 project_math=m["project_math"])
    P, C = P0.copy(), C0.copy()
    prior, lik = port.run_block(c, P, C, g["x"], g["y"], g["sd"], m["steps"], m["seed"])
    np.testing.assert_array_equal(P, g["P1"])
    np.testing.assert_array_equal(C.view(np.int32), g["C1"].view(np.int32))
    np.testing.assert_array_equal(prior, g["prior1"])
    np.testing.assert_array_equal(lik, g["lik1"])


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[:-4] for p in CASES])
def test_host_formatter_reproduces_golden(path):
    gpr = pytest.importorskip("gpuropolis_gb300")
    try:
        gpr.library()
    except ImportError as e:
        pytest.skip(str(e))
    g, m = _load(path)
    strings = json.load(open(path[:-4] + "_strings.json"))
    for i, (s_c, s_f, s_l) in enumerate(strings):
        for ref, (fmt, latex) in ((s_c, ("C", False)), (s_f, ("%.10f", False)), (s_l, ("%.2f", True))):
            if len(ref) < 99:   # the reference's own buffers hold 99 characters
                assert gpr.format_expression(g["P0"], g["C0"], i, fmt, latex) == ref
