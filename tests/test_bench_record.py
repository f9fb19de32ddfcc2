"""The bench line's record helpers, on CPU: the roofline objects carry the
fields the record asks for, with frac = achieved / peak; both arms report the
same config keys; and the ESS comparison's estimator reads a run that never
moves as zero."""
import argparse

import numpy as np

import bench
from gpuropolis_gb300.diagnostics import population_ess


def test_fp32_roofline_fields_and_arithmetic():
    r = bench.fp32_roofline(node_points=4.0e12, seconds=2.0, nsm=152, peaks={"sm_max_mhz": 2000.0},
                            sm_mhz=1000.0, traffic=113.43e6)
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r
    assert r["bound"] == "fp32-issue" and r["unit"] == "TFLOP/s"
    assert np.isclose(r["achieved"], 2.0)
    assert np.isclose(r["peak"], 152 * 128 * 2000e6 / 1e12)
    assert np.isclose(r["frac"], r["achieved"] / r["peak"])
    assert np.isclose(r["frac_at_measured_clock"], 2.0 / (152 * 128 * 1000e6 / 1e12))
    assert r["traffic"] == 113.43e6 and "ncu" in r["traffic_source"]
    assert bench.fp32_roofline(1.0, 1.0, 152, {})["traffic"] is None


def test_hbm_roofline_fields():
    r = bench.hbm_roofline(point_evals=1.0e9, seconds=1.0, peaks={"hbm_gbs": 6000.0}, traffic=None)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert np.isclose(r["achieved"], 12.0) and np.isclose(r["frac"], 12.0 / 6000.0)


def test_both_arms_share_the_config_keys():
    """The GPU arm and the reference arm build their config from the same
    workload through config_of: same keys, same values."""
    w = bench.WORKLOADS["plain-mh-131k"]
    a = bench.config_of(argparse.Namespace(workload="plain-mh-131k", impl="gb300"), w)
    b = bench.config_of(argparse.Namespace(workload="plain-mh-131k", impl="reference"), w)
    assert a == b
    assert {"workload", "N", "PL", "nd", "mh_steps", "map_delta", "ops", "const_proposal", "rng"} <= set(a)


def test_population_ess_of_chains_that_never_move_is_zero():
    x = np.repeat(np.random.default_rng(0).normal(size=(64, 1)), 200, axis=1)[:, :, None]
    used = np.ones((1, 64), bool)
    assert population_ess(x, used) == 0.0
