"""Every evaluation layout gives the same chains, bit for bit.

The likelihood's reduction tree is fixed by point index (FP32 sums of
128-point chunks, added in FP64 in chunk order), and every layout runs each
chain's proposals, prior and accept rule in the same order, so the layout the
autotuner picks changes speed only.  Checked here across the pipelined kernel
(two chains per warp, one barrier per half-step) and the lockstep kernel (CTA
barriers every step, every 5 steps, or none), K = 4 and 8 points per lane, data
in registers, staged in shared memory or streamed from device memory, heavy
ops unrolled or rolled, 8 and 4 warps per CTA; with chain counts that leave a
CTA's groups partly empty, datasets of one pass, several passes, and more
chunks than the pipelined kernel's shared-memory board holds."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")

LAYOUTS = [
    dict(K=4, onepass=0, rolled=0, pipe=1),
    dict(K=4, onepass=1, rolled=0, pipe=1),
    dict(K=8, onepass=1, rolled=0, pipe=1),
    dict(K=8, onepass=0, rolled=0, pipe=1),
    dict(K=4, onepass=0, rolled=0, pipe=1, warps_per_cta=4),
    dict(K=4, onepass=0, rolled=0, pipe=1, stream=True),
    dict(K=4, onepass=0, rolled=0, pipe=0),
    dict(K=8, onepass=1, rolled=1, pipe=0),
    dict(K=4, onepass=0, rolled=0, pipe=0, lockstep=5, warps_per_cta=4),
    dict(K=4, onepass=0, rolled=1, pipe=0, lockstep=0, warps_per_cta=2),
    dict(K=4, onepass=0, rolled=0, pipe=0, stream=True, lockstep=0),
]

CASES = {
    # one pass at K = 8, two at K = 4; 1001 chains leave partial chain groups
    "expdecay250-rw-lcg": (dict(program_length=63, ops=H.OPSET_BASIC, const_proposal=g.CONST_RANDOM_WALK,
                                rw_sd=0.1), lambda: H.expdecay_data(250, seed=3), 1001, 30),
    # the reference's independence proposals and op set, Philox stream, 101 points
    "quad101-ref-philox": (dict(program_length=31, rng=g.RNG_PHILOX), lambda: H.quad_data(101, seed=4), 640, 30),
    # 9,000 points: 71 chunks, more than the pipelined kernel's shared board
    "expdecay9000-rw": (dict(program_length=31, ops=H.OPSET_BASIC, const_proposal=g.CONST_RANDOM_WALK,
                             rw_sd=0.1), lambda: H.expdecay_data(9000, seed=5), 160, 6),
}


def _run(kw, data, N, steps, layout, P, C):
    s = g.Sampler(N, **kw)
    try:
        s.set_data(*data)
        lay = dict(layout)
        stream = lay.pop("stream", False)
        if stream:
            s.set_streaming(True)
        nd = len(data[0])
        if lay.get("onepass") and nd > 32 * lay["K"]:
            return None                     # not a valid layout for this dataset
        s.set_layout(lay["K"], lay["onepass"], lay["rolled"], lay.get("lockstep", 1),
                     lay.get("warps_per_cta", 8), lay["pipe"])
        geo = s.launch_geometry()
        assert geo["pipe"] == lay["pipe"] and geo["K"] == lay["K"] and geo["stream"] == int(stream)
        s.set_state(P, C)
        s.run_block(steps, 12345)
        return s.get_state()
    finally:
        s.close()


@pytest.mark.parametrize("case", list(CASES))
def test_all_layouts_give_the_same_chains(case):
    kw, make, N, steps = CASES[case]
    data = make()
    P, C = g.host_init_chains(N, kw["program_length"], 77, ops=kw.get("ops"))
    ref = None
    ran = 0
    for lay in LAYOUTS:
        got = _run(kw, data, N, steps, lay, P, C)
        if got is None:
            continue
        ran += 1
        if ref is None:
            ref = (lay, got)
            continue
        Pa, Ca, pra, lia = ref[1]
        Pb, Cb, prb, lib_ = got
        where = "%s vs %s" % (ref[0], lay)
        assert np.array_equal(Pa, Pb), where
        assert np.array_equal(Ca.view(np.uint32), Cb.view(np.uint32)), where
        assert np.array_equal(pra.view(np.uint64), prb.view(np.uint64)), where
        assert np.array_equal(lia.view(np.uint64), lib_.view(np.uint64)), where
    assert ran >= 8
    # the block did something: some chains moved, some scores are finite
    assert np.isfinite(ref[1][3]).mean() > 0.2
    assert not np.array_equal(ref[1][1], C)


PROF_LAYOUTS = [
    dict(K=4, onepass=0, rolled=0, pipe=0),
    dict(K=4, onepass=0, rolled=0, pipe=0, stream=True),
    dict(K=8, onepass=1, rolled=0, pipe=0),
    dict(K=4, onepass=0, rolled=0, pipe=1),
    dict(K=4, onepass=0, rolled=0, pipe=1, stream=True),
    dict(K=8, onepass=1, rolled=0, pipe=1),
]


@pytest.mark.parametrize("layout", PROF_LAYOUTS, ids=lambda l: "-".join("%s%s" % kv for kv in sorted(l.items())))
def test_phase_timed_build_gives_the_same_chains(layout):
    """gpr_debug_phase_profile runs the layout's phase-timed build: the same
    chains as run_block, bit for bit (1001 chains, so the last chain group is
    partly empty), its own consistency checks quiet, and counters that add up
    (every phase's cycles counted, the passes of every evaluation)."""
    kw, make, N, steps = CASES["expdecay250-rw-lcg"]
    data = make()
    P, C = g.host_init_chains(N, kw["program_length"], 77, ops=kw["ops"])
    want = _run(kw, data, N, steps, layout, P, C)
    s = g.Sampler(N, **kw)
    try:
        s.set_data(*data)
        lay = dict(layout)
        if lay.pop("stream", False):
            s.set_streaming(True)
        s.set_layout(lay["K"], lay["onepass"], lay["rolled"], 1, 8, lay["pipe"])
        s.set_state(P, C)
        s.reset_stats()
        ph = s.phase_profile(steps, 12345)
        got = s.get_state()
        st = s.stats()
    finally:
        s.close()
    assert np.array_equal(got[0], want[0])
    assert np.array_equal(got[1].view(np.uint32), want[1].view(np.uint32))
    np.testing.assert_array_equal(got[2], want[2])
    np.testing.assert_array_equal(got[3], want[3])
    cyc = ph["cycles"]
    assert cyc["evaluation"] > 0 and cyc["constant_proposal"] > 0 and cyc["compile"] > 0
    # at most ceil(250 / (32 K)) passes per evaluation (one in the one-pass
    # layouts); an evaluation that meets an invalid value may skip the rest
    npass = 1 if layout["onepass"] else -(-250 // (32 * layout["K"]))
    assert st["evals"] >= N * steps
    assert 0.5 * st["evals"] * npass < ph["passes"] <= st["evals"] * npass, (ph["passes"], st["evals"], npass)
