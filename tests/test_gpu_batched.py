"""Batched data and captured block sequences.

Batched data (gpr_set_batched_data): many datasets of uneven size in one
launch, chain c fitting dataset c // (N / n_datasets).  Every chain must end
bit-identical -- programs, constants, prior and likelihood -- to the same
chain run by a handle that holds its dataset alone (gpr_set_data) in the same
evaluation layout, for the MH kernel (staged per chain group or streamed), the
Hamiltonian-move kernel and the gradient.

Captured block sequences (gpr_capture_blocks / gpr_run_captured): replaying
the captured graph with a list of seeds gives exactly the chains of one
gpr_run_block call per seed."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
g = pytest.importorskip("gpuropolis_gb300")

SIZES = [130, 7, 1000, 0, 64, 513]


def _datasets(sizes, seed=0, three=False):
    out = []
    for d, n in enumerate(sizes):
        if three:
            x1, x2, x3, y, sd = H.multivar_data(n, seed=seed + d) if n else [np.zeros(0, np.float32)] * 5
            out.append((x1, x2, x3, y, sd))
        else:
            x, y, sd = H.expdecay_data(n, seed=seed + d) if n else [np.zeros(0, np.float32)] * 3
            out.append((x, y, sd))
    return out


def _same_state(a, b, what=""):
    Pa, Ca, pa, la = a
    Pb, Cb, pb, lb = b
    assert np.array_equal(Pa, Pb), what
    assert np.array_equal(Ca.view(np.uint32), Cb.view(np.uint32)), what
    assert np.array_equal(pa, pb, equal_nan=True), what
    assert np.array_equal(la, lb, equal_nan=True), what


def _cols(state, lo, hi):
    P, C, pr, li = state
    return P[:, lo:hi], C[:, lo:hi], pr[lo:hi], li[lo:hi]


MODES = {
    "ref-lcg": dict(program_length=31),
    "rw-philox": dict(program_length=63, ops=H.OPSET_BASIC, rng=g.RNG_PHILOX,
                      const_proposal=g.CONST_RANDOM_WALK, rw_sd=0.1),
    "hmc": dict(program_length=31, ops=H.OPSET_BASIC, const_proposal=g.CONST_HMC),
}


def _setup(s, mode):
    if mode == "hmc":
        s.set_moves(5, 0.002, 4)


@pytest.mark.parametrize("stream", [False, True], ids=["staged", "streamed"])
@pytest.mark.parametrize("cpd", [64, 12])
@pytest.mark.parametrize("mode", list(MODES))
def test_batched_chains_equal_single_dataset_runs(mode, cpd, stream):
    if mode == "hmc" and stream:
        pytest.skip("batched Hamiltonian moves always stream")
    kw = MODES[mode]
    PL = kw["program_length"]
    sets = _datasets(SIZES, seed=40)
    N = cpd * len(sets)
    P, C = g.host_init_chains(N, PL, 5150, ops=kw.get("ops"))
    b = g.Sampler(N, **kw)
    try:
        b.set_batched_data(sets)
        if stream:
            b.set_streaming(True)
        _setup(b, mode)
        geo = b.launch_geometry()
        assert geo["onepass"] == 0
        if mode != "hmc":   # chain groups claimed per CTA, never straddling datasets
            assert geo["lockstep"] >= 1 and cpd % geo["warps_per_cta"] == 0
        assert geo["stream"] == int(stream or mode == "hmc")
        b.set_state(P, C)
        b.run_block(25, 31337)
        got = b.get_state()
        grad_b = b.loglik_grad() if mode == "hmc" else None
    finally:
        b.close()
    for d, (x, y, sd) in enumerate(sets):
        s = g.Sampler(N, **kw)
        try:
            s.set_data(x, y, sd)
            if mode == "hmc":
                s.set_streaming(True)
            else:
                s.set_layout(4, 0, 0, lockstep=geo["lockstep"], warps_per_cta=geo["warps_per_cta"])
                if stream:
                    s.set_streaming(True)
            _setup(s, mode)
            s.set_state(P, C)
            s.run_block(25, 31337)
            lo, hi = d * cpd, (d + 1) * cpd
            _same_state(_cols(got, lo, hi), _cols(s.get_state(), lo, hi), "dataset %d (%d points)" % (d, len(x)))
            if mode == "hmc":
                gs, ls = s.loglik_grad()
                assert np.array_equal(grad_b[0][:, lo:hi], gs[:, lo:hi], equal_nan=True)
                assert np.array_equal(grad_b[1][lo:hi], ls[lo:hi], equal_nan=True)
        finally:
            s.close()


def test_batched_three_variables():
    kw = dict(program_length=31, ops=H.OPSET_MULTI, n_vars=3, rng=g.RNG_PHILOX,
              const_proposal=g.CONST_RANDOM_WALK, rw_sd=0.1)
    sets = _datasets([300, 17, 64], seed=3, three=True)
    cpd = 32
    N = cpd * len(sets)
    P, C = g.host_init_chains(N, 31, 77, ops=H.OPSET_MULTI)
    b = g.Sampler(N, **kw)
    try:
        b.set_batched_data(sets)
        geo = b.launch_geometry()
        b.set_state(P, C)
        b.run_block(20, 4)
        got = b.get_state()
    finally:
        b.close()
    for d, ds in enumerate(sets):
        s = g.Sampler(N, **kw)
        try:
            s.set_data3(*ds)
            s.set_layout(4, 0, 0, lockstep=geo["lockstep"], warps_per_cta=geo["warps_per_cta"])
            s.set_state(P, C)
            s.run_block(20, 4)
            lo, hi = d * cpd, (d + 1) * cpd
            _same_state(_cols(got, lo, hi), _cols(s.get_state(), lo, hi), "dataset %d" % d)
        finally:
            s.close()


def test_batched_data_rejects_bad_arguments():
    s = g.Sampler(96, program_length=31)
    try:
        with pytest.raises(g.GprError, match="split evenly"):
            s.set_batched_data(_datasets([5, 5, 5, 5, 5]))
        with pytest.raises(g.GprError, match="n_datasets"):
            s.set_batched_data([])
        x, y, sd = H.quad_data(10)
        sd = sd.copy()
        sd[3] = 0.0
        with pytest.raises(g.GprError, match="not > 0"):
            s.set_batched_data([(x, y, sd), H.quad_data(4), H.quad_data(6)])
    finally:
        s.close()


@pytest.mark.parametrize("mode", ["ref-lcg", "hmc"])
def test_captured_replay_equals_blocks(mode):
    kw = MODES[mode]
    N, PL = 1024, kw["program_length"]
    x, y, sd = H.quad_data(101, seed=2)
    P, C = g.host_init_chains(N, PL, 99, ops=kw.get("ops"))
    a, b = g.Sampler(N, **kw), g.Sampler(N, **kw)
    try:
        for s in (a, b):
            s.set_data(x, y, sd)
            _setup(s, mode)
            s.set_state(P, C)
        b.capture_blocks(3, 12)
        n0 = b.launch_count()
        for seeds in ([5, 77, 123456], [2 ** 31 - 1, 0, 42]):
            for sd_ in seeds:
                a.run_block(12, sd_)
            b.run_captured(seeds)
            _same_state(a.get_state(), b.get_state(), str(seeds))
        assert b.launch_count() - n0 == 6
        with pytest.raises(g.GprError):
            b.run_captured([1, 2])
        # new data drops the capture
        b.set_data(x[:50], y[:50], sd[:50])
        with pytest.raises(g.GprError, match="captured"):
            b.run_captured([1, 2, 3])
    finally:
        a.close()
        b.close()


def test_captured_replay_over_batched_data():
    sets = _datasets([40, 900, 3, 250], seed=8)
    N = 64 * len(sets)
    kw = MODES["rw-philox"]
    P, C = g.host_init_chains(N, kw["program_length"], 12, ops=kw["ops"])
    a, b = g.Sampler(N, **kw), g.Sampler(N, **kw)
    try:
        for s in (a, b):
            s.set_batched_data(sets)
            s.set_state(P, C)
        b.capture_blocks(4, 10)
        seeds = [9, 8, 7, 6]
        for sd_ in seeds:
            a.run_block(10, sd_)
        b.run_captured(seeds)
        _same_state(a.get_state(), b.get_state())
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("layout", [dict(K=4, onepass=0, rolled=1),
                                    dict(K=4, onepass=0, rolled=0, lockstep=5, warps_per_cta=4),
                                    dict(K=4, onepass=0, rolled=1, lockstep=0, warps_per_cta=2)],
                         ids=["rolled", "lockstep5-wpc4", "free-wpc2"])
def test_batched_layouts_equal_single_dataset_runs(layout):
    kw = MODES["rw-philox"]
    sets = _datasets([200, 33, 700], seed=17)
    cpd = 64
    N = cpd * len(sets)
    P, C = g.host_init_chains(N, kw["program_length"], 21, ops=kw["ops"])
    b = g.Sampler(N, **kw)
    try:
        b.set_batched_data(sets)
        with pytest.raises(g.GprError, match="K=4 in passes"):
            b.set_layout(8, 0, 0)
        b.set_layout(**layout)
        geo = b.launch_geometry()
        assert geo["K"] == layout["K"] and geo["rolled"] == layout["rolled"]
        b.set_state(P, C)
        b.run_block(20, 5)
        got = b.get_state()
    finally:
        b.close()
    for d, ds in enumerate(sets):
        s = g.Sampler(N, **kw)
        try:
            s.set_data(*ds)
            s.set_layout(**{**layout, "lockstep": geo["lockstep"], "warps_per_cta": geo["warps_per_cta"]})
            s.set_state(P, C)
            s.run_block(20, 5)
            lo, hi = d * cpd, (d + 1) * cpd
            _same_state(_cols(got, lo, hi), _cols(s.get_state(), lo, hi), "dataset %d" % d)
        finally:
            s.close()


@pytest.mark.parametrize("mode", ["rw-philox", "hmc"])
@pytest.mark.parametrize("batched", [False, True])
def test_autotune_leaves_the_state_and_sets_its_layout(batched, mode):
    """The autotuner's trial blocks (staged and streamed layouts; for
    Hamiltonian moves CTA shapes and residency caps) leave the chains, scores
    and counters as they were, and the layout it reports is the one the
    handle then runs."""
    kw = MODES[mode]
    N = 64 * 4
    P, C = g.host_init_chains(N, kw["program_length"], 8, ops=kw["ops"])
    s = g.Sampler(N, **kw)
    try:
        _setup(s, mode)
        if batched:
            s.set_batched_data(_datasets([90, 400, 12, 150], seed=2))
        else:
            s.set_data(*H.expdecay_data(250, seed=1))
        s.set_state(P, C)
        s.run_block(5, 1)
        before, st0 = s.get_state(), s.stats()
        t = s.autotune(steps=10, seed=3)
        _same_state(before, s.get_state())
        assert s.stats() == st0
        geo = s.launch_geometry()
        assert (geo["K"], geo["onepass"], geo["rolled"]) == (t["K"], t["onepass"], t["rolled"])
        assert t["ms"] > 0
        s.run_block(5, 2)
        s.sync()
    finally:
        s.close()


@pytest.mark.parametrize("mode,param", [(0, 0.5), (0, 0.0), (0, 0.9), (1, 20.0), (1, 0.0)])
def test_resample_per_dataset_matches_oracle(mode, param):
    """Batched data: each dataset's chains are resampled against the cutoff of
    their own posteriors; cutoffs, the chains re-drawn and their new programs
    and constants equal the oracle's per-dataset restatement bit for bit."""
    port = pytest.importorskip("oracle.port")
    sets = _datasets([50, 700, 9, 260], seed=5)
    cpd = 96
    N = cpd * len(sets)
    kw = MODES["rw-philox"]
    P0, C0 = g.host_init_chains(N, kw["program_length"], 44, ops=kw["ops"])
    s = g.Sampler(N, **kw)
    try:
        s.set_batched_data(sets)
        s.set_state(P0, C0)
        s.run_block(30, 7)
        P, C, prior, lik = s.get_state()
        n_dev, cuts_dev = s.resample_datasets(len(sets), mode, param, seed=2024)
        P1, C1, _, _ = s.get_state()
        # gpr_resample on batched data: the same per-dataset rule, NaN cutoff
        s.set_state(P, C)
        s.set_scores(prior, lik)
        n2, cut2 = s.resample(mode, param, seed=2024)
        P2, C2, _, _ = s.get_state()
    finally:
        s.close()
    Pr, Cr = P.copy(), C.copy()
    n_ref, cuts_ref = port.resample_segments(port.cfg(PL=kw["program_length"], ops=kw["ops"]), Pr, Cr, prior, lik,
                                             len(sets), mode, param, 2024)
    assert np.array_equal(cuts_dev, cuts_ref, equal_nan=True), (cuts_dev, cuts_ref)
    assert n_dev == n_ref == n2 and np.isnan(cut2)
    assert np.array_equal(P1, Pr) and np.array_equal(C1.view(np.uint32), Cr.view(np.uint32))
    assert np.array_equal(P2, Pr) and np.array_equal(C2.view(np.uint32), Cr.view(np.uint32))
    # per dataset, the cutoff is the rank rule over that dataset's chains alone
    post = prior + lik
    for d in range(len(sets)):
        seg = post[d * cpd:(d + 1) * cpd]
        srt = np.concatenate([seg[np.isnan(seg)], np.sort(seg[~np.isnan(seg)])])
        want = srt[-1] - param if mode == 1 else srt[int(cpd * param)]
        assert (np.isnan(want) and np.isnan(cuts_dev[d])) or want == cuts_dev[d]
