"""The resampling exchange of one population of chains spread over ranks
(gpuropolis_gb300/population.py), on CPU with the gloo backend and two
ranks: the cutoff every rank computes equals the cutoff of main.cu:1215-1219
over the concatenation of all ranks' posteriors (reference comparator: NaN
lowest), for MAP-delta and quantile modes, and each rank's chain offset is
the count of the chains before it."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")

from gpuropolis_gb300 import population as pop  # noqa: E402

SIZES = [700, 513]          # chains per rank (unequal, to exercise the padding)
CASES = [(0, 0.5), (0, 0.0), (0, 0.99), (1, 20.0), (1, 0.0)]


def _posteriors(rank, n, kind):
    r = np.random.default_rng(100 + rank)
    post = r.normal(-500, 200, n)
    if kind == "mixed":
        post[r.random(n) < 0.2] = np.nan
        post[r.random(n) < 0.1] = -np.inf
    elif kind == "nan":
        post[:] = np.nan
    return post


def _worker(rank, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        res = {"offset": pop.rank_chain_offset(SIZES[rank])}
        for kind in ("plain", "mixed", "nan"):
            post = _posteriors(rank, SIZES[rank], kind)
            for mode, param in CASES:
                res["%s-%d-%g" % (kind, mode, param)] = pop.population_cutoff(post, mode, param)
        np.save(os.path.join(out_dir, "rank%d.npy" % rank), res, allow_pickle=True)
    finally:
        dist.destroy_process_group()


class _RecordingSampler:
    """Stands in for a Sampler on a rank without a GPU: the scores it holds,
    and the (cutoff, seed, chain offset) of the re-draw it is asked for."""

    def __init__(self, prior, lik):
        self.prior, self.lik = prior, lik
        self.N = len(prior)
        self.calls = []

    def get_scores(self):
        return self.prior, self.lik

    def resample_below(self, cutoff, seed, chain_offset):
        self.calls.append((cutoff, seed, chain_offset))
        return int(np.sum(self.prior + self.lik < cutoff))


def _resample_worker(rank, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        post = _posteriors(rank, SIZES[rank], "mixed")
        s = _RecordingSampler(post * 0.25, post * 0.75)
        res = {}
        for mode, param in CASES:
            n, cut = pop.resample_population(s, mode, param, seed=99)
            res["%d-%g" % (mode, param)] = (n, cut, s.calls[-1])
        np.save(os.path.join(out_dir, "res%d.npy" % rank), res, allow_pickle=True)
    finally:
        dist.destroy_process_group()


def test_resample_population_over_two_gloo_ranks(tmp_path):
    """Each rank asks its own handle for the re-draw below the population's
    cutoff, with the shared seed and its first chain's population index; the
    ranks' re-draw counts add up to the population's count below the cutoff."""
    import torch.multiprocessing as mp
    mp.start_processes(_resample_worker, args=(_free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = [np.load(tmp_path / ("res%d.npy" % r), allow_pickle=True).item() for r in range(2)]
    allpost = np.concatenate([_posteriors(r, SIZES[r], "mixed") for r in range(2)])
    # the ranks' scores are 0.25 and 0.75 of these posteriors: their sums, as the sampler adds them
    allsum = np.concatenate([p * 0.25 + p * 0.75 for p in (_posteriors(r, SIZES[r], "mixed") for r in range(2))])
    for mode, param in CASES:
        key = "%d-%g" % (mode, param)
        cut = pop.local_cutoff(allsum, mode, param)
        total = 0
        for r in range(2):
            n, c, (call_cut, call_seed, call_off) = got[r][key]
            assert (np.isnan(cut) and np.isnan(c)) or c == cut, (key, r, c, cut)
            assert call_seed == 99 and call_off == (0 if r == 0 else SIZES[0])
            total += n
        assert total == int(np.sum(allsum < cut)), key
    assert len(allpost) == sum(SIZES)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_population_cutoff_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(_free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = [np.load(tmp_path / ("rank%d.npy" % r), allow_pickle=True).item() for r in range(2)]
    assert got[0]["offset"] == 0 and got[1]["offset"] == SIZES[0]
    for kind in ("plain", "mixed", "nan"):
        allpost = np.concatenate([_posteriors(r, SIZES[r], kind) for r in range(2)])
        srt = pop.sorted_reference_order(allpost)
        for mode, param in CASES:
            key = "%s-%d-%g" % (kind, mode, param)
            want = srt[-1] - param if mode == 1 else srt[int(len(srt) * param)]
            for r in range(2):
                v = got[r][key]
                assert (np.isnan(want) and np.isnan(v)) or v == want, (key, r, v, want)


def test_local_cutoff_is_the_single_rank_rule():
    post = np.array([np.nan, -3.0, 5.0, -np.inf, 1.0])
    assert pop.local_cutoff(post, 1, 2.0) == 3.0
    assert np.isnan(pop.local_cutoff(post, 0, 0.0))         # NaN sorts first
    assert pop.local_cutoff(post, 0, 0.5) == -3.0            # [nan, -inf, -3, 1, 5][2]
    assert pop.population_cutoff(post, 0, 0.5) == -3.0       # no process group: local rule
    assert pop.rank_chain_offset(5) == 0
