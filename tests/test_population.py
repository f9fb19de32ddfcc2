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
