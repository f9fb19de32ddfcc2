"""One population of chains spread over several GPUs (one handle per rank):
the exchange of the reference's outer loop, whose resampling cutoff is taken
over every chain (main.cu:1215-1219), with the re-draw itself staying on each
rank's device (gpr_resample_below).

  * MAP-delta (mode 1): the largest posterior over all ranks minus delta, one
    all_reduce(MAX) of a double (and of a count, for the all-NaN case);
  * quantile (mode 0): the posterior at ascending rank int(N_total * q) in the
    reference's comparator order (NaN lowest, main.cu:987-995), from an
    all_gather of every rank's posteriors (8 bytes per chain).

Each rank then re-draws its own chains below the cutoff with the streams of
their population-wide indices, so that the ranks together do exactly what
one handle holding every chain would.  torch.distributed is the transport
(NCCL between GPUs, gloo on CPU); without an initialised process group the
functions work on the local chains alone.
"""
import math

import numpy as np


def _dist(group):
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return None
    return dist


def _device(dist, group):
    import torch
    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def sorted_reference_order(post):
    """Posteriors in the reference comparator's ascending order: NaN first."""
    post = np.asarray(post, np.float64)
    nan = np.isnan(post)
    return np.concatenate([post[nan], np.sort(post[~nan])])


def local_cutoff(post, mode, param):
    """The cutoff of main.cu:1215-1219 over these chains alone."""
    s = sorted_reference_order(post)
    if len(s) == 0:
        return math.nan
    if mode == 1:
        return s[-1] - param
    return s[int(len(s) * param)]


def rank_chain_offset(n_local, group=None):
    """Index of this rank's first chain in the population: the chains of the
    ranks before it."""
    dist = _dist(group)
    if dist is None:
        return 0
    import torch
    dev = _device(dist, group)
    n = torch.tensor([int(n_local)], dtype=torch.int64, device=dev)
    sizes = [torch.zeros_like(n) for _ in range(dist.get_world_size(group))]
    dist.all_gather(sizes, n, group=group)
    me = dist.get_rank(group)
    return int(sum(int(s.item()) for s in sizes[:me]))


def population_cutoff(post_local, mode, param, group=None):
    """The resampling cutoff over the posteriors of every rank's chains
    (mode 1: MAP - param; mode 0: the param-quantile), the same on every rank."""
    if mode not in (0, 1):
        raise ValueError("mode must be 0 (quantile) or 1 (MAP-delta)")
    post = np.ascontiguousarray(post_local, np.float64)
    dist = _dist(group)
    if dist is None:
        return local_cutoff(post, mode, param)
    import torch
    dev = _device(dist, group)
    if mode == 1:
        finite = post[~np.isnan(post)]
        v = torch.tensor([finite.max() if finite.size else -math.inf, float(finite.size)],
                         dtype=torch.float64, device=dev)
        m = v[:1].clone()
        c = v[1:].clone()
        dist.all_reduce(m, op=dist.ReduceOp.MAX, group=group)
        dist.all_reduce(c, op=dist.ReduceOp.SUM, group=group)
        if c.item() == 0:
            return math.nan          # every posterior NaN: the last in comparator order is NaN
        return m.item() - param
    world = dist.get_world_size(group)
    n = torch.tensor([post.size], dtype=torch.int64, device=dev)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    sizes = [int(s.item()) for s in sizes]
    buf = torch.full((max(sizes),), math.nan, dtype=torch.float64, device=dev)
    buf[:post.size] = torch.from_numpy(post).to(dev)
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    everything = np.concatenate([p[:k].cpu().numpy() for p, k in zip(parts, sizes)])
    return local_cutoff(everything, mode, param)


def resample_population(sampler, mode, param, seed, group=None):
    """Resample one handle's chains as part of the population: the cutoff over
    every rank's chains, then the re-draw of this handle's chains below it
    with their population-wide streams.  Returns (re-drawn here, cutoff)."""
    prior, lik = sampler.get_scores()
    cut = population_cutoff(prior + lik, mode, param, group)
    off = rank_chain_offset(sampler.N, group)
    return sampler.resample_below(cut, seed, off), cut
