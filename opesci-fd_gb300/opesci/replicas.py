"""Replicas on several GPUs: the elastic path has no exchange step, so N
GPUs run N independent simulations (one process per GPU, launched by
torchrun).  Shots and requests are independent units and are split across
ranks without any collective on the data path; the only collective is the
timing reduction (slowest rank) of the benchmark.
"""
import os


def rank_env():
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get('RANK', '0')), int(os.environ.get('WORLD_SIZE', '1')),
            int(os.environ.get('LOCAL_RANK', '0')))


def shard(items, rank, world):
    """This rank's share of independent units (round robin, so that
    log-uniform sizes spread evenly)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError('rank %d outside a world of %d' % (rank, world))
    return list(items)[rank::world]


def max_over_ranks(value, dist=None, device='cpu'):
    """The largest ``value`` over all ranks (the job's time is the slowest
    rank's); ``dist`` is torch.distributed (None or one rank: value)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, seconds, dist=None, device='cpu'):
    """Whole-job throughput: the units of all ranks over the slowest rank's
    time (weak scaling: every rank does the same work)."""
    world = dist.get_world_size() if (dist is not None and dist.is_initialized()) else 1
    t = max_over_ranks(seconds, dist, device)
    return units_per_rank * world / t, t
