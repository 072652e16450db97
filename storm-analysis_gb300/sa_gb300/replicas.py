"""
Host logic of multi-GPU runs.  The LM fit does not shard: frames are
independent, so N GPUs run N replicas of the single-GPU engine, each on
its own frames, with no data-path collective.  What the ranks share is the
measurement: a barrier before the timed region, the maximum of the ranks'
times after it, and the whole-job throughput computed from that maximum.
"""
import os


def rank_env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def replica_seed(config, rank):
    """Seed of a rank's synthetic frames: every replica fits its own frames."""
    return int(config) + 1000 * int(rank)


def max_over_ranks(ms, dist=None, device="cpu"):
    """The slowest rank's time (the job is done when the last replica is)."""
    if dist is None:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, ms_per_step):
    """Whole-job units per second: every rank's units over the slowest
    rank's step time."""
    return float(units_per_rank) * int(world) / (float(ms_per_step) / 1e3)
