"""Replica coordination for several GPUs of one node (one process per GPU).

The deconvolution path has no exchange step: images, channels, facets and
requests are independent, so N GPUs run N replicas, each on its own images,
with no collective on the data path. The only cross-rank traffic is timing:
every rank brackets its timed region with a barrier and the job's time is the
slowest rank's (max over ranks), from which the whole-job throughput follows.
"""
import torch


def reduce_max(values, dist=None, device="cpu"):
    """Element-wise maximum of ``values`` (floats) over all ranks; the local values when not distributed."""
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job_rate(units_per_rank, world, seconds_max):
    """Units per second of the whole job: every rank processed units_per_rank in at most seconds_max."""
    return world * units_per_rank / seconds_max


def rank_seed(base, rank):
    """Seed of a rank's own images (weak scaling: each rank a different, equally sized set)."""
    return base + 7919 * rank
