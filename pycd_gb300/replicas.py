"""Replica parallelism for multi-GPU runs.

The KMC path shards into independent trajectories with no exchange step, so
N GPUs run N independent replicas: rank r owns Philox stream ids
[r * T, (r + 1) * T) and the job-wide throughput is the sum of every rank's
steps over the slowest rank's wall time.  Only this timing reduction crosses
ranks; it works over any torch.distributed backend (NCCL on GPUs, gloo on
CPU).
"""


def stream_offset(rank, n_traj_per_rank):
    """First Philox stream id of `rank`'s trajectories."""
    return int(rank) * int(n_traj_per_rank)


def aggregate(wall_s, steps, device=None):
    """(max wall over ranks, total steps over ranks); identity without a
    process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(wall_s), float(steps)
    t = torch.tensor([float(wall_s), float(steps)], dtype=torch.float64, device=device)
    parts = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, t)
    return max(float(p[0]) for p in parts), sum(float(p[1]) for p in parts)
