"""Replicas on several GPUs (one process per GPU, launched by torchrun): the
scoring path has no exchange step, so each rank scores its own seeded
replica of the workload and only the timing is combined — the whole-job
rate is the cells of all ranks over the slowest rank's time (weak scaling).
The process group carries nothing but these two reductions."""


def rank_seed(seed, rank):
    """The workload seed of a rank: distinct replicas per rank."""
    return seed + 1000 * rank


def whole_job(local_units, local_ms, world):
    """(units of all ranks, max ms over ranks) through torch.distributed
    (any backend); the local values when world == 1."""
    if world <= 1:
        return float(local_units), float(local_ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(local_ms)], dtype=torch.float64)
    u = torch.tensor([float(local_units)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return u.item(), t.item()
