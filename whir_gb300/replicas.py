"""Replica parallelism across GPUs: proofs are independent, so N ranks (one process per GPU) each run
their own prover on their own share of the jobs. There is no data-path collective; the only
cross-rank steps are a barrier around the timed region and a max over ranks of the elapsed time."""


def shard(n_jobs, rank, world):
    """Job indices owned by `rank`: round-robin, so every job is owned by exactly one rank and the
    shares differ by at most one job."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(range(rank, n_jobs, world))


def max_over_ranks(dist, value):
    """Max of a float over all ranks of an initialised torch.distributed group (identity when
    `dist` is None)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
