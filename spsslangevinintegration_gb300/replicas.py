"""Replica sharding across processes (one GPU each), replacing the reference's
MPI_PARAMETER_SCAN mode (one parameter point per rank,
ControlEngines/SimulationEngineFirstOrder.cpp:105-113).  Replicas are
independent: ranks exchange nothing on the data path, only the timing
maximum and, at the end, the per-replica results."""


def shard(count, world, rank):
    """Contiguous block of replica indices for `rank` (sizes differ by at most 1)."""
    base, extra = divmod(count, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value):
    """Maximum of a float over all ranks (identity without torch.distributed)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_results(local, dst=0):
    """Per-replica results of every rank, concatenated in rank order on `dst`."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(local)
    out = [None] * dist.get_world_size() if dist.get_rank() == dst else None
    dist.gather_object(list(local), out, dst=dst)
    if dist.get_rank() != dst:
        return None
    return [r for part in out for r in part]
