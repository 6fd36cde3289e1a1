"""Multi-GPU = independent replicas (the path has no exchange step: every
request, right-hand side and Newton amplitude is an independent unit).
One process per GPU; the only cross-rank operation is the timing
aggregate: the maximum of the per-rank step times (a barrier plus one
all-reduce of a scalar, outside the solves)."""
import torch
import torch.distributed as dist


def max_over_ranks(value: float, device=None) -> float:
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
