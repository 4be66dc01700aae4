"""Independent replicas across GPUs (ALF's one-walker-per-MPI-rank model,
Documentation/performance.tex): each rank advances its own chains with its own
seeds and no data-path collective; the only exchange is the end-of-run reduction
of timings (and, in the Fortran driver, the per-bin observable sums of
observables_mod.F90:828-834, which stay on the host)."""
from __future__ import annotations

from typing import Sequence


def replica_seed(base: int, rank: int, chain: int = 0) -> int:
    """Seed of chain `chain` on rank `rank` (distinct across ranks and chains)."""
    return base + 1000 * rank + chain


def max_over_ranks(values: Sequence[float], device=None) -> list:
    """Element-wise maximum over all ranks of the initialised process group (the
    slowest rank sets the whole-job time).  Works on the gloo (CPU tensors) and
    nccl (device tensors) backends; without a process group returns the input."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor(list(values), dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def whole_job_rate(world_size: int, chains_per_rank: int, sweeps: int, t_max: float) -> float:
    """Aggregate sweeps/s of all chains on all ranks over the slowest rank's time."""
    return world_size * chains_per_rank * sweeps / t_max
