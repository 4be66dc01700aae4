"""Independent replicas across GPUs (ALF's one-walker-per-MPI-rank model,
Documentation/performance.tex): each rank advances its own chains with its own
seeds and no data-path collective; the only exchange is the end-of-run reduction
of timings (and, in the Fortran driver, the per-bin observable sums of
observables_mod.F90:828-834, which stay on the host)."""
from __future__ import annotations

from typing import Sequence

# bit widths of the injective packing of (base, rank, chain) below
_BASE_BITS, _RANK_BITS, _CHAIN_BITS = 24, 20, 20
_MASK64 = (1 << 64) - 1


def _splitmix64_finalize(z: int) -> int:
    """The splitmix64 output function: a bijection of the 64-bit integers."""
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
    return z ^ (z >> 31)


def replica_seed(base: int, rank: int, chain: int = 0) -> int:
    """Seed of chain `chain` on rank `rank` of a run with base seed `base`.

    (base, rank, chain) is packed injectively into 64 bits (base < 2^24, rank < 2^20,
    chain < 2^20) and passed through a bijective mix, so two different triples never
    share a seed: no (base, rank) pair can land on another run's or another rank's
    chains.  Values outside those ranges raise ValueError."""
    if not (0 <= base < (1 << _BASE_BITS) and 0 <= rank < (1 << _RANK_BITS) and 0 <= chain < (1 << _CHAIN_BITS)):
        raise ValueError(f"replica_seed({base}, {rank}, {chain}): base < 2^24, rank and chain < 2^20 required")
    packed = (base << (_RANK_BITS + _CHAIN_BITS)) | (rank << _CHAIN_BITS) | chain
    return _splitmix64_finalize(packed)


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
