"""Ensembles on several GPUs: every rank solves its own samples, with no
exchange between ranks, as ParameterStudy::run distributes its runs over
ranks (cpp/memilio/compartments/parameter_studies.h:173-213). The job's time
is the slowest rank's; its throughput is all ranks' work over that time.
One process per GPU (torchrun); the same functions run on CPU with gloo."""
from __future__ import annotations

from . import workloads as W

# seed stride between ranks: every rank draws an independent stream of samples
RANK_SEED_STRIDE = 7919


def ensemble_for_rank(num_samples: int, rank: int, seed: int = 2, base=None, **kw):
    """The samples of rank `rank`; rank 0 gets exactly the single-GPU ensemble."""
    return W.ensemble(num_samples=num_samples, seed=seed + RANK_SEED_STRIDE * rank, base=base, **kw)


def max_over_ranks(value: float, device: str = "cpu") -> float:
    """Largest value over all ranks of the default process group (the job's time)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(work_per_rank: float, seconds_max: float, world: int) -> float:
    """Weak scaling: every rank does work_per_rank; the job ends with the slowest rank."""
    return world * work_per_rank / seconds_max
