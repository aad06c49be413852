"""Independent replicas across ranks: one crystal (or batch, or request
stream) per GPU, no exchange of simulation data.

The solver path does not shard in the reference (one simulation per solver
object, simulation/base_solver.py:224-280), and the benchmark workloads are
independent crystals, so several GPUs run several simulations.  The only
collectives are on the timing: the slowest rank's time and the sum of the
work make the whole-job rate (weak scaling).
"""
from __future__ import annotations


def rank_seed(rank: int, base: int = 0) -> int:
    """Seed of the crystal a rank simulates (each rank its own crystal)."""
    return base + rank


def aggregate(ms: float, work: float, dist=None):
    """(max of ms over ranks, sum of work over ranks, work / max ms).

    dist: torch.distributed when a process group is initialised (NCCL: CUDA
    tensors; gloo: CPU tensors), else None for a single process.
    """
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return ms, work, work / ms if ms > 0 else 0.0
    import torch

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t_ms = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    t_work = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(t_ms, op=dist.ReduceOp.MAX)
    dist.all_reduce(t_work, op=dist.ReduceOp.SUM)
    m, w = float(t_ms.item()), float(t_work.item())
    return m, w, w / m if m > 0 else 0.0
