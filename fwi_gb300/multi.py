"""Shots split over ranks (one process per GPU), with the reference's one
exchange step.

calculate_misfit_gradient spreads the shots over MPI ranks and then sums the
gradient and the misfit over them (MPI_REDUCE + MPI_BCAST,
calculate_misfit_gradient.f90:299-300 and :339-340).  Here every rank holds a
contiguous range of the survey's shots (balanced by padded grid size), runs
its own device-resident survey, and the ranks sum-allreduce the FP64 gradient
stack and the misfit (NCCL for CUDA tensors, gloo on the host); every rank
then applies the survey's finalisation (Grad = Grad + stack/numtasks, water
rows zeroed) with the same arithmetic as the device kernel, so one rank
reproduces the single-process gradient bit for bit.
"""
from __future__ import annotations

import copy
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .survey import SurveySpec


def shot_weights(spec: SurveySpec) -> List[float]:
    """Relative cost of each shot: its padded grid cells (the step kernels'
    bytes per time step scale with them)."""
    dn = spec.dpml + 2 * spec.acc
    return [float((spec.ny + 2 * dn) * (sh.nx + 2 * dn)) for sh in spec.shots]


def shard_ranges(weights: Sequence[float], world: int) -> List[Tuple[int, int]]:
    """Contiguous shot ranges [a, b), one per rank, that minimise the largest
    total weight of a rank (bisection on that bound with a greedy fill; ranks
    may get empty ranges when there are fewer shots than ranks)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = [float(x) for x in weights]
    n = len(w)

    def fill(cap):
        cuts, a, acc = [], 0, 0.0
        for i, x in enumerate(w):
            if acc + x > cap and i > a:
                cuts.append((a, i))
                a, acc = i, 0.0
            acc += x
        cuts.append((a, n))
        return cuts

    if n == 0:
        return [(0, 0)] * world
    lo, hi = max(w), sum(w)
    for _ in range(100):
        if hi - lo <= 1e-9 * hi:
            break
        mid = 0.5 * (lo + hi)
        if len(fill(mid)) <= world:
            hi = mid
        else:
            lo = mid
    cuts = fill(hi)
    while len(cuts) < world:
        cuts.append((n, n))
    return cuts


def shard_spec(spec: SurveySpec, rank: int, world: int) -> Tuple[SurveySpec, Tuple[int, int]]:
    """This rank's survey: the same model and time axis, its range of shots."""
    a, b = shard_ranges(shot_weights(spec), world)[rank]
    local = copy.copy(spec)
    local.shots = list(spec.shots[a:b])
    return local, (a, b)


def finalize(grad: np.ndarray, stack: np.ndarray, numtasks: int, water_rows: Optional[np.ndarray]) -> np.ndarray:
    """Grad = Grad + float32(stack / numtasks), rows 1..water_rows(i) of column i
    zeroed: the device finalisation's arithmetic (a double division rounded to
    float, then a float add), in place on the (ny, nx_model) float32 array."""
    add = (np.asarray(stack, np.float64) / np.float64(numtasks)).astype(np.float32)
    grad[...] = grad + add
    if water_rows is not None:
        rows = np.arange(grad.shape[0])[:, None]
        grad[rows < np.asarray(water_rows)[None, :]] = 0.0
    return grad


def _device(group):
    import torch
    import torch.distributed as dist

    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def allreduce_misfit(misfit: float, group=None) -> float:
    """Sum of the misfits of all ranks of `group`."""
    import torch
    import torch.distributed as dist

    m = torch.tensor([float(misfit)], dtype=torch.float64, device=_device(group))
    dist.all_reduce(m, op=dist.ReduceOp.SUM, group=group)
    return float(m.item())


def allreduce_stack(stack: np.ndarray, misfit: float, group=None) -> Tuple[np.ndarray, float]:
    """Sum the FP64 stacks and misfits of all ranks of `group`: on the current
    CUDA device for NCCL, on the host for gloo."""
    import torch
    import torch.distributed as dist

    flat = np.asarray(stack, np.float64).reshape(-1, order="F")
    t = torch.from_numpy(np.ascontiguousarray(flat)).to(_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy().reshape(stack.shape, order="F"), allreduce_misfit(misfit, group)


def misfit_gradient(survey, spec: SurveySpec, step: int = 1, grad: Optional[np.ndarray] = None,
                    misfit: float = 0.0, group=None) -> Tuple[float, Optional[np.ndarray]]:
    """calculate_misfit_gradient over the ranks of `group`: `survey` is this
    rank's Survey (built on shard_spec's shots; None for a rank without
    shots, which still takes part in the sums), `spec` the whole survey (its
    numtasks and water rows).  Returns (misfit + the survey's misfit, grad),
    grad updated in place on every rank for step 1."""
    m_local = survey.run(step, None)[0] if survey is not None else 0.0
    if step != 1:
        return misfit + allreduce_misfit(m_local, group), grad
    stack = survey.stack() if survey is not None else np.zeros((spec.ny, spec.nx_model), np.float64, order="F")
    total, m = allreduce_stack(stack, m_local, group)
    if grad is not None:
        finalize(grad, total, spec.numtasks, spec.water_rows)
    return misfit + m, grad
