"""Multi-GPU by replicas: independent units (random vectors, disorder instances)
are split across ranks with no per-step exchange; the only communication is
one sum of the M-length (or M x M) moment arrays at the end and the max of the
ranks' times.  The reference is single-process and averages vectors in a
caller loop; this is that loop spread over ranks.

Works with any torch.distributed backend (NCCL on GPUs, gloo on CPU tensors);
with no process group initialised every function acts on the single process.
"""
from __future__ import annotations

import numpy as np


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def world():
    d = _dist()
    return (d.get_rank(), d.get_world_size()) if d else (0, 1)


def split_range(n_units, rank, world_size):
    """Contiguous block [lo, hi) of n_units for `rank` (sizes differ by at most one)."""
    base, extra = divmod(int(n_units), int(world_size))
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def vector_seeds(R_total, rank, world_size, seed0=1000):
    """Seeds of this rank's share of R_total random vectors (seed0 + global index)."""
    lo, hi = split_range(R_total, rank, world_size)
    return [seed0 + i for i in range(lo, hi)]


def sum_over_ranks(x):
    """Sum a torch tensor (or numpy array) over ranks; returns the same kind."""
    import torch

    d = _dist()
    if d is None:
        return x
    was_np = not isinstance(x, torch.Tensor)
    t = torch.as_tensor(np.ascontiguousarray(x)) if was_np else x
    if t.is_complex():
        r = torch.view_as_real(t).contiguous()
        d.all_reduce(r)
        t = torch.view_as_complex(r)
    else:
        t = t.contiguous()
        d.all_reduce(t)
    return t.numpy() if was_np else t


def max_over_ranks(value, device=None):
    import torch

    d = _dist()
    if d is None:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def mean_moments(local_mu_sum, R_total):
    """Average of per-vector moments: local sums (over this rank's vectors) summed over ranks / R_total."""
    return sum_over_ranks(local_mu_sum) / float(R_total)
