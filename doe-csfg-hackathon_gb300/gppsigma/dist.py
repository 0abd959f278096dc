"""Multi-rank bookkeeping for runs with one process per GPU.

GPP sigma states are independent: by default each rank runs its own state
(seed offset by rank) and nothing on the data path is exchanged; only the
timing is combined -- the job's time is the slowest rank's.  One state can
also be sharded by G' rows (row_range); then the per-rank partial sums are
the one exchange step, added on rank 0 in rank order (fixed order, so the
result does not depend on arrival order).
"""
from __future__ import annotations

import os


def env() -> tuple[int, int, int]:
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def row_range(ngpown: int, rank: int, world: int) -> tuple[int, int]:
    """G' rows [r0, r1) of one state handled by `rank` when the state is
    sharded across ranks, as the reference's MPI version splits its my_igp
    loop (gppMPIOpenMP3.cpp:171-172, partial sums reduced at :360-370).
    Ranges are contiguous and start on even rows, so each rank's rows form
    whole row pairs of the mixed-precision tiles."""
    pairs = (ngpown + 1) // 2
    p0, p1 = pairs * rank // world, pairs * (rank + 1) // world
    return min(2 * p0, ngpown), min(2 * p1, ngpown)


def rank_rows_inputs(shape, seed: int, rank: int, world: int, device="cuda"):
    """One rank's share of a state sharded by G' rows: rows row_range(...) of
    I_eps / wtilde / inv_igp_index, generated where they are used, plus the
    band arrays every rank needs.  The rank holds its rows only (about
    1/world of the G'-indexed arrays).  Returns (inputs, (r0, r1))."""
    from . import ops
    r0, r1 = row_range(shape.ngpown, rank, world)
    return ops.device_inputs(shape, seed, device=device, rows=(r0, r1)), (r0, r1)


def state_seed(base: int, rank: int) -> int:
    """Seed of the independent state a rank runs."""
    return base + 1000003 * rank


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Maximum of a per-rank float (e.g. milliseconds per step)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds_per_rank: float, dist=None, device=None) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    ws = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    slowest = max_over_ranks(seconds_per_rank, dist, device)
    return ws * units_per_rank / slowest


def sum_in_rank_order(partial, dist=None, device=None):
    """Sum a per-rank complex128 array on rank 0 in rank order 0, 1, 2, ...
    Returns the sum on rank 0 and None elsewhere."""
    import numpy as np
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return np.array(partial, dtype=np.complex128)
    import torch
    ws, rank = dist.get_world_size(), dist.get_rank()
    local = torch.view_as_real(torch.as_tensor(np.asarray(partial, dtype=np.complex128))).to(device)
    gathered = [torch.empty_like(local) for _ in range(ws)] if rank == 0 else None
    dist.gather(local, gathered, dst=0)
    if rank != 0:
        return None
    total = np.zeros(local.shape[0], dtype=np.complex128)
    for r in range(ws):
        g = gathered[r].cpu().numpy()
        total = total + (g[:, 0] + 1j * g[:, 1])
    return total
