"""Row-sharded sigma over several ranks.

The reference distributes sigma with ZeroMQ (H_S2_u_0_nstates_zmq,
src/Davidson/davidson_parallel.irp.f:260-393): the rows are cut into tasks of
50,000 determinants (:338-366), each worker computes its task with the range
variant H_S2_u_0_nstates_openmp_work(v_t,s_t,u_t,N_st,sze,istart,iend,ishift,
istep) (:122), and a collector adds the partial vectors (:220-255).  A worker
that dies leaves its task 'running' forever and the collector blocks.

Here rank r of a torch.distributed process group owns the contiguous block
of bilinear rows [r N / world, (r+1) N / world), computes it in tasks of
50,000 rows with a row-range sigma callable (on a GB300 the C-ABI's
qpgpu_h_s2_u0_work), and one all-gather of the owned blocks (H and S^2 rows
packed together) gives every rank the whole v_t and s_t, as the reference
broadcasts the vectors to its workers (davidson_parallel.irp.f:98-104,325).
A rank that fails or leaves is detected by the process group (closed
connection or timeout) and reported as ShardError instead of a hang.  The
multi-rank logic is exercised with gloo ranks on the CPU and, with the CUDA
range sigma, with two gloo ranks sharing one GPU (tests/test_shard_gloo.py).
"""
from __future__ import annotations

import numpy as np

TASK_ROWS = 50_000  # davidson_parallel.irp.f:338-366


class ShardError(RuntimeError):
    pass


def row_tasks(n_det: int, task_rows: int = TASK_ROWS):
    """1-based (istart, iend) row blocks of the bilinear order."""
    return [(i, min(i + task_rows - 1, n_det)) for i in range(1, n_det + 1, task_rows)]


def owned_block(n_det: int, rank: int, world: int):
    """0-based half-open row block [lo, hi) of the bilinear order owned by `rank`."""
    return rank * n_det // world, (rank + 1) * n_det // world


def my_tasks(n_det: int, rank: int, world: int, task_rows: int = TASK_ROWS):
    """1-based (istart, iend) tasks of at most task_rows rows covering the owned block."""
    lo, hi = owned_block(n_det, rank, world)
    return [(i, min(i + task_rows - 1, hi)) for i in range(lo + 1, hi + 1, task_rows)]


def sharded_sigma(sigma_rows, u_t, rank: int, world: int, task_rows: int = TASK_ROWS, group=None):
    """v_t, s_t = sigma(u_t) with the rows split over `world` ranks.

    sigma_rows(u_t, istart, iend) -> (v_t, s_t): full-size arrays whose rows
    istart..iend (1-based, bilinear order) hold sigma.
    u_t: (N_det, N_st) float64 in bilinear order, identical on every rank.
    """
    import torch
    import torch.distributed as dist

    u_t = np.ascontiguousarray(u_t, dtype=np.float64)
    n, nst = u_t.shape
    lo, hi = owned_block(n, rank, world)
    width = (n + world - 1) // world  # the largest block; smaller ones are padded
    mine = np.zeros((2, width, nst))
    for i0, i1 in my_tasks(n, rank, world, task_rows):
        vv, ss = sigma_rows(u_t, i0, i1)
        mine[0, i0 - 1 - lo:i1 - lo] = vv[i0 - 1:i1]
        mine[1, i0 - 1 - lo:i1 - lo] = ss[i0 - 1:i1]
    if world == 1:
        return mine[0, :n].copy(), mine[1, :n].copy()
    parts = [torch.empty((2, width, nst), dtype=torch.float64) for _ in range(world)]
    try:
        dist.all_gather(parts, torch.from_numpy(mine), group=group)
    except Exception as e:  # a peer failed, left, or timed out
        raise ShardError(f"rank {rank}: sigma all-gather failed ({type(e).__name__}: {e})") from e
    v = np.empty_like(u_t)
    s = np.empty_like(u_t)
    for r, t in enumerate(parts):
        a, b = owned_block(n, r, world)
        x = t.numpy()
        v[a:b] = x[0, :b - a]
        s[a:b] = x[1, :b - a]
    return v, s
