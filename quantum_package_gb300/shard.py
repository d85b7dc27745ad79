"""Row-sharded sigma over several ranks.

The reference distributes sigma with ZeroMQ (H_S2_u_0_nstates_zmq,
src/Davidson/davidson_parallel.irp.f:260-393): the rows are cut into tasks of
50,000 determinants (:338-366), each worker computes its task with the range
variant H_S2_u_0_nstates_openmp_work(v_t,s_t,u_t,N_st,sze,istart,iend,ishift,
istep) (:122), and a collector adds the partial vectors (:220-255).  A worker
that dies leaves its task 'running' forever and the collector blocks.

Here the ranks of a torch.distributed process group take the tasks
round-robin, compute them with a row-range sigma callable (on a GB300 the
C-ABI's qpgpu_h_s2_u0_work), and one all_reduce sums the row-disjoint
results, so every rank ends with the whole v_t and s_t.  A rank that fails or
leaves is detected by the process group (closed connection or timeout) and
reported as ShardError instead of a hang.  The multi-rank logic is exercised
with gloo ranks on the CPU (tests/test_shard_gloo.py).
"""
from __future__ import annotations

import numpy as np

TASK_ROWS = 50_000  # davidson_parallel.irp.f:338-366


class ShardError(RuntimeError):
    pass


def row_tasks(n_det: int, task_rows: int = TASK_ROWS):
    """1-based (istart, iend) row blocks of the bilinear order."""
    return [(i, min(i + task_rows - 1, n_det)) for i in range(1, n_det + 1, task_rows)]


def my_tasks(n_det: int, rank: int, world: int, task_rows: int = TASK_ROWS):
    return row_tasks(n_det, task_rows)[rank::world]


def sharded_sigma(sigma_rows, u_t, rank: int, world: int, task_rows: int = TASK_ROWS, group=None):
    """v_t, s_t = sigma(u_t) with the rows split over `world` ranks.

    sigma_rows(u_t, istart, iend) -> (v_t, s_t): full-size arrays whose rows
    istart..iend (1-based, bilinear order) hold sigma; other rows are zero.
    u_t: (N_det, N_st) float64 in bilinear order, identical on every rank.
    """
    import torch
    import torch.distributed as dist

    u_t = np.ascontiguousarray(u_t, dtype=np.float64)
    n = u_t.shape[0]
    v = np.zeros_like(u_t)
    s = np.zeros_like(u_t)
    for i0, i1 in my_tasks(n, rank, world, task_rows):
        vv, ss = sigma_rows(u_t, i0, i1)
        v[i0 - 1:i1] = vv[i0 - 1:i1]
        s[i0 - 1:i1] = ss[i0 - 1:i1]
    if world == 1:
        return v, s
    tv = torch.from_numpy(v)
    ts = torch.from_numpy(s)
    try:
        dist.all_reduce(tv, group=group)
        dist.all_reduce(ts, group=group)
    except Exception as e:  # a peer failed, left, or timed out
        raise ShardError(f"rank {rank}: sigma collective failed ({type(e).__name__}: {e})") from e
    return tv.numpy(), ts.numpy()
