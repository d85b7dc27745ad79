"""Row-sharded sigma on two gloo ranks, with an injected rank failure.

Each rank computes the tasks of its row block with a range sigma -- the CPU
oracle's restatement of H_S2_u_0_nstates_openmp_work, or (marked gpu) the
CUDA qpgpu_h_s2_u0_work, both ranks sharing the one GPU -- and one all-gather
of the owned blocks gives every rank the whole result, which must equal the
one-rank result to 1e-12.  The failure case makes rank 1 raise before the
collective: rank 0 must report a ShardError instead of hanging.
"""
import datetime
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, fail_rank, outdir, backend="oracle"):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    from oracle import Oracle
    from quantum_package_gb300 import generate as G
    from quantum_package_gb300.shard import ShardError, sharded_sigma

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    p = G.make_problem(1, n_det=3000)
    u = G.random_coefficients(p.n_det, 2, 5)
    if backend == "cuda":
        import torch
        from quantum_package_gb300.sigma import Wavefunction
        torch.cuda.set_device(0)
        o = Wavefunction.from_problem(p)
        u_t = np.ascontiguousarray(u[:, o.bilinear_order()].T)

        def rows(uu, i0, i1):
            return o.H_S2_u_0_nstates_openmp_work(uu, i0, i1, 0, 1)
    else:
        o = Oracle.from_problem(p)
        u_t = np.ascontiguousarray(u[:, o.bilinear()["order"] - 1].T)

        def rows(uu, i0, i1):
            return o.h_s2_u0_work(uu, i0, i1, 0, 1)

    status = "ok"
    try:
        if rank == fail_rank:
            raise RuntimeError("injected failure")
        v, s = sharded_sigma(rows, u_t, rank, world, task_rows=700)
        vf, sf = rows(u_t, 1, p.n_det)
        err = max(np.abs(v - vf).max(), np.abs(s - sf).max())
        status = f"ok {err:.3e}"
    except ShardError as e:
        status = f"shard_error {e}"
    except RuntimeError as e:
        status = f"raised {e}"
    with open(os.path.join(outdir, f"rank{rank}.txt"), "w") as f:
        f.write(status)
    if rank != fail_rank:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, fail_rank, tmp_path, backend="oracle"):
    ctx = mp.get_context("spawn")
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, fail_rank, str(tmp_path), backend))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        if p.is_alive():
            p.kill()
            pytest.fail("rank did not finish")
    return [open(tmp_path / f"rank{r}.txt").read() for r in range(world)]


def test_two_ranks_match_single_rank(tmp_path):
    out = _run(2, -1, tmp_path)
    for s in out:
        assert s.startswith("ok"), s
        assert float(s.split()[1]) < 1e-12


def test_failed_rank_is_detected(tmp_path):
    out = _run(2, 1, tmp_path)
    assert out[1].startswith("raised injected failure")
    assert out[0].startswith("shard_error"), out[0]


@pytest.mark.gpu
def test_two_ranks_cuda_range_sigma_match_single_rank(tmp_path):
    out = _run(2, -1, tmp_path, backend="cuda")
    for s in out:
        assert s.startswith("ok"), s
        assert float(s.split()[1]) < 1e-12
