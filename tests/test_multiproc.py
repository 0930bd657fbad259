"""Replicas-only multi-GPU path of bench.py, exercised on the CPU with two gloo
ranks: every rank times its own replica, the job time is the slowest rank's
(all_reduce MAX) and the whole-job throughput counts every rank's DOFs. The
CPU oracle stands in for the per-rank work, so each rank also checks that its
replica computes the same result as the other's."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from mfem_gb300 import fem
    from tests import oracle_lib
    # per-rank replica: identical problem, oracle apply as the rank's work
    o = oracle_lib.load()
    m = fem.CartesianMesh(3, jitter=0.1, seed=1)
    sp = fem.H1Space(m, 2)
    t = fem.Tables(2, 4)
    off, ind, gm = o.restriction_build(m.ne, 27, sp.ndofs, sp.element_dofs(), None)
    gt = fem.Tables(1, 4)
    J = o.geom_jacobians3d(m.ne, 2, 4, gt.B, gt.G, m.nodes_evector(1))
    qd = o.diffusion_setup3d(m.ne, 4, 1, t.W, J, np.array([1.0]))
    y = o.pa_mult(0, m.ne, sp.ndofs, True, 3, 4, gm, off, ind, t.B, t.G, qd, np.ones(sp.ndofs))
    ys = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(ys, torch.tensor([float(np.abs(y).sum())], dtype=torch.float64))
    my_ms = 10.0 + 5.0 * rank
    job_ms = bench.max_over_ranks(my_ms, world)
    value = bench.job_throughput(sp.ndofs, 4, world, job_ms)
    q.put((rank, job_ms, value, [float(v) for v in ys]))
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world = 2
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, job_ms, value, ys in res:
        assert job_ms == 15.0                      # the slowest rank
        assert ys[0] == ys[1]                      # identical replicas
    ndofs = (2 * 3 + 1) ** 3
    assert abs(res[0][2] - 2 * ndofs * 4 / 15e-3 / 1e9) < 1e-15
