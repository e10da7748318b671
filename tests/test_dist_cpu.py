"""The N > 1 path of bench.py on CPU: two gloo ranks on 127.0.0.1.

bench.py runs one replica per rank ("replicas only": the single-graph path
has no data-path collective); what it needs from the process group is the
barrier and the slowest rank's time.  These tests drive those helpers with
two real ranks, and check that the reference arm does no work on rank 1.
"""
from __future__ import annotations

import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out) -> None:
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.dist_barrier()
    # rank r "took" (r + 1) seconds for 10 steps of 1e9 edges
    t = bench.dist_max(float(rank + 1))
    v = bench.job_gteps(10**9, world, t, 10)
    assert bench.dist() == (world, rank, rank)
    out.put((rank, t, v))
    bench.dist_barrier()
    tdist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(world))
    for rank, t, v in res:
        assert t == 2.0  # max over ranks
        # 2 ranks x 1e9 edges per step, 10 steps in 2 s
        assert v == pytest.approx(2 * 1e9 / 0.2 / 1e9)


def test_single_rank_helpers_are_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert not tdist.is_initialized()
    assert bench.dist_max(3.5) == 3.5
    bench.dist_barrier()
    assert bench.job_gteps(263434267, 1, 0.769e-3, 1) == pytest.approx(342.57, rel=1e-3)


def test_reference_arm_does_nothing_on_rank_1(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = bench.argparse.Namespace(steps=1, warmup=1, gpus=2)
    bench.run_reference(args)
    assert capsys.readouterr().out == ""


def _shard_rank_main(rank: int, world: int, port: int, out) -> None:
    """One rank of a sharded batch: its graphs by the shared plan, labels
    computed on the CPU (the oracle stands in for the rank's GPU run), then
    the host gather to rank 0."""
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    import numpy as np

    import connectivity_gb300 as gb
    from connectivity_gb300 import shard
    import oracle
    ns, efs, seeds = gb.batch_sizes(30, median=200.0, n_max=3000)
    graphs = [oracle.rmat_edges_n(int(n), int(e), int(s)) for n, e, s in zip(ns, efs, seeds)]
    of, _ = shard.plan(shard.graph_costs(ns, [g[1].size for g in graphs]), world)
    mine = [oracle.scc(oracle.CpuGraph(*graphs[int(i)])) for i in shard.members(of, rank)]
    got = shard.gather_ranks(mine, of, rank, world)
    if rank == 0:
        ok = all(np.array_equal(lab, oracle.scc(oracle.CpuGraph(*g)))
                 for g, lab in zip(graphs, got))
        out.put((rank, len(got), ok, int((of == 1).sum())))
    else:
        out.put((rank, None, got is None, len(mine)))
    tdist.destroy_process_group()


def test_sharded_batch_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(world))
    (r0, count, ok0, n1), (r1, _, ok1, mine1) = res
    assert (r0, r1) == (0, 1)
    assert count == 30 and ok0 and ok1
    assert n1 == mine1 > 0  # rank 1 ran exactly the graphs the plan gave it
