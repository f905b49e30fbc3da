"""The replica (N>1) measurement path on CPU: two gloo ranks, as under
torchrun. Each rank runs its own copy; the job rate is all ranks' units over
the slowest rank's time, on every rank, and only rank 0 reports."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from femx_gb300.replicas import Replicas
        rep = Replicas(dist)
        rep.barrier()
        t_local = 1.0 + rank            # rank 1 is slower
        out.put((rank, rep.reporter, rep.max_time(t_local), rep.job_rate(1000.0, t_local)))
        rep.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_benchmark():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [True, False]
    for _, _, tmax, rate in res:
        assert tmax == 2.0
        assert rate == pytest.approx(2 * 1000.0 / 2.0)


def test_single_process_is_a_no_op(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.setenv("RANK", "0")
    from femx_gb300.replicas import Replicas
    rep = Replicas(None)
    rep.barrier()
    assert rep.reporter and rep.max_time(0.5) == 0.5 and rep.job_rate(10.0, 0.5) == 20.0
