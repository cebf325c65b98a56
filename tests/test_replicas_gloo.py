"""The multi-rank (replica) path of the benchmark on CPU: two gloo ranks, the start
barrier, the maximum over ranks of the timed duration and the whole-job rate."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    from hybird_gb300.replicas import Replicas
    rep = Replicas()
    rep.barrier()
    t = rep.max(1.0 + rank)                 # per-rank "duration"
    rate = rep.aggregate_rate(1000, t)       # 1000 units per rank
    out.put((rep.rank, rep.world, t, rate))
    rep.close()


def test_two_gloo_ranks_agree_on_max_time_and_rate():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for _, w, t, rate in res:
        assert w == 2 and t == 2.0 and rate == 1000.0


def test_single_process_needs_no_process_group():
    from hybird_gb300.replicas import Replicas
    rep = Replicas()
    assert rep.world == 1 and rep.dist is None
    assert rep.max(3.5) == 3.5
    assert rep.aggregate_rate(10, 2.0) == 5.0
    rep.close()
