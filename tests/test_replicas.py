"""Replica timing across ranks (gloo, world size 2, CPU): every rank joins,
the slowest rank's time wins, whole-job throughput counts all ranks' units,
and a rank that never joins surfaces as an error on the others instead of a
hang."""
import datetime
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, times, out):
    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from vulkanhybridraytracer_gb300 import replicas

    assert replicas.env() == (ws, rank, rank)
    assert replicas.init("gloo")
    replicas.barrier()
    t = replicas.max_over_ranks(times[rank])
    out[rank] = (t, replicas.throughput(1000.0, t, ws))
    replicas.finalize()


def test_max_over_ranks_and_throughput():
    ws, port = 2, _free_port()
    times = [0.25, 0.5]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(ws, port, times, out), nprocs=ws, join=True)
        res = dict(out)
    for r in range(ws):
        t, thr = res[r]
        assert t == 0.5
        assert thr == pytest.approx(1000.0 * 2 / 0.5)


def _lonely(rank, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist

    try:
        dist.init_process_group("gloo", rank=rank, world_size=2, timeout=datetime.timedelta(seconds=3))
        out[rank] = "joined"
    except Exception as e:  # the peer never came: the store times out
        out[rank] = type(e).__name__


def test_missing_rank_times_out_instead_of_hanging():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_lonely, args=(port, out), nprocs=1, join=True)  # only rank 0 of 2 starts
        assert out[0] != "joined"


def test_single_rank_needs_no_process_group(monkeypatch):
    from vulkanhybridraytracer_gb300 import replicas

    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert replicas.env()[0] == 1
    assert replicas.init() is False
    assert replicas.max_over_ranks(1.5) == 1.5
    assert replicas.throughput(10.0, 2.0, 1) == 5.0
