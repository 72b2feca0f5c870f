"""The replicas path (N GPUs = N independent boxes) on the CPU: two gloo ranks
on 127.0.0.1 exchange only a barrier and the maximum of their times."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from heterogeneous_mhd_gb300.replicas import Replicas
    rep = Replicas("gloo")
    rep.barrier()
    ms_local = 10.0 + 5.0 * rank           # rank 1 is the slowest
    value, ms = rep.throughput(cells_per_rank=1000, steps=4, ms_local=ms_local)
    out[rank] = (rep.seed(7), value, ms, rep.max([rank, -rank]))
    rep.close()


def test_two_gloo_replicas():
    world, port = 2, _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    assert out[0][0] == 7 and out[1][0] == 8            # a box per rank
    for r in range(world):
        _, value, ms, mx = out[r]
        assert ms == 15.0                                # the slowest rank's time
        assert value == pytest.approx(world * 1000 * 4 / 15e-3)
        assert mx == [1.0, 0.0]


def test_single_process_without_launcher(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from heterogeneous_mhd_gb300.replicas import Replicas
    rep = Replicas("gloo")
    assert rep.world == 1 and rep.dist is None
    assert rep.throughput(100, 2, 4.0) == (100 * 2 / 4e-3, 4.0)
