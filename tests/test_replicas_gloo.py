"""The replica path of bench.py on two CPU ranks (gloo): every rank times its own
independent H psi, the job reports the slowest rank's time and all ranks' bands
(one GPU per rank on a multi-GPU node; no collective on the data path)."""

from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        t_local = 0.5 + rank                        # rank 1 is the slow one
        t = bench.max_over_ranks(t_local, world)
        q.put((rank, t, bench.replica_value(64, 10, t, world)))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_report_the_slowest_rank_and_all_bands():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [1.5, 1.5]                  # both ranks see the max
    assert out[0][2] == pytest.approx(2 * 64 * 10 / 1.5)      # whole-job bands/s


def test_single_rank_is_the_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(0.7, 1) == 0.7
    assert bench.replica_value(64, 10, 0.5, 1) == pytest.approx(1280.0)


def test_reference_arm_prints_only_on_rank_zero(capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        steps, warmup = 1, 0
    bench.run_reference(A(), rank=1, world=2)
    assert capsys.readouterr().out == ""
