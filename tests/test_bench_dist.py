"""The multi-process host logic of bench.py (replicas only: one process per GPU,
no data exchange, job time = the slowest rank's), run as two gloo ranks on CPU."""
from __future__ import annotations

import importlib.util
import os
import socket
import sys

import pytest

from conftest import ROOT


def _bench():
    spec = importlib.util.spec_from_file_location("isg_bench", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["isg_bench"] = mod
    spec.loader.exec_module(mod)
    return mod


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = _bench()
        ws, r, local = b.dist_info()
        mx = b.max_over_ranks(10.0 + 5.0 * rank)       # rank 1 is the slowest
        v = b.job_flips_per_ns(1000, 20, ws, mx)
        out.put((r, ws, local, mx, v))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    for _, _, _, mx, v in got:
        assert mx == 15.0                                # max over ranks
        assert v == pytest.approx(1000 * 20 * 2 / (15.0 * 1e6))


def test_single_process_needs_no_process_group():
    b = _bench()
    assert b.max_over_ranks(3.5) == 3.5
    assert b.job_flips_per_ns(76693504, 10, 1, 1.0) == pytest.approx(766.93504)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys):
    """Under torchrun only rank 0 times the reference CPU path; the others exit 0."""
    b = _bench()
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    args = type("A", (), {"gpus": 2, "steps": 1, "warmup": 3, "ref_seconds": 1.0})()
    assert b.run_reference(args) == 0
    assert capsys.readouterr().out == ""
