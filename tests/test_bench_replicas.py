"""The N > 1 path of bench.py on the CPU: replicas reduced by a maximum over gloo ranks.

bench.py runs one independent replica of the sweeps per rank (the VUMPS path has no data-path
exchange); the only collective is the maximum of the per-rank step times, and only rank 0
prints.  These tests run that reduction on two gloo ranks and the reference arm's rank gate.
"""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r reports step time 1 + r and wall time 10 - r: the maximum takes each from another rank
        t_step, t_wall = bench._max_over_ranks(dist, [1.0 + rank, 10.0 - rank], "cpu")
        ws, rk, _ = bench._dist()
        q.put((rank, t_step, t_wall, ws, rk))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in range(world))
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    for rank, (r, t_step, t_wall, ws, rk) in enumerate(got):
        assert (r, rk, ws) == (rank, rank, world)
        assert (t_step, t_wall) == (2.0, 10.0)


def test_reference_arm_prints_on_rank0_only(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    def fail(*a, **k):
        raise AssertionError("a non-zero rank must not time the CPU arm")

    monkeypatch.setattr(bench, "_oracle_vumps", fail)
    out = io.StringIO()
    with redirect_stdout(out):
        bench.run_reference(type("A", (), {"steps": 1, "warmup": 3})())
    assert out.getvalue() == ""


class _FakeOracle:
    """Stands in for the oracle's VUMPS: each site update takes a fixed, known time."""

    def __init__(self, dt):
        self.dt, self.calls = dt, []

    def site_update(self, nn):
        import time
        self.calls.append(nn)
        time.sleep(self.dt)


def test_reference_arm_line_on_rank0(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("LOCAL_RANK", "0")
    fake = _FakeOracle(0.02)
    made = []

    def make(name, state):
        made.append(state)
        return fake
    monkeypatch.setattr(bench, "_oracle_vumps", make)
    out = io.StringIO()
    with redirect_stdout(out):
        bench.run_reference(type("A", (), {"steps": 2, "warmup": 3})())
    line = json.loads(out.getvalue())
    assert fake.calls == [0, 1, 0, 1, 0]  # 3 untimed + 2 timed site updates, alternating sites
    assert len(made) == 3  # every cycle of two site updates starts from the start state
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["steps"] == 2
    # a step is one site update: sweeps/s = 1 / (2 x site-update time)
    assert line["value"] == pytest.approx(1.0 / (2 * 0.02), rel=0.3)
    assert line["ms_per_step"] == pytest.approx(20.0, rel=0.3)
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
