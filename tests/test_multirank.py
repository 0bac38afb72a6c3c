"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2).

The hot path does not exchange data between GPUs (replicas: each rank
advances its own box), so the multi-rank logic is the host's: the whole
job's time is the slowest rank's (max over ranks), the value counts every
rank's cells, and the reference arm runs on rank 0 alone."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # per-rank timings: rank r measured (r + 1) ms and (10 - r) ms
        res = bench.max_over_ranks([rank + 1.0, 10.0 - rank], world, device="cpu")
        out.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_on_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    del torch
    # every rank sees the slowest rank's time for each quantity
    assert got[0] == got[1] == [2.0, 10.0]


def test_single_rank_is_identity():
    assert bench.max_over_ranks([3.5, 1.25], 1) == [3.5, 1.25]


def test_whole_job_rate_counts_every_rank():
    # 2 ranks x 256^3 cells x 20 cycles in 2.7 s
    v = bench.whole_job_rate(256**3, 20, 2, 2.7)
    assert v == pytest.approx(2 * 256**3 * 20 / 2.7)
    assert bench.whole_job_rate(256**3, 20, 4, 2.7) == pytest.approx(2 * v)


def test_reference_arm_runs_on_rank_zero_only():
    class Args:
        steps, warmup, gpus = 1, 1, 2

    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(Args(), 2, 1) is None  # rank 1: no work, no line
    assert buf.getvalue() == ""


def test_dist_setup_reads_the_launcher_environment(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.dist_setup() == (2, 1, 1)


def test_reference_arm_line_matches_our_arms_contract():
    """--impl reference: the same metric, unit, direction and config as our
    arm's line, a cpu_baseline describing the run and an e2e with no copies"""
    import json

    class Args:
        steps, warmup, gpus, size = 1, 1, 1, 24

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args(), 1, 0)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["config"] == bench.workload_config(24, "fp64", bench.state_bytes_of(24))
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT,
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_state_bytes_formula_matches_the_arrays():
    from idefix_gb300 import ic

    Vc, Vs = ic.turbulence_3d(16, seed=1)
    assert bench.state_bytes_of(16) == Vc.nbytes + Vs.nbytes
