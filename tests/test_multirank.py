"""The N > 1 path of bench.py on CPU (gloo, world size 2): cells are
independent, so ranks are replicas with no data-path collective; the only
collective is the max over ranks of the step time, and the reference arm runs
on rank 0 alone."""
import os
import sys

import pytest

from conftest import ROOT


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each replica timed its own step; the job's step is the slowest one
        t = bench.max_over_ranks(100.0 + 10.0 * rank)
        ws, r, local = bench.dist_info()
        q.put((rank, t, ws, r, local))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_rank_info_with_gloo():
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [110.0, 110.0]
    assert [(g[2], g[3], g[4]) for g in got] == [(2, 0, 0), (2, 1, 1)]


def test_max_over_ranks_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    bench.main()
    assert capsys.readouterr().out == ""


def test_reference_arm_line(monkeypatch, capsys):
    """Rank 0 of the reference arm prints one JSON line with the contract's
    keys: the CPU integrator (the reference core where it is built, else the
    oracle port, then with a note) on a bounded sample of the headline field."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                                      "--cpu-seconds", "1"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "cells/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["jacobians_per_cell"] > 1 and cb["single_core"] > 0
    assert "note" in cb and cb["note"].startswith("oracle port") == (cb["kind"] == "port")
    assert line["config"]["workload"] == "counterflow_53s"
    # the same config keys as the GPU arm's line, and a measured step time
    for k in ("cells", "species", "reactions", "solver", "precision", "jacobian", "dt", "abs_tol", "rel_tol"):
        assert k in line["config"], k
    assert 0 < line["ms_per_step"] < 60e3
