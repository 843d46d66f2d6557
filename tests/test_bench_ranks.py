"""bench.py's multi-rank host logic on CPU (gloo, world size 2): the box does
not shard, so N ranks are N independent replicas and the only collective is
the max over ranks of the timed region; under torchrun the reference arm
runs on rank 0 alone and the other ranks exit without output."""
import contextlib
import io
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        q.put((rank, bench.slowest_rank_ms(10.0 + 5.0 * rank, world, torch, "cpu")))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 15.0, 1: 15.0}  # every rank reports the slower rank's time


def test_single_rank_needs_no_collective():
    import torch

    import bench

    assert bench.slowest_rank_ms(12.5, 1, torch, "cpu") == 12.5


def test_reference_arm_prints_on_rank_zero_only(monkeypatch):
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = bench.argparse.Namespace(workload="eam_al_256k", ncell=0, steps=1, warmup=0)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(args)
    assert out.getvalue() == ""


def test_reference_arm_line_keeps_the_contract(oracle_lib, monkeypatch):
    """Rank 0 of the reference arm prints one JSON line with the base keys,
    impl "reference", both rebuild policies, a cpu_baseline describing the
    run and an e2e object with no host-device bytes (LJ Ar 4000, the oracle
    port on this host)."""
    import json

    import bench

    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    args = bench.argparse.Namespace(workload="lj_ar_4000", ncell=0, steps=1, warmup=0)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(args)
    lines = [ln for ln in out.getvalue().splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == bench.UNIT and d["metric"] == bench.METRIC
    assert set(d["rebuild_policies"]) == {"every_step", "refresh_10"}
    assert d["value"] == max(p["value"] for p in d["rebuild_policies"].values())
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
