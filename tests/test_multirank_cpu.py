"""The multi-GPU path of bench.py on CPU: two gloo ranks on 127.0.0.1.  Chains shard by
rank with no data-path collective (each rank gets its own occupations and Philox seeds);
the only exchange is the reduction of the timed region to the slowest rank, from which the
whole-job throughput is taken; the reference arm runs on rank 0 only."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        eci, occ, T, mu, seeds = bench.make_inputs(rank)
        local_ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
        ms = bench.max_over_ranks(local_ms, dist, "cpu")
        value = bench.job_throughput(1000.0, world, ms)
        q.put((rank, ms, value, occ[:, :64].copy(), seeds.copy(), bench._env_rank()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_chains_and_reduce_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        r = q.get(timeout=120)
        out[r[0]] = r
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, ms0, v0, occ0, seeds0, env0), (_, ms1, v1, occ1, seeds1, env1) = out[0], out[1]
    assert ms0 == ms1 == 15.0  # the slowest rank's time on every rank
    assert v0 == v1 == 1000.0 * 2 / 15e-3  # units of both ranks over that time
    assert env0 == (0, 2, 0) and env1 == (1, 2, 1)
    assert not np.array_equal(occ0, occ1)  # independent chains per rank
    assert not set(seeds0.tolist()) & set(seeds1.tolist())


def test_single_rank_helpers():
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.job_throughput(2e6, 1, 2.0) == 1e9


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(gpus=2, steps=3, warmup=1, ref_steps_per_sample=1e4)
    bench.run_reference(args)  # returns at once, prints nothing
    assert capsys.readouterr().out == ""


def test_gpus_flag_starts_its_own_ranks():
    """``bench.py --gpus 2`` outside torchrun starts two ranks itself (RANK/WORLD_SIZE set per
    process, 127.0.0.1 rendezvous): here through the reference arm, which needs no GPU; rank 0
    prints the one line and rank 1 exits 0 without work."""
    import json
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "3", "--warmup", "3", "--ref-steps-per-sample", "2000"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2


def test_gpus_flag_must_match_world_size():
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "3", "--warmup", "3"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "WORLD_SIZE" in r.stderr
