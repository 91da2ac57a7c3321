"""The multi-GPU path's host logic on CPU: two gloo ranks (world size 2).
Each rank works on its own shard with its own seed; the only exchange is
the maximum of the ranks' timings; the whole-job rate is all units over the
slowest rank's time; under torchrun the reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from bamf_gb300 import replicas

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = 1.5 + rank            # rank 1 is the slow one
        slowest = replicas.max_over_ranks(local, dist, "cpu")
        sh = replicas.shard(10, rank, world)
        q.put((rank, slowest, replicas.rank_seed(2, rank), (sh.start, sh.stop),
               replicas.whole_job_rate(100, world, slowest)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_only_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.5, 2.5]           # both see the slower rank's time
    assert got[0][2] != got[1][2]                      # each rank its own workload seed
    assert got[0][3] == (0, 5) and got[1][3] == (5, 10)
    assert got[0][4] == pytest.approx(2 * 100 / 2.5)


def test_shard_covers_every_unit_once():
    for n in (0, 1, 7, 100, 101):
        for w in (1, 2, 3, 8):
            seen = [i for r in range(w) for i in replicas.shard(n, r, w)]
            assert seen == list(range(n))
    assert replicas.max_over_ranks(3.0) == 3.0
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_reference_arm_runs_on_rank_zero_only():
    """bench.py --impl reference under torchrun: rank 1 exits 0 without a
    line; rank 0 prints one JSON line (a tiny sample of the CPU restatement)."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    args = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
            "--warmup", "0", "--n-rois", "64", "--jumps", "20", "--cpu-sample", "8"]
    r1 = subprocess.run(args, env=env, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r1.returncode == 0 and r1.stdout.strip() == ""
    env.update(RANK="0", LOCAL_RANK="0")
    r0 = subprocess.run(args, env=env, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r0.returncode == 0, r0.stderr[-2000:]
    line = json.loads(r0.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
