"""The multi-GPU form is independent replicas (one run per GPU, no data-path
collective): the bench takes the slowest rank's time and reports the
whole-job steps/s. These tests run that host logic as two gloo ranks on the
CPU, and the reference arm's rank handling as separate processes."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
    got = bench.max_over_ranks(ms, dist, "cpu")
    q.put((rank, got, bench.replica_value(world, 20, got)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in procs)
    for rank, got, value in res:
        assert got == 150.0  # both ranks see the slowest time
        assert value == pytest.approx(2 * 20 / 0.150)


def _bench(env_extra, *args):
    env = dict(os.environ)
    env.update(env_extra)
    env["OMP_NUM_THREADS"] = "2"
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                          env=env, timeout=600, cwd=ROOT)


def test_reference_arm_other_ranks_exit_quietly():
    r = _bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--impl", "reference", "--gpus", "2",
               "--case", "he100_xe_32", "--steps", "1", "--warmup", "0")
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_reference_arm_rank0_prints_one_line():
    r = _bench({"RANK": "0", "WORLD_SIZE": "2", "LOCAL_RANK": "0"}, "--impl", "reference", "--gpus", "2",
               "--case", "he100_xe_32", "--steps", "1", "--warmup", "0")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "steps/s" and d["value"] > 0
    assert d["config"]["grid"] == [32, 32, 32]
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
