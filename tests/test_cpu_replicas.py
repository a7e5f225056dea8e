"""The N > 1 path of bench.py is N independent replicas (one level on one GPU
has no exchange): its host logic -- the maximum of the ranks' times and the
whole-job value -- on two gloo ranks on the CPU, and the reference arm's
rank rule (rank 0 prints, the others exit without work)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    m = bench.max_over_ranks(ms, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, m, bench.replica_value(1000, 4, world, m)))


def test_max_over_ranks_and_replica_value_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [m for _, m, _ in out] == [150.0, 150.0]
    # 2 replicas x 1000 cells x 4 steps in 150 ms
    assert out[0][2] == pytest.approx(2 * 1000 * 4 / 0.150)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
