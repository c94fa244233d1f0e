"""bench.py with several GPUs runs replicas: one job per rank, no data-path collective. The
host-side pieces are checked here with two gloo ranks on the CPU: the job time is the slowest
rank's (max over ranks) and the work the sum of every rank's rays; each replica renders its own
samples; the reference arm's other ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench
        sec, rays = bench.aggregate_ranks(dist, 1.0 + 0.5 * rank, 1000 * (rank + 1), device="cpu")
        q.put((rank, sec, rays, [bench.replica_seed(rank, k) for k in range(3)]))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        r, sec, rays, seeds = q.get(timeout=120)
        out[r] = (sec, rays, seeds)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][:2] == out[1][:2] == (1.5, 3000)        # max of the times, sum of the rays
    assert not set(out[0][2]) & set(out[1][2])            # replicas render different samples


def test_single_process_aggregation_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_ranks(None, 2.5, 77) == (2.5, 77)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
