"""The multi-GPU path of bench.py is N independent replicas (a frame does not
shard): each rank draws its own frames, the job's time is the slowest
rank's, and the value is all ranks' frames over that time. These run the
cross-rank reduction as two gloo ranks on the CPU, and the reference arm's
rule that ranks other than 0 exit without work."""
import os
import socket
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    slowest = bench.max_over_ranks(times[rank], world, device="cpu")
    out.put((rank, slowest, bench.replica_throughput(world, 20, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_slowest_rank_sets_the_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [0.250, 0.400]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, slowest, fps in got:
        assert slowest == pytest.approx(0.400)
        assert fps == pytest.approx(2 * 20 / 0.400)


def test_one_rank_is_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, 1) == 1.5
    assert bench.replica_throughput(1, 10, 2.0) == 5.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
