"""The N>1 path of bench.py on CPU: world_size-2 gloo ranks (127.0.0.1).
Replicas only: each rank runs the whole workload on its own GPU; the one
collective is the max over ranks of the step time, and the whole-job value
is the units of all ranks over that time.  Non-zero ranks of the reference
arm exit without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, times, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms = bench.replica_max_ms(times[rank], world, "cpu")
    dist.barrier()
    q.put((rank, ms, bench.replica_value(1_000_000, world, ms)))
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [10.0, 12.5]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == 12.5
        assert value == pytest.approx(2 * 1_000_000 / 0.0125)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_max_ms(7.0, 1, "cpu") == 7.0
    assert bench.replica_value(10, 1, 1000.0) == 10.0


@pytest.mark.parametrize("workload", ["uneven20k", "constraints_uneven20k"])
def test_reference_arm_nonzero_rank_exits_without_work(workload):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", workload, "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
