"""The N > 1 path of bench.py (independent replicas, one per rank, with a
barrier and max-over-ranks timing) run as two gloo ranks on the CPU: the
slowest rank's time reaches every rank, the whole-job rate counts all ranks'
design iterations over that time, and the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    assert bench.dist_setup() == (ws, rank, rank)
    bench.barrier(ws)
    t = 1.0 + 0.5 * rank               # rank 1 is the slower one
    tmax = bench.max_over_ranks(t, ws, device="cpu")
    q.put((rank, tmax, bench.replica_rate(10, ws, tmax)))
    bench.barrier(ws)
    dist.destroy_process_group()


def test_two_gloo_ranks_max_and_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, tmax, rate in res:
        assert tmax == 1.5          # the slowest rank's time on every rank
        assert rate == 2 * 10 / 1.5


def test_reference_arm_runs_on_rank0_only():
    """A rank other than 0 of the reference arm exits 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
