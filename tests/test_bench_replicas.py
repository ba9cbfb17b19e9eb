"""bench.py's replica path (one rank per GPU, no data-path collective): two gloo ranks on the
CPU agree on the slowest rank's time and on the whole-job throughput."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.replica_throughput(10.0 + 3.0 * rank, ws, 1000, 5, dist)
    el = bench.max_over_ranks(0.5 * (rank + 1), dist)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ms, value, el))


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value, el in res:
        assert ms == 13.0 and el == 1.0
        assert abs(value - 2 * 1000 * 5 / 13.0e-3) < 1e-6 * value


def test_one_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(20.0, 1, 100, 4) == (20.0, 100 * 4 / 20.0e-3)
