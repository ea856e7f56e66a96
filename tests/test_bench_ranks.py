"""The multi-GPU (replica) path of bench.py on CPU: two gloo ranks, each with its
own timing, agree on the max-over-ranks time and the whole-job throughput."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    import bench
    times = [[50.0, 60.0, 55.0], [52.5, 58.0, 61.0]][rank]
    dist.barrier()
    m = bench.max_over_ranks(times, ws)
    out.put((rank, m, bench.job_throughput(1 << 18, ws, m[0])))
    dist.destroy_process_group()


def test_two_replicas_report_max_time_and_job_throughput():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict((r, (m, v)) for r, m, v in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        m, v = res[r]
        assert m == [52.5, 60.0, 61.0]
        assert v == pytest.approx(2 * (1 << 18) / 52.5e-3)
