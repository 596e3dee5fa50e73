"""The replicas path of bench.py (N > 1, one process per GPU, no data-path collective) on
CPU: two ranks over gloo on 127.0.0.1 -- the rank set-up from the torchrun environment, the
barrier, the max-over-ranks of the timed region, and the reference arm's rule that only
rank 0 works and prints."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class _Args:
    workload = "euler256"
    steps = 1
    warmup = 0


def _worker(rank, ws, port, q):
    os.environ.update(WORLD_SIZE=str(ws), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r, local = bench._dist()
    bench._barrier(w)
    m = bench._max_over_ranks(w, 1.0 + 2.0 * r)  # rank-dependent timings: every rank sees the slowest
    ref = bench.reference_arm(_Args, w, r) if r != 0 else "rank 0 works"
    bench._barrier(w)
    dist.destroy_process_group()
    q.put((r, w, local, m, ref))


def test_two_ranks_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    assert [(r[0], r[1], r[2]) for r in res] == [(0, 2, 0), (1, 2, 1)]
    assert [r[3] for r in res] == [3.0, 3.0]
    assert res[1][4] is None  # the reference arm: ranks other than 0 do no work
