"""The multi-process path of bench.py on CPU (gloo, world size 2): each
rank is an independent replica; the helpers take the maximum time and the
summed work over ranks, and the barrier joins the ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_dist", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    import torch.distributed as dist
    # CPU only: gloo backend regardless of what the bench would pick
    dist.init_process_group(backend="gloo", rank=rank, world_size=world)
    bench.barrier(dist)
    mx = bench.max_over_ranks(dist, float(rank + 1))
    sm = bench.sum_over_ranks(dist, 10.0)
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((rank, mx, sm))


def test_two_rank_helpers():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2.0, 20.0), (1, 2.0, 20.0)]
