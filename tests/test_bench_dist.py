"""The replica path of bench.py (N > 1 ranks, one GPU each, no collective on
the data path): process-group setup, the barrier and the max-over-ranks
timing, as world_size-2 gloo ranks on the CPU."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    os.environ.update(WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    world, r, local = bench.dist_setup()
    bench.barrier(world)
    v = bench.max_over_ranks(0.5 + rank, world, "cpu")   # per-rank step times 0.5 and 1.5
    q.put((r, world, local, v, dist.get_backend()))
    dist.destroy_process_group()


def test_replica_timing_is_the_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 0, 1.5, "gloo"), (1, 2, 1, 1.5, "gloo")]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_setup() == (1, 0, 0)
    assert bench.max_over_ranks(3.25, 1, "cpu") == 3.25
