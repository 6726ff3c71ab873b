"""Multi-GPU path of bench.py on the CPU: two gloo ranks run the rank set-up
and the max-over-ranks reduction that times a replicated step (the solver has
no inter-GPU exchange: N GPUs run N independent replicas)."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    dist, r, ws = bench.dist_init()
    t = bench.max_over_ranks(dist, 1.5 + rank)      # per-rank step time
    dist.barrier()
    q.put((r, ws, t))
    dist.destroy_process_group()


def test_two_rank_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == 2.5 for o in out)   # both ranks see the slowest rank's time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    os.environ.pop("WORLD_SIZE", None)
    dist, r, ws = bench.dist_init()
    assert dist is None and r == 0 and ws == 1
    assert bench.max_over_ranks(dist, 3.25) == 3.25
