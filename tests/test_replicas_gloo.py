"""The multi-replica path of bench.py (one process per GPU, no data exchange): the host-side
barrier, max-over-ranks time and summed work, run as two gloo ranks on CPU."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    r, w, local = bench.dist_env()
    d = bench.Dist(w)
    d.barrier()
    ms = d.max(10.0 * (r + 1))   # the slowest rank's time
    work = d.sum(100.0)          # every rank's cell updates
    d.barrier()
    d.close()
    q.put((r, local, ms, work))


def test_two_gloo_ranks_take_max_time_and_total_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and [o[1] for o in out] == [0, 1]
    for _, _, ms, work in out:
        assert ms == 20.0 and work == 200.0
