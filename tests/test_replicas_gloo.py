"""Multi-GPU path of the benchmark (replicas only) on CPU with gloo, world size 2:
the max-over-ranks timing and the whole-job rate, and failure detection (a rank
that dies makes the survivor's next collective fail instead of hanging)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, mode, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    class A:
        impl = "reference"
    try:
        w, r, _, dist = bench.dist_setup(A, backend="gloo", timeout_s=20.0)
        if mode == "ok":
            t = bench.max_over_ranks(1.0 + r, dist)
            q.put((r, "ok", t, bench.replica_rate(w, 1000, t)))
            dist.barrier()
        else:   # after one completed step rank 1 dies; rank 0's next collective must fail
            bench.max_over_ranks(1.0, dist)
            if r == 1:
                os._exit(3)
            try:
                bench.max_over_ranks(1.0, dist)
                msg = (r, "no error", None, None)
            except Exception as e:   # noqa: BLE001 - any collective failure is the expected outcome
                msg = (r, "error", type(e).__name__, None)
            q.put(msg)
            q.close()
            q.join_thread()   # the message is in the pipe before the hard exit
            os._exit(0)
        dist.destroy_process_group()
    except Exception as e:   # noqa: BLE001
        q.put((rank, "exception", repr(e), None))


def _run(mode, timeout=180):   # spawn + import torch can be slow on a loaded host; the collective timeout is 20 s
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, mode, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = []
    want = 2 if mode == "ok" else 1
    for _ in range(want):
        out.append(q.get(timeout=timeout))
    for p in ps:
        p.join(timeout=timeout)
        if p.is_alive():
            p.kill()
    return sorted(out)


def test_replicas_max_over_ranks_and_rate():
    out = _run("ok")
    assert [o[1] for o in out] == ["ok", "ok"], out
    assert all(o[2] == 2.0 for o in out)            # max of 1.0 and 2.0
    assert all(o[3] == 2 * 1000 / 2.0 for o in out)  # both ranks' trajectories over the slowest time


def test_dead_rank_fails_the_collective_instead_of_hanging():
    out = _run("die")
    assert out[0][0] == 0 and out[0][1] == "error", out
