"""The replicas-only multi-process path of bench.py on CPU: two gloo ranks.

Each rank of `bench.py --gpus N` synthesises its own clip on its own GPU;
the ranks only meet at a barrier and a max over ranks of the timed interval
(no data-path collective).  These tests run that plumbing with world size 2
over gloo, without a GPU.
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    try:
        import bench
        d = bench.Dist()
        d.barrier()
        m = d.max(10.0 + 5.0 * rank)  # each rank's own timed interval
        skipped = None
        if rank == 1:
            # the reference arm runs on rank 0 only; the other ranks return at once
            class A:
                frames, steps, warmup, gpus = 1, 1, 0, 2
            skipped = bench.run_reference(A(), d)
        d.barrier()
        d.close()
        out.put((rank, d.ws, m, skipped))
    except Exception as e:  # reported to the parent
        out.put((rank, "error", repr(e), None))


def test_two_gloo_ranks_barrier_and_max_over_ranks():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, ws, m, skipped = out.get(timeout=120)
        res[rank] = (ws, m, skipped)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        assert res[rank][0] == 2, res
        assert res[rank][1] == 15.0, res  # the slowest rank's interval, seen by every rank
    assert res[1][2] == 0  # reference arm: rank 1 did no work and exited 0


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    old = {k: os.environ.pop(k, None) for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    try:
        d = bench.Dist()
        assert d.ws == 1 and d.rank == 0
        assert d.max(3.5) == 3.5
        d.barrier()
        d.close()
    finally:
        for k, v in old.items():
            if v is not None:
                os.environ[k] = v


def test_gpus_flag_must_match_the_launched_ranks():
    """`--gpus N` without N launched ranks fails loudly instead of running
    one replica."""
    sys.path.insert(0, ROOT)
    import bench
    old = {k: os.environ.pop(k, None) for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    try:
        d = bench.Dist()

        class A:
            frames, steps, warmup, gpus = 1, 1, 0, 8
        with pytest.raises(SystemExit):
            bench.run_reference(A(), d)
        d.close()
    finally:
        for k, v in old.items():
            if v is not None:
                os.environ[k] = v
