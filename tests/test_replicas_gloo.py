"""Several GPUs run independent replicas (one bunch per rank, no data-path
collective).  The host logic the bench runs under torchrun, on CPU with the
gloo backend at world size 2: every rank reads its place from the
environment, the slowest replica's time becomes every rank's (the job's
time), the line says "replicas", and the reference arm's other ranks
return without work (rank 0 alone times the CPU path and prints)."""
import contextlib
import io
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, _ = bench.dist_env()
    t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, device="cpu")
    cfg = bench.bench_config(1000, 160, "plain", w)
    printed = ""
    if rank != 0:
        out = io.StringIO()
        with contextlib.redirect_stdout(out):
            bench.run_reference(None)  # returns before touching its arguments
        printed = out.getvalue()
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, r, w, t, cfg["parallelism"], printed))


def test_replicas_take_the_slowest_rank_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (k, r, w, t, par, printed) in enumerate(got):
        assert (k, r, w) == (rank, rank, 2)
        assert t == 15.0          # the slower replica's time on every rank
        assert par == "replicas"
    assert got[1][5] == ""        # the reference arm's rank 1 printed nothing


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.bench_config(10, 160, "plain", 1)["parallelism"] == "single"
