"""The multi-GPU arm of bench.py on CPU: two ranks over gloo (127.0.0.1).  Each
rank steps its own images (weak scaling, no collective on the data path); the
only exchange is the timing reduction (max time, summed lattice updates), and the
reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp
from conftest import ROOT

sys.path.insert(0, str(ROOT))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        # per-rank work differs: rank r owns images r*k .. r*k+k-1 and its own time
        lu = [2.0e6, 3.0e6][rank]
        ms = [100.0, 125.0][rank]
        value, ms_max, lu_job = bench.job_rate(lu, ms, 50, dist, "cpu")
        # the reference arm: every rank but 0 returns without work
        ref = bench.run_reference(None, rank, world) if rank else "rank0"
        q.put((rank, value, ms_max, lu_job, ref))
    finally:
        dist.destroy_process_group()


def test_two_rank_job_rate():
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
    for rank, value, ms_max, lu_job, ref in out:
        assert ms_max == 125.0 and lu_job == 5.0e6
        assert value == pytest.approx(5.0e6 * 50 / 0.125 / 1e6)
    assert out[1][4] is None


def test_ranks_own_distinct_images():
    import bench

    a = bench.make_images(1, 0 * 1, "config2")[0]
    b = bench.make_images(1, 1 * 1, "config2")[0]
    assert (a["pore"] != b["pore"]).any()
