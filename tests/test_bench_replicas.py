"""The replica split of bench.py under torchrun, on CPU with the gloo backend (world size 2).

Energy points are independent, so every rank solves its own sweep and the only exchange is the max of the
ranks' timed seconds (no collective on the data path).  Checked here without a GPU: the process group comes up
from the torchrun environment, the max over ranks is every rank's answer, and the ranks' energy windows differ.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, root, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, root)
    import bench
    from refeff_gb300 import workloads as wl
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    seconds = bench.max_over_ranks(1.0 + rank, w)
    bench.barrier(w)
    cl, _ = wl.config0()
    grid = wl.energy_grid(cl, 8, -20.0 + 0.37 * r, 150.0 + 0.37 * r, seed=1 + r)
    out.put((r, seconds, float(grid.energies_ev[0])))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_bench_replicas_gloo_world_size_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    procs = [ctx.Process(target=_rank, args=(r, 2, port, root, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.0, 2.0]          # both ranks see the slowest rank's time
    assert got[0][2] != got[1][2]                      # independent energy windows per rank
