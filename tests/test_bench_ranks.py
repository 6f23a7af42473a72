"""The N > 1 launch path of bench.py on CPU: two ranks over gloo.

Each rank runs its own replica (independent ensembles, no data-path
collective); bench.py reports the maximum time over ranks and the units of
all ranks.  The reference arm runs on rank 0 only.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench._dist() == (ws, rank, rank)
        ms = 10.0 + 5.0 * rank          # rank 1 is the slower one
        units = 1000.0 * (rank + 1)
        t, u = bench.reduce_over_ranks(ms, units, ws)
        out[rank] = (t, u)
    finally:
        dist.destroy_process_group()


def test_reduce_over_ranks_gloo_two_ranks():
    """Time = maximum over ranks, units = sum over ranks, on every rank."""
    ws, port = 2, _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank_main, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert res[0] == res[1] == (15.0, 3000.0)


def test_reduce_over_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(12.5, 7.0, 1) == (12.5, 7.0)


def _ref_rank_main(rank, ws, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    if rank == 0:
        out[rank] = "skipped"  # rank 0 would run the CPU reference; not here
        return
    args = bench.build_parser().parse_args(["--impl", "reference", "--gpus", str(ws)])
    bench.run_reference(args)  # returns at once on rank != 0
    out[rank] = "returned"


def test_reference_arm_runs_on_rank_zero_only():
    ws, port = 2, _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_ref_rank_main, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert res == {0: "skipped", 1: "returned"}
