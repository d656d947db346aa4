"""Multi-process (world size 2, gloo, CPU) checks of bench.py's replica
bookkeeping: the rank setup, the barrier, the max over ranks that the timed
value takes, and that only rank 0 runs and prints the reference arm.

One solve does not shard (the preconditioner is global), so N > 1 runs N
independent replicas; these are the only cross-rank operations there are.
"""
import os
import socket
import sys
import types

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench

    args = types.SimpleNamespace(impl="reference", gpus=world)
    w, r, local = bench.dist_init(args)
    assert (w, r, local) == (world, rank, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # every rank times its own replica; the line reports the slowest
    v = bench.allmax(w, 10.0 + rank)
    bench.barrier(w)
    # the reference arm runs on rank 0 only: other ranks return at once
    if rank != 0:
        assert bench.run_reference(args, w, rank) is None
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(v))
    dist.destroy_process_group()


def test_replicas_gloo_world2(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    vals = [float(open(tmp_path / f"rank{r}.txt").read()) for r in range(world)]
    assert vals == [11.0, 11.0]


def test_single_rank_is_passthrough():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.allmax(1, 3.5) == 3.5
    bench.barrier(1)  # no process group needed
