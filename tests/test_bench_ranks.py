"""The multi-rank harness of bench.py on CPU: two gloo ranks on 127.0.0.1.
The path runs as independent replicas, so the only cross-rank steps are the
barrier around the timed region and the max of the step time over ranks;
the reference arm runs on rank 0 alone and other ranks leave without work."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench as B
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert B.dist_init()[:2] == (world, rank)
        B.barrier(world)
        got = B.reduce_max(1.5 + rank, world)
        # the reference arm: rank 0 alone works; the others return at once
        ran = "skipped" if rank != 0 else "rank0"
        if rank != 0:
            assert B.run_reference(None, world, rank) is None
        B.barrier(world)
        with open(os.path.join(out_dir, "r%d" % rank), "w") as f:
            f.write("%r %s" % (got, ran))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_barrier_max_and_reference_arm(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0 = open(tmp_path / "r0").read().split()
    r1 = open(tmp_path / "r1").read().split()
    assert float(r0[0]) == 2.5 and float(r1[0]) == 2.5   # max over ranks
    assert r0[1] == "rank0" and r1[1] == "skipped"


def test_single_process_helpers_are_identities():
    sys.path.insert(0, ROOT)
    import bench as B
    assert B.reduce_max(3.25, 1) == 3.25
    B.barrier(1)
