"""Multi-process host logic of the replica / view-shard path, on CPU with gloo.

Two ranks each render their contiguous share of a list of small views (through
the oracle: this tests the sharding and the gather, not a kernel) and gather the
per-view digests on rank 0; the merged list must equal a single-process render
of all views in order."""
import hashlib
import os
import socket
import tempfile

import numpy as np
import pytest

from rosy_gb300.replicas import merge_in_rank_order, shard_range


def _views():
    from rosy_gb300 import scene as sc

    base = sc.tiny(3)
    sizes = [(48, 32, 64), (96, 64, 128), (40, 40, 64), (64, 48, 128), (32, 96, 64)]
    return [sc.view_of(base, w, h, s, camera=i % len(base.cameras)) for i, (w, h, s) in enumerate(sizes)]


def _digest(out) -> str:
    h = hashlib.sha256()
    for k in ("color", "depth", "ids", "shadow"):
        h.update(np.ascontiguousarray(out[k]).tobytes())
    return h.hexdigest()


def _rank_main(rank, world, port, result_path):
    import torch.distributed as dist

    from oracle import oracle
    from rosy_gb300.replicas import gather_to_rank0

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        views = _views()
        b, e = shard_range(len(views), rank, world)
        mine = [(i, _digest(oracle.render(views[i], threads=1))) for i in range(b, e)]
        parts = gather_to_rank0(mine, world)
        if rank == 0:
            with open(result_path, "w") as f:
                for i, d in merge_in_rank_order(parts):
                    f.write(f"{i} {d}\n")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_range_partitions_in_order():
    for count in range(0, 20):
        for world in range(1, 6):
            spans = [shard_range(count, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == count
            for (b0, e0), (b1, e1) in zip(spans, spans[1:]):
                assert e0 == b1
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def test_two_gloo_ranks_render_their_shards(oracle):
    import torch.multiprocessing as mp

    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "digests.txt")
        mp.start_processes(_rank_main, args=(2, _free_port(), path), nprocs=2, join=True, start_method="spawn")
        got = [line.split() for line in open(path).read().splitlines()]
    views = _views()
    want = [[str(i), _digest(oracle.render(v, threads=1))] for i, v in enumerate(views)]
    assert got == want
