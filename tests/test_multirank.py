"""The cosmology-sharded multi-process path on CPU: world_size-2 gloo process
groups, with a stand-in per-rank evaluation (the GPU evaluation itself is the
single-GPU path the other tests cover)."""
import os
import socket

import numpy as np
import pytest

from threepoint_gb300.shard import gather_blocks, map3_sharded, shard_range


@pytest.mark.parametrize("n,world", [(0, 2), (1, 2), (5, 2), (4096, 8), (7, 3), (3, 5)])
def test_shard_range_partitions(n, world):
    blocks = [shard_range(n, r, world) for r in range(world)]
    assert blocks[0][0] == 0 and blocks[-1][1] == n
    for (a, b), (c, d) in zip(blocks, blocks[1:]):
        assert b == c and a <= b
    sizes = [b - a for a, b in blocks]
    assert max(sizes) - min(sizes) <= 1


def test_shard_range_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def stand_in(block, lo):
    """A per-cosmology result that identifies the cosmology and the triplet."""
    return np.array([[c["om"] * 1000 + c["sigma8"] + t for t in range(4)] for c in block])


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, outdir):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        cos = [dict(om=0.2 + 0.01 * i, sigma8=0.7 + 0.001 * i) for i in range(n)]
        res = map3_sharded(cos, stand_in)
        if rank == 0:
            np.save(os.path.join(outdir, "res.npy"), res)
        else:
            assert res is None
        # a rank with an empty block still takes part in the gather
        empty = gather_blocks(np.zeros((0, 4)), 0, 0)
        if rank == 0:
            assert empty.shape == (0, 4)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n", [5, 64])
def test_gloo_two_ranks_gather_in_global_order(tmp_path, n):
    import torch.multiprocessing as mp

    mp.start_processes(_worker, args=(2, _free_port(), n, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(tmp_path / "res.npy")
    cos = [dict(om=0.2 + 0.01 * i, sigma8=0.7 + 0.001 * i) for i in range(n)]
    assert np.array_equal(got, stand_in(cos, 0))


def test_single_process_is_identity():
    cos = [dict(om=0.3, sigma8=0.8), dict(om=0.31, sigma8=0.81)]
    assert np.array_equal(map3_sharded(cos, stand_in), stand_in(cos, 0))
