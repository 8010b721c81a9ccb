"""Checkpointed batch runner (threepoint_gb300/batch.py): chunks, manifest,
resume after an interruption, refusal of a directory of other inputs, and
two gloo ranks writing their blocks. The evaluation is a stand-in (the GPU
evaluation is covered by the other tests); one GPU test runs the real one."""
import os
import socket

import numpy as np
import pytest

from threepoint_gb300 import batch as BT

TH = np.array([[1.0, 2.0, 3.0], [2.0, 2.0, 2.0]]) * 2.9e-4


def cosmos(n):
    return [dict(om=0.2 + 0.001 * i, sigma8=0.8) for i in range(n)]


class Counting:
    def __init__(self, fail_after=None):
        self.calls, self.fail_after = 0, fail_after

    def __call__(self, cs, th):
        if self.fail_after is not None and self.calls >= self.fail_after:
            raise KeyboardInterrupt("simulated interruption")
        self.calls += 1
        v = np.array([[c["om"] * 1e3 + t for t in range(len(th))] for c in cs])
        return {"value": v, "status": np.zeros_like(v, dtype=np.int32)}


def test_chunks_and_assemble(tmp_path):
    ev = Counting()
    files = BT.run(cosmos(10), TH, str(tmp_path), ev, chunk=4)
    assert len(files) == 3 and ev.calls == 3
    v = BT.assemble(str(tmp_path))
    assert v.shape == (10, 2)
    assert np.array_equal(v, Counting()(cosmos(10), TH)["value"])


def test_resume_after_interruption(tmp_path):
    with pytest.raises(KeyboardInterrupt):
        BT.run(cosmos(10), TH, str(tmp_path), Counting(fail_after=2), chunk=4)
    with pytest.raises(RuntimeError):
        BT.assemble(str(tmp_path))  # 2 of 3 chunks present
    ev = Counting()
    BT.run(cosmos(10), TH, str(tmp_path), ev, chunk=4)
    assert ev.calls == 1  # only the missing chunk is evaluated
    assert np.array_equal(BT.assemble(str(tmp_path)), Counting()(cosmos(10), TH)["value"])


def test_other_inputs_refused(tmp_path):
    BT.run(cosmos(5), TH, str(tmp_path), Counting(), chunk=4)
    with pytest.raises(ValueError):
        BT.run(cosmos(6), TH, str(tmp_path), Counting(), chunk=4)
    with pytest.raises(ValueError):
        BT.run(cosmos(5), TH * 2, str(tmp_path), Counting(), chunk=4)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, outdir):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        BT.run(cosmos(11), TH, outdir, Counting(), chunk=4, rank=rank, world=world)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_write_disjoint_blocks(tmp_path):
    import torch.multiprocessing as mp

    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    assert os.path.exists(tmp_path / "manifest.rank1.json")
    assert np.array_equal(BT.assemble(str(tmp_path)), Counting()(cosmos(11), TH)["value"])


@pytest.mark.gpu
def test_gpu_batch_matches_direct(tmp_path, nz256):
    import threepoint_gb300 as tp
    from conftest import COSMO1

    cs = [tp.cosmology(**dict(COSMO1, sigma8=s)) for s in (0.75, 0.8, 0.85)]
    ctx = tp.Context(0)
    BT.run(cs, TH, str(tmp_path), BT.context_evaluator(ctx, nz256), chunk=2)
    got = BT.assemble(str(tmp_path))
    ctx.set_cosmologies(cs, nz256)
    ref = ctx.map3_batch(TH, precision=tp.FP32)
    assert np.array_equal(got, ref)
    ctx.close()
