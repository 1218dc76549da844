"""The N > 1 path on CPU: the reference's direction slicing, the max over
ranks the benchmark times with, and reconstructVol sharded over two gloo ranks
(the oracle's reference-rule back projection as each rank's work) equal to one
process over all directions within relative L2 1e-6 (only the order of the
float sums differs)."""
import os
import socket

import numpy as np
import pytest

from oracle import oracle as O


def test_shard_matches_the_reference_plan():
    from multigpugridder_gb300.sharding import shard

    # MultiGPUGridder.cpp:37-96: ceil(n/G) per GPU in order, the last the rest
    assert [shard(10, 3, r) for r in range(3)] == [(0, 4), (4, 4), (8, 2)]
    assert [shard(2, 4, r) for r in range(4)] == [(0, 1), (1, 1), (2, 0), (2, 0)]
    for n in (0, 1, 7, 100, 10000):
        for world in (1, 2, 3, 8):
            parts = [shard(n, world, r) for r in range(world)]
            assert sum(c for _, c in parts) == n
            pos = 0
            for s, c in parts:
                if c:
                    assert s == pos
                pos += c


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _OracleBackend:
    def __init__(self, p):
        self.p = p

    def back_project(self, axes, cas_images):
        import torch

        p = self.p
        cas = O.bp_ref_f32(cas_images, axes, p.V, p.mask_radius, p.ker) if len(axes) else np.zeros((p.V,) * 3, np.float32)
        pd = (O.bp_ref_f32(np.ones_like(cas_images), axes, p.V, p.mask_radius, p.ker) if len(axes)
              else np.zeros((p.V,) * 3, np.float32))
        return torch.from_numpy(np.ascontiguousarray(cas)), torch.from_numpy(np.ascontiguousarray(pd))

    def finish(self, cas, pd):
        return cas / (pd + 1e-6)


def _worker(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    from multigpugridder_gb300.sharding import max_over_ranks, reconstruct_sharded

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        m = max_over_ranks(1.0 + rank * 2.5)
        p = O.Params(16)
        rng = np.random.default_rng(7)
        axes = O.quaternion_axes(9, 8).astype(np.float32)
        imgs = rng.standard_normal((9, p.M, p.M)).astype(np.float32)
        vol = reconstruct_sharded(_OracleBackend(p), axes, imgs)
        np.save(os.path.join(out_dir, "vol%d.npy" % rank), vol.numpy())
        np.save(os.path.join(out_dir, "max%d.npy" % rank), np.array([m]))
    finally:
        dist.destroy_process_group()


def test_reconstruct_sharded_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    p = O.Params(16)
    rng = np.random.default_rng(7)
    axes = O.quaternion_axes(9, 8).astype(np.float32)
    imgs = rng.standard_normal((9, p.M, p.M)).astype(np.float32)
    whole = _OracleBackend(p).back_project(axes, imgs)
    ref = (whole[0] / (whole[1] + 1e-6)).numpy()
    for r in range(world):
        got = np.load(tmp_path / ("vol%d.npy" % r))
        assert O.rel_l2(got, ref) < 1e-6
        assert float(np.load(tmp_path / ("max%d.npy" % r))[0]) == 3.5
