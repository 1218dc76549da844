"""The N > 1 path on CPU: the reference's direction slicing, the max over
ranks the benchmark times with, and reconstructVol sharded over two gloo ranks.

Each rank's work is a backend with the CUDA backend's interface
(sharding.GridderBackend): back_project(axes, images N x N) -> one (2, V, V, V)
tensor of un-divided sums (CAS volume, plane density), finish(sums) -> the
N^3 volume.  Here that work is the oracle's (images -> CAS images, the
reference-rule back projections in FP32, the division, getVol), and the
sharded result must equal the oracle's reconstructVol over all directions
in one process within relative L2 1e-6 (only the order of the float sums of
the two ranks' parts differs)."""
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
    """GridderBackend's interface and result shapes, computed by the oracle."""

    def __init__(self, p):
        self.p = p

    def back_project(self, axes, images):
        import torch

        p = self.p
        sums = np.zeros((2,) + (p.V,) * 3, np.float32)
        if len(axes):
            ci = O.cas_imgs_from_imgs(np.asarray(images, np.float64), p.M).astype(np.float32)
            sums[0] = O.bp_ref_f32(ci, axes, p.V, p.mask_radius, p.ker)
            sums[1] = O.bp_ref_f32(np.ones_like(ci), axes, p.V, p.mask_radius, p.ker)
        return torch.from_numpy(sums)

    def finish(self, sums):
        import torch

        cas = (sums[0] / (sums[1] + 1e-6)).numpy().astype(np.float64)
        return torch.from_numpy(O.vol_from_cas(cas, self.p.N).astype(np.float32))


def _case():
    N = 16
    p = O.Params(N)
    axes = O.quaternion_axes(9, 8).astype(np.float32)
    imgs = O.blob_volume(N, 5, seed=9)[:9] + np.random.default_rng(7).standard_normal((9, N, N)).astype(np.float32)
    return p, axes, imgs.astype(np.float32)


def _worker(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    from multigpugridder_gb300.sharding import max_over_ranks, reconstruct_sharded

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        m = max_over_ranks(1.0 + rank * 2.5)
        p, axes, imgs = _case()
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
    p, axes, imgs = _case()
    ref, _, _ = O.reconstruct_vol(imgs, axes, p, precision="f32")
    for r in range(world):
        got = np.load(tmp_path / ("vol%d.npy" % r))
        assert got.shape == (p.N,) * 3
        assert O.rel_l2(got, ref) < 1e-6
        assert float(np.load(tmp_path / ("max%d.npy" % r))[0]) == 3.5
