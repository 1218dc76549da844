"""Orientation sharding over ranks (one GPU per process) for the N > 1 path.

The reference gives each GPU a contiguous slice of ceil(n / G) directions,
the last GPU the remainder (MultiGPUGridder::PlanCoordinateAxes,
MultiGPUGridder.cpp:37-96).  A forward projection needs no exchange: each
rank projects its slice.  A back projection has one: the per-GPU CAS volumes
are summed (MultiGPUGridder.cpp:376-411); reconstructVol sums the plane
density the same way before dividing (MultiGPUGridder_Matlab_Class.m:293-308).
Here the sum is one all-reduce over the process group of the stacked CAS
volume and plane density (NCCL between GPUs, gloo on CPU).

`reconstruct_sharded` takes the per-rank work as a backend object, so the
reduction and the bookkeeping run the same way with the library's CUDA path
(`GridderBackend`) and with any other implementation of the two calls.
"""
import ctypes
import math

import numpy as np


def shard(n, world, rank):
    """(start, count) of rank's directions: ceil(n / world) per rank, in order."""
    per = int(math.ceil(n / world)) if world > 0 else n
    start = min(rank * per, n)
    return start, max(0, min(per, n - start))


def max_over_ranks(x, device="cpu"):
    """The largest value of x over the default process group (x on one rank if
    torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reconstruct_sharded(backend, axes, images, group=None):
    """reconstructVol over the ranks of `group`: each rank back-projects its
    slice of (axes, images) into one buffer of two stacked V^3 sums, the CAS
    volume and the plane density (backend.back_project(axes, images) ->
    tensor (2, V, V, V)); one all-reduce sums the buffer in place; and
    backend.finish(sums) divides (+1e-6) and returns the volume.  Every rank
    returns the same volume."""
    import torch.distributed as dist

    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    start, count = shard(len(axes), world, rank)
    sums = backend.back_project(axes[start:start + count], images[start:start + count])
    if world > 1:
        dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
    return backend.finish(sums)


class GridderBackend:
    """The per-rank work of `reconstruct_sharded` on this rank's GPU, through
    the library's device-pointer calls: gg_back_project_sums_dev (the images'
    back projection and the plane density in one fused pass, un-divided) and,
    after the sum over ranks, gg_volume_from_sums_dev (the division and
    getVol)."""

    def __init__(self, gridder, stream=None):
        import torch

        self.g = gridder
        self.h = gridder.handle
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.stream = stream

    def _sp(self):
        import torch

        s = self.stream or torch.cuda.current_stream(self.dev)
        return ctypes.c_void_p(s.cuda_stream)

    def back_project(self, axes, images, out=None):
        """This rank's sums (2, V, V, V) on its GPU; axes (n, 9) and images
        (n, N, N), numpy arrays or tensors (moved to the GPU if needed)."""
        import torch

        from . import _lib
        from ._lib import check

        L, h, V = _lib.lib(), self.h, self.g.V
        ax = torch.as_tensor(np.ascontiguousarray(axes, np.float32) if isinstance(axes, np.ndarray) else axes)
        im = torch.as_tensor(np.ascontiguousarray(images, np.float32) if isinstance(images, np.ndarray) else images)
        ax = ax.to(self.dev, torch.float32).contiguous()
        im = im.to(self.dev, torch.float32).contiguous()
        sums = out if out is not None else torch.empty((2, V, V, V), dtype=torch.float32, device=self.dev)
        check(L.gg_back_project_sums_dev(h, ctypes.c_void_p(ax.data_ptr()), ax.shape[0],
                                         ctypes.c_void_p(im.data_ptr()), ctypes.c_void_p(sums.data_ptr()),
                                         self._sp()), h)
        return sums

    def finish(self, sums, out=None):
        import torch

        from . import _lib
        from ._lib import check

        L, h, N = _lib.lib(), self.h, self.g.VolumeSize
        vol = out if out is not None else torch.empty((N, N, N), dtype=torch.float32, device=self.dev)
        check(L.gg_volume_from_sums_dev(h, ctypes.c_void_p(sums.data_ptr()), ctypes.c_void_p(vol.data_ptr()),
                                        self._sp()), h)
        return vol
