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
    slice of (axes, images) into a CAS volume and a plane density
    (backend.back_project(axes, images) -> two V^3 tensors), one all-reduce
    sums both, and backend.finish(cas_sum, pd_sum) divides (+1e-6) and returns
    the volume.  Every rank returns the same volume."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    start, count = shard(len(axes), world, rank)
    cas, pd = backend.back_project(axes[start:start + count], images[start:start + count])
    both = torch.stack([cas, pd])
    if world > 1:
        dist.all_reduce(both, op=dist.ReduceOp.SUM, group=group)
    return backend.finish(both[0], both[1])


class GridderBackend:
    """The per-rank work of `reconstruct_sharded` on this rank's GPU, through
    the library's device-pointer calls: the reference-rule back projection of
    the images and of all-ones CAS images (the plane density), then, after the
    sum, the division and getVol."""

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

    def back_project(self, axes, images):
        import torch

        from . import _lib
        from ._lib import check

        L, h, V, M = _lib.lib(), self.h, self.g.V, self.g.M
        vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        ax = torch.as_tensor(np.ascontiguousarray(axes, np.float32)).to(self.dev)
        im = torch.as_tensor(np.ascontiguousarray(images, np.float32)).to(self.dev)
        n = ax.shape[0]
        cas = torch.zeros((V, V, V), dtype=torch.float32, device=self.dev)
        pd = torch.zeros_like(cas)
        if n > 0:
            sp = self._sp()
            check(L.gg_back_project_dev(h, vp(ax), n, vp(im), None, 0, sp), h)
            check(L.gg_get_cas_volume_dev(h, vp(cas), sp), h)
            ones = torch.ones((n, M, M), dtype=torch.float32, device=self.dev)
            check(L.gg_back_project_dev(h, vp(ax), n, None, vp(ones), 0, sp), h)
            check(L.gg_get_cas_volume_dev(h, vp(pd), sp), h)
        return cas, pd

    def finish(self, cas_sum, pd_sum):
        import torch

        from . import _lib
        from ._lib import check

        L, h, N = _lib.lib(), self.h, self.g.VolumeSize
        vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        div = (cas_sum / (pd_sum + 1e-6)).contiguous()  # tmpCASVolume ./ (PlaneDensity + 1e-6)
        out = torch.empty((N, N, N), dtype=torch.float32, device=self.dev)
        sp = self._sp()
        check(L.gg_set_cas_volume_dev(h, vp(div), sp), h)
        check(L.gg_get_volume_dev(h, vp(out), sp), h)
        return out
