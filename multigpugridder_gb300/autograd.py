"""Differentiable forward projection for PyTorch.

`ForwardProjector.project(vol, axes)` maps a CUDA volume (N^3, FP32) to its
projection images (n x N x N) through the library's device-pointer calls:
the CAS preparation of setVolume, the forward projection and the CAS-image to
image path.  Its backward is the exact adjoint of that whole linear map
(`gg_forward_project_adjoint_dev`, built on the exact-adjoint back-projection
kernel with the forward kernel's pair set and weights), so gradients agree
with finite differences of the forward operator.  The reference has no
gradient; its back projection (the window rule of gpuBackProject.cu) is not
the adjoint of its forward projection at general orientations.

All work is enqueued on torch's current stream; no host synchronisation.
"""
import ctypes

import torch

from . import _lib
from ._lib import check


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


class ForwardProjector:
    """Owns one gridder handle on one GPU for volumes of edge N."""

    def __init__(self, N, interp=2.0, device=None, max_batch=4096, precision="f32"):
        L = _lib.lib()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.N = int(N)
        h = ctypes.c_void_p()
        dev = (ctypes.c_int * 1)(self.device.index or 0)
        check(L.gg_create(self.N, 0, ctypes.c_float(interp), 3, 1, dev, 1, 0, ctypes.byref(h)))
        self._h = h
        check(L.gg_set_max_axes_to_allocate(h, int(max_batch)), h)
        check(L.gg_set_precision(h, _lib.PRECISIONS[precision]), h)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check_inputs(self, vol, axes):
        n = self.N
        if vol.shape != (n, n, n) or vol.dtype != torch.float32 or not vol.is_cuda:
            raise ValueError("vol must be a CUDA float32 tensor of shape (%d, %d, %d)" % (n, n, n))
        if axes.dtype != torch.float32 or not axes.is_cuda or axes.numel() % 9:
            raise ValueError("axes must be a CUDA float32 tensor with 9 values per direction")

    def project(self, vol, axes):
        """Images (n, N, N) of vol along axes (n, 9); differentiable in vol."""
        self._check_inputs(vol, axes)
        return _ForwardProject.apply(vol, axes, self)

    def adjoint(self, image_grads, axes):
        """The exact adjoint applied to image gradients (n, N, N) -> (N, N, N)."""
        g = image_grads.contiguous().float()
        ax = axes.contiguous()
        n = ax.numel() // 9
        out = torch.empty((self.N,) * 3, dtype=torch.float32, device=g.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(g.device).cuda_stream)
        check(_lib.lib().gg_forward_project_adjoint_dev(self._h, _vp(ax), n, _vp(g), _vp(out), stream), self._h)
        return out


class _ForwardProject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vol, axes, proj):
        L = _lib.lib()
        v = vol.detach().contiguous()
        ax = axes.detach().contiguous()
        n = ax.numel() // 9
        out = torch.empty((n, proj.N, proj.N), dtype=torch.float32, device=v.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(v.device).cuda_stream)
        h = proj.handle
        check(L.gg_set_volume_dev(h, _vp(v), stream), h)
        if n > 0:
            check(L.gg_forward_project_dev(h, _vp(ax), n, _vp(out), None, stream), h)
        ctx.save_for_backward(ax)
        ctx.proj = proj
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (ax,) = ctx.saved_tensors
        return ctx.proj.adjoint(grad_out, ax), None, None


def forward_project(vol, axes, projector):
    """Functional form of ForwardProjector.project."""
    return projector.project(vol, axes)
