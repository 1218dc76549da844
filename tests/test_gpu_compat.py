"""The older entry points of include/gg_compat.h, driven in the order the
reference's Python ctypes class uses them (SetNumberGPUs, SetNumberStreams,
SetAxes, SetVolume, SetImgSize, SetMaskRadius, Forward_Project, GetImages,
ResetVolume, SetImages, Back_Project, GetVolume), with the argtypes that class
declares.  Results must equal the stateless kernel entry points exactly and the
oracle within relative L2 1e-5."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

F = ctypes.POINTER(ctypes.c_float)
I = ctypes.POINTER(ctypes.c_int)


def _bind(L):
    sig = {"Gridder_new": ([], ctypes.c_void_p), "Gridder_delete": ([ctypes.c_void_p], None),
           "SetNumberGPUs": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_void_p),
           "SetNumberStreams": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_void_p),
           "SetVolume": ([ctypes.c_void_p, F, I], ctypes.c_void_p), "GetVolume": ([ctypes.c_void_p], F),
           "ResetVolume": ([ctypes.c_void_p], ctypes.c_void_p), "SetImages": ([ctypes.c_void_p, F], ctypes.c_void_p),
           "GetImages": ([ctypes.c_void_p], F), "SetAxes": ([ctypes.c_void_p, F, I], ctypes.c_void_p),
           "SetImgSize": ([ctypes.c_void_p, I], ctypes.c_void_p), "SetMaskRadius": ([ctypes.c_void_p, F], ctypes.c_void_p),
           "Forward_Project": ([ctypes.c_void_p], ctypes.c_void_p), "Back_Project": ([ctypes.c_void_p], ctypes.c_void_p)}
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res


def test_reference_ctypes_call_sequence(cuda, gglib):
    import torch

    L = gglib
    _bind(L)
    V = 48
    vol = O.blob_volume(V, 8, seed=81).astype(np.float64)
    spec = np.fft.fftshift(np.fft.fftn(np.fft.fftshift(vol)))
    cas = np.ascontiguousarray((spec.real + spec.imag).astype(np.float32))
    axes = np.concatenate([O.quaternion_axes(18, 82), np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1], [1, 0, 0, 1, 0, 0, 0, 0, 1]])])
    axes = np.ascontiguousarray(axes.astype(np.float32))
    n, R = len(axes), V // 2 - 2
    ker = O.Params(16).ker

    vol_arr = cas.copy()
    g = L.Gridder_new()
    try:
        L.SetNumberGPUs(g, 1)
        L.SetNumberStreams(g, 20)
        L.SetAxes(g, axes.ctypes.data_as(F), (ctypes.c_int * 3)(n * 9, 1, 1))
        L.SetVolume(g, vol_arr.ctypes.data_as(F), (ctypes.c_int * 3)(V, V, V))
        L.SetImgSize(g, (ctypes.c_int * 3)(V, V, V))
        L.SetMaskRadius(g, ctypes.byref(ctypes.c_float(R)))
        L.Forward_Project(g)
        p = L.GetImages(g)
        assert p, L.gg_global_error()
        imgs = np.ctypeslib.as_array(p, shape=(n, V, V)).copy()

        # the stateless entry point on the same inputs
        d = {k: torch.from_numpy(a).to(cuda) for k, a in (("cas", cas), ("axes", axes), ("ker", ker))}
        vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        out = torch.empty((n, V, V), device=cuda)
        assert L.gg_forward_project_kernel(vp(d["cas"]), vp(out), vp(d["ker"]), vp(d["axes"]), 2.0, n, V, V, 0, R, 501,
                                           None) == 0
        torch.cuda.synchronize()
        assert np.array_equal(imgs, out.cpu().numpy())
        assert O.rel_l2(imgs, O.fp_ref_f32(cas, axes, V, R, ker)) < 1e-5

        L.ResetVolume(g)
        assert not vol_arr.any()
        L.SetImages(g, p)
        L.Back_Project(g)
        q = L.GetVolume(g)
        assert ctypes.addressof(q.contents) == vol_arr.ctypes.data  # the registered array, written in place
        bp = torch.zeros((V,) * 3, device=cuda)
        d_img = torch.from_numpy(imgs).to(cuda)
        assert L.gg_back_project_kernel(vp(bp), vp(d_img), vp(d["ker"]), vp(d["axes"]), 2.0, n, V, V, R, 501, 0,
                                        None) == 0
        torch.cuda.synchronize()
        assert np.array_equal(vol_arr, bp.cpu().numpy())
        assert O.rel_l2(vol_arr, O.bp_ref_f32(imgs, axes, V, R, ker)) < 1e-5
    finally:
        L.Gridder_delete(g)
