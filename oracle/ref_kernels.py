"""Runs the reference's own projection kernels (TEST INFRASTRUCTURE ONLY).

oracle/build.py compiles src/Projection/gpuForwardProject.cu and
src/Projection/gpuBackProject.cu of tagarelab/MultiGPUGridder, unmodified,
into sm_103a cubins under oracle/_ref/.  This module loads those cubins with
the CUDA driver API (libcuda, through ctypes) and launches
gpuForwardProjectKernel / gpuBackProjectKernel with the launch geometry of
their RunKernel functions (gpuForwardProject.cu:117-139,
gpuBackProject.cu:130-150), on device buffers owned by the caller (torch
tensors).  It shares the primary context that torch uses.
"""
import ctypes
import math
import os

from . import build as _build

FP_SYMBOL = b"_Z23gpuForwardProjectKernelPKfiPfiS1_ifS1_if"
BP_SYMBOL = b"_Z20gpuBackProjectKernelPfiS_iS_ifPKfif"


def available():
    return all(os.path.exists(p) for _, p in _build.REF_CUBINS.values())


class RefKernels:
    def __init__(self):
        if not available():
            raise FileNotFoundError("reference cubins not built (oracle/build.py build_ref)")
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            dev = ctypes.c_int()
            self._check(self.cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
            self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
            self._check(self.cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.fp_fn = self._load(_build.REF_CUBINS["fp"][1], FP_SYMBOL)
        self.bp_fn = self._load(_build.REF_CUBINS["bp"][1], BP_SYMBOL)

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed with CUresult %d" % (what, rc))

    def _load(self, path, sym):
        mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(mod), path.encode()), "cuModuleLoad(%s)" % path)
        fn = ctypes.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(fn), mod, sym), "cuModuleGetFunction")
        return fn

    def _launch(self, fn, grid, block, args, stream=0):
        # args: list of ctypes scalars; kernelParams is an array of pointers to them
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1], block[2], 0,
                                           ctypes.c_void_p(stream), ptrs, None), "cuLaunchKernel")

    def forward_project(self, d_vol, V, d_img, M, d_axes, n, mask_radius, d_ker, ker_size, ker_hw=2.0, stream=0):
        """gpuForwardProject::RunKernel: grid (32,32), block ceil(M/32)^2.
        The CAS images must be zeroed by the caller (gpuGridder.cpp:232-236)."""
        bs = int(math.ceil(M / 32.0))
        args = [ctypes.c_void_p(d_vol), ctypes.c_int(V), ctypes.c_void_p(d_img), ctypes.c_int(M),
                ctypes.c_void_p(d_axes), ctypes.c_int(n), ctypes.c_float(float(int(mask_radius))),
                ctypes.c_void_p(d_ker), ctypes.c_int(ker_size), ctypes.c_float(ker_hw)]
        self._launch(self.fp_fn, (32, 32, 1), (bs, bs, 1), args, stream)

    def back_project(self, d_vol, V, d_img, M, d_axes, n, mask_radius, d_ker, ker_size, ker_hw=2.0, stream=0):
        """gpuBackProject::RunKernel: block 4^3, grid ceil(V/4)^3; adds into d_vol."""
        g = int(math.ceil(V / 4.0))
        args = [ctypes.c_void_p(d_vol), ctypes.c_int(V), ctypes.c_void_p(d_img), ctypes.c_int(M),
                ctypes.c_void_p(d_axes), ctypes.c_int(n), ctypes.c_float(float(int(mask_radius))),
                ctypes.c_void_p(d_ker), ctypes.c_int(ker_size), ctypes.c_float(ker_hw)]
        self._launch(self.bp_fn, (g, g, g), (4, 4, 4), args, stream)
