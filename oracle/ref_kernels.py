"""Runs the reference's own kernels (TEST INFRASTRUCTURE ONLY).

oracle/build.py compiles src/Projection/gpuForwardProject.cu,
src/Projection/gpuBackProject.cu and the twelve src/Filters/*Filter.cu of
tagarelab/MultiGPUGridder, unmodified, into sm_103a cubins under oracle/_ref/.
This module loads those cubins with the CUDA driver API (libcuda, through
ctypes) and launches their kernels with the launch geometry of the
reference's own host code (RunKernel, gpuForwardProject.cu:117-139 and
gpuBackProject.cu:130-150; each filter's UpdateFilter), on device buffers
owned by the caller (torch tensors).  It shares the primary context that
torch uses.

RefFilters also assembles the reference's two image-stage chains from those
filters and cuFFT (gpuGridder::CASImgsToImgs and ::ImgsToCASImgs,
gpuGridder.cpp:432-596): one cufftPlan2d C2C plan and one cufftExecC2C per
image, as the reference runs them.
"""
import ctypes
import math
import os

from . import build as _build

FP_SYMBOL = b"_Z23gpuForwardProjectKernelPKfiPfiS1_ifS1_if"
BP_SYMBOL = b"_Z20gpuBackProjectKernelPfiS_iS_ifPKfif"


def available():
    return all(os.path.exists(_build.REF_CUBINS[k][1]) for k in ("fp", "bp"))


def filters_available():
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


# Mangled names of the filter kernels (the filters declare them with C++
# linkage; cufftComplex is CUDA's float2).
FILTER_SYMBOLS = {
    "complex_to_cas": ("ComplexToCAS", b"_Z18ComplexToCASKernelP6float2Pfii"),
    "cas_to_complex": ("CASToComplex", b"_Z24CASVolumeToComplexKernelPfP6float2iib"),
    "shift2d_f": ("FFTShift2D", b"_Z20cufftShift_2D_kernelIfEvPT_ii"),
    "shift2d_c": ("FFTShift2D", b"_Z20cufftShift_2D_kernelI6float2EvPT_ii"),
    "shift3d_f": ("FFTShift3D", b"_Z16FFTShift3DKernelIfEvPT_i"),
    "shift3d_c": ("FFTShift3D", b"_Z16FFTShift3DKernelI6float2EvPT_i"),
    "pad": ("PadVolume", b"_Z15PadVolumeKernelPfS_iiiiiiiii"),
    "crop": ("CropVolume", b"_Z16CropVolumeKernelIfEvPT_S1_iiiiiiiii"),
    "divide": ("DivideVolume", b"_Z19DivideVolumesKernelPfS_ii"),
    "multiply_c": ("MultiplyVolume", b"_Z21MultiplyVolumesKernelP6float2Pfii"),
    "multiply_f": ("MultiplyVolume", b"_Z21MultiplyVolumesKernelPfS_ii"),
    "add": ("AddVolume", b"_Z15AddVolumeKernelIfEvPT_S1_ii"),
    "divide_scalar": ("DivideScalar", b"_Z18DivideScalarKernelPffii"),
    "real_to_complex": ("RealToComplex", b"_Z19RealToComplexKernelPfP6float2ii"),
    "complex_to_real": ("ComplexToReal", b"_Z19ComplexToRealKernelP6float2Pfii"),
}

CUFFT_C2C = 0x29
CUFFT_FORWARD = -1
CUFFT_INVERSE = 1


def _grid32(n):
    """The filters' launch grid: ceil(n / 32) blocks of 32 x 32 per axis, at least one."""
    return max(int(math.ceil(n / 32.0)), 1)


class RefFilters(RefKernels):
    """The reference's filter kernels, launched as their UpdateFilter does:
    block 32 x 32, grid ceil(size / 32)^2; n_slices <= 0 selects the size^3
    volume form where the filter has one."""

    def __init__(self):
        if not filters_available():
            raise FileNotFoundError("reference filter cubins not built (oracle/build.py build_ref)")
        super().__init__()
        self.fn = {k: self._load(_build.REF_CUBINS["filter_" + f][1], sym) for k, (f, sym) in FILTER_SYMBOLS.items()}
        self.cufft = None

    def _run(self, key, size, args, grid_size=None):
        g = _grid32(size if grid_size is None else grid_size)
        self._launch(self.fn[key], (g, g, 1), (32, 32, 1), args)

    @staticmethod
    def _p(x):
        return ctypes.c_void_p(x)

    def complex_to_cas(self, d_c, d_r, size, n_slices):
        """ComplexToCASFilter::UpdateFilter (ComplexToCASFilter.cu:28-81)."""
        ns = size if n_slices <= 0 else n_slices
        self._run("complex_to_cas", size, [self._p(d_c), self._p(d_r), ctypes.c_int(size), ctypes.c_int(ns)])

    def cas_to_complex(self, d_r, d_c, size, n_slices):
        """CASToComplexFilter::UpdateFilter (CASToComplexFilter.cu:83-134)."""
        vol = n_slices <= 0
        ns = size if vol else n_slices
        self._run("cas_to_complex", size, [self._p(d_r), self._p(d_c), ctypes.c_int(size), ctypes.c_int(ns),
                                           ctypes.c_bool(vol)])

    def fftshift_2d(self, d, size, n_slices, complex_elems):
        """FFTShift2DFilter<float | cufftComplex>::UpdateFilter (FFTShift2DFilter.cu:70-108)."""
        self._run("shift2d_c" if complex_elems else "shift2d_f", size,
                  [self._p(d), ctypes.c_int(size), ctypes.c_int(n_slices)])

    def fftshift_3d(self, d, size, complex_elems):
        """FFTShift3DFilter<float | cufftComplex>::UpdateFilter (FFTShift3DFilter.cu:104-140)."""
        self._run("shift3d_c" if complex_elems else "shift3d_f", size, [self._p(d), ctypes.c_int(size)])

    def pad_volume(self, d_in, d_out, ix, iy, iz, px, py, pz):
        """PadVolumeFilter::UpdateFilter (PadVolumeFilter.cu:38-98): writes
        the interior only (the caller zeroes the output first)."""
        ox, oy, oz = ix + 2 * px, iy + 2 * py, iz + 2 * pz
        args = [self._p(d_in), self._p(d_out)] + [ctypes.c_int(v) for v in (ix, iy, iz, ox, oy, oz, px, py, pz)]
        self._run("pad", 0, args, grid_size=max(ox, oy))

    def crop_volume(self, d_in, d_out, ix, iy, iz, cx, cy, cz):
        """CropVolumeFilter::UpdateFilter (CropVolumeFilter.cu:41-98)."""
        ox, oy, oz = ix - 2 * cx, iy - 2 * cy, iz - 2 * cz
        args = [self._p(d_in), self._p(d_out)] + [ctypes.c_int(v) for v in (ix, iy, iz, ox, oy, oz, cx, cy, cz)]
        self._run("crop", 0, args, grid_size=ix)

    def _slices(self, key, d_a, d_b, size, n_slices):
        ns = size if n_slices <= 0 else n_slices
        self._run(key, size, [self._p(d_a), self._p(d_b), ctypes.c_int(size), ctypes.c_int(ns)])

    def divide_volumes(self, d_a, d_b, size, n_slices):
        """DivideVolumeFilter::UpdateFilter (DivideVolumeFilter.cu:35-83)."""
        self._slices("divide", d_a, d_b, size, n_slices)

    def multiply_volumes(self, d_a, d_b, size, n_slices, complex_elems):
        """MultiplyVolumeFilter<float | cufftComplex>::UpdateFilter (MultiplyVolumeFilter.cu:57-105)."""
        self._slices("multiply_c" if complex_elems else "multiply_f", d_a, d_b, size, n_slices)

    def add_volumes(self, d_a, d_b, size, n_slices):
        """AddVolumeFilter::UpdateFilter (AddVolumeFilter.cu:29-69); the
        reference requires n_slices > 0."""
        self._slices("add", d_a, d_b, size, n_slices)

    def divide_scalar(self, d_a, scalar, size, n_slices):
        """DivideScalarFilter::UpdateFilter (DivideScalarFilter.cu:27-75)."""
        ns = size if n_slices <= 0 else n_slices
        self._run("divide_scalar", size, [self._p(d_a), ctypes.c_float(scalar), ctypes.c_int(size), ctypes.c_int(ns)])

    def real_to_complex(self, d_r, d_c, size, n_slices):
        """RealToComplexFilter::UpdateFilter (RealToComplexFilter.cu:27-74)."""
        self._slices("real_to_complex", d_r, d_c, size, n_slices)

    def complex_to_real(self, d_c, d_r, size, n_slices):
        """ComplexToRealFilter::UpdateFilter (ComplexToRealFilter.cu:27-73)."""
        self._slices("complex_to_real", d_c, d_r, size, n_slices)

    # ---- the reference's image stages -------------------------------------
    def _fft_each(self, d_c, M, n, direction):
        """One cufftPlan2d(M, M, C2C) plan, cufftExecC2C in place per image
        (gpuGridder.cpp:447-451, 473-479 and 555-559, 576-582)."""
        if self.cufft is None:
            self.cufft = ctypes.CDLL("libcufft.so.12")
        plan = ctypes.c_int()
        rc = self.cufft.cufftPlan2d(ctypes.byref(plan), M, M, CUFFT_C2C)
        if rc != 0:
            raise RuntimeError("cufftPlan2d failed with %d" % rc)
        try:
            step = M * M * 8
            for i in range(n):
                ptr = ctypes.c_void_p(d_c + i * step)
                rc = self.cufft.cufftExecC2C(plan, ptr, ptr, direction)
                if rc != 0:
                    raise RuntimeError("cufftExecC2C failed with %d" % rc)
        finally:
            self.cufft.cufftDestroy(plan)

    def cas_imgs_to_imgs(self, d_cas, d_imgs, d_complex, M, N, n, interp):
        """gpuGridder::CASImgsToImgs (gpuGridder.cpp:432-518): CAS -> complex,
        2-D shift, inverse C2C per image, shift, real part (into d_cas), crop
        the centre N x N into d_imgs, divide by N^2 interp^2.  d_complex holds
        n*M*M complex values; all on the default stream."""
        self.cas_to_complex(d_cas, d_complex, M, n)
        self.fftshift_2d(d_complex, M, n, True)
        self._fft_each(d_complex, M, n, CUFFT_INVERSE)
        self.fftshift_2d(d_complex, M, n, True)
        self.complex_to_real(d_complex, d_cas, M, n)
        c = (M - N) // 2
        self.crop_volume(d_cas, d_imgs, M, M, n, c, c, 0)
        self.divide_scalar(d_imgs, float(N * N * interp * interp), N, n)

    def imgs_to_cas_imgs(self, d_imgs, d_cas, d_complex, M, N, n):
        """gpuGridder::ImgsToCASImgs (gpuGridder.cpp:520-596): pad into the
        zeroed d_cas, real -> complex, shift, forward C2C per image, shift,
        complex -> CAS into d_cas."""
        p = (M - N) // 2
        self.pad_volume(d_imgs, d_cas, N, N, n, p, p, 0)
        self.real_to_complex(d_cas, d_complex, M, n)
        self.fftshift_2d(d_complex, M, n, True)
        self._fft_each(d_complex, M, n, CUFFT_FORWARD)
        self.fftshift_2d(d_complex, M, n, True)
        self.complex_to_cas(d_complex, d_cas, M, n)
