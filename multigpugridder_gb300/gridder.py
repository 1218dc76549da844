"""MultiGPUGridder: the reference's user-facing gridder object, over the C ABI.

Mirrors MultiGPUGridder_Matlab_Class (src/Matlab/MultiGPUGridder_Matlab_Class.m)
method for method -- setVolume, forwardProject, backProject, resetVolume,
getVol, reconstructVol, CheckParameters -- with the same defaults and checks.
Arrays are NumPy in the reference's memory layout (x fastest): volumes
[N, N, N] indexed [k, j, i], image stacks [n, N, N], coordAxes [n, 9] (the
MATLAB 9 x n matrix).

Differences from the MATLAB class, all on purpose:
* the CAS volume is prepared on the GPU in setVolume and stays resident; it
  is rebuilt from `Volume` before a forward projection only when a back
  projection has replaced it (the MATLAB class rebuilds it on the host on
  every forwardProject, MultiGPUGridder_Matlab_Class.m:226-227);
* reconstructVol works with the FFTs on the GPU (the MATLAB class refuses,
  :286-288) and takes the images and axes as arguments;
* one GPU per object; use one object per GPU to shard directions
  (multigpugridder_gb300.sharding).
"""
import ctypes
import warnings

import numpy as np

from . import _lib
from ._lib import check


def adjust_interp_factor(volume_size, interp_factor):
    """The power-of-two adjustment of MultiGPUGridder_Matlab_Class.m:69-83."""
    v = int(volume_size)
    f = float(interp_factor)
    if v < 64:
        f = float(np.float32(128) / np.float32(v))
    elif 64 < v < 128:
        f = float(np.float32(256) / np.float32(v))
    elif 128 < v < 256:
        f = float(np.float32(512.0 / v))
    return f


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _own(a):
    """A private FP32 copy: the object keeps arrays by value, as MATLAB does,
    so resetVolume() and later calls never write into the caller's arrays."""
    return np.array(a, dtype=np.float32, order="C", copy=True)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class MultiGPUGridder:
    kerHWidth = 2
    kerTblSize = 501
    extraPadding = 3

    def __init__(self, VolumeSize=0, NumAxes=0, interpFactor=2.0, GPUs=None, RunFFTOnGPU=1, verbose=0,
                 nStreamsFP=10, nStreamsBP=4, MaxAxesToAllocate=1000, precision="f32", bp_mode="ref",
                 adjustInterpFactor=True):
        if VolumeSize == 0:
            raise ValueError("VolumeSize is a required input.")
        if NumAxes == 0:
            raise ValueError("NumAxes is a required input.")
        self.VolumeSize = int(VolumeSize)
        self.NumAxes = int(NumAxes)
        f = adjust_interp_factor(self.VolumeSize, interpFactor) if adjustInterpFactor else float(interpFactor)
        if f != float(interpFactor):
            warnings.warn("interpFactor adjusted from %g to %g so that the volume size will be on the order of 2^n."
                          % (interpFactor, f))
        self.interpFactor = f
        self.GPUs = [0] if GPUs is None or len(GPUs) == 0 else [int(g) for g in GPUs]
        self.RunFFTOnGPU = int(RunFFTOnGPU)
        self.verbose = int(verbose)
        self.nStreamsFP = int(nStreamsFP)
        self.nStreamsBP = int(nStreamsBP)
        self.MaxAxesToAllocate = int(MaxAxesToAllocate)
        # MaskRadius = VolumeSize*interpFactor/2 - 1 (MultiGPUGridder_Matlab_Class.m:101)
        self.MaskRadius = float(np.float32(self.VolumeSize) * np.float32(self.interpFactor) / np.float32(2) - 1)

        L = _lib.lib()
        h = ctypes.c_void_p()
        devs = (ctypes.c_int * len(self.GPUs))(*self.GPUs)
        check(L.gg_create(self.VolumeSize, self.NumAxes, ctypes.c_float(self.interpFactor), self.extraPadding,
                          len(self.GPUs), devs, self.RunFFTOnGPU, self.verbose, ctypes.byref(h)))
        self._h = h
        N, M, V, R = (ctypes.c_int() for _ in range(4))
        L.gg_get_sizes(h, ctypes.byref(N), ctypes.byref(M), ctypes.byref(V), ctypes.byref(R))
        self.M, self.V = M.value, V.value
        self._call("gg_set_max_axes_to_allocate", self.MaxAxesToAllocate)
        self._call("gg_set_num_streams_fp", self.nStreamsFP)
        self._call("gg_set_num_streams_bp", self.nStreamsBP)
        self.set_precision(precision)
        self.set_bp_mode(bp_mode)

        n = self.VolumeSize
        self.Volume = np.zeros((n, n, n), dtype=np.float32)
        self.Images = np.zeros((self.NumAxes, n, n), dtype=np.float32)
        self.coordAxes = np.zeros((self.NumAxes, 9), dtype=np.float32)
        self.CASVolume = np.zeros((self.V,) * 3, dtype=np.float32)
        self.CASImages = np.zeros((self.NumAxes, self.M, self.M), dtype=np.float32) if (not self.RunFFTOnGPU or self.verbose) else None
        self.KBTable = None
        self._cas_from_volume = False

    # ------------------------------------------------------------------ plumbing
    def _call(self, name, *args):
        return check(getattr(_lib.lib(), name)(self._h, *args), self._h)

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

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_precision(self, precision):
        self._call("gg_set_precision", _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision))

    def set_image_precision(self, precision):
        """Storage of the CAS images the back projection reads ("f32",
        "bf16", "f16"), or None to follow set_precision (the default)."""
        if precision is None:
            code = -1
        else:
            code = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self._call("gg_set_image_precision", code)

    def set_bp_mode(self, mode):
        self._call("gg_set_bp_mode", _lib.BP_MODES[mode] if isinstance(mode, str) else int(mode))

    def setKBTable(self, table):
        t = _f32(table).ravel()
        self._call("gg_set_kb_table", _ptr(t), t.size)
        self.KBTable = t

    def setMaskRadius(self, r):
        self.MaskRadius = float(r)
        self._call("gg_set_mask_radius", ctypes.c_float(self.MaskRadius))

    # ---------------------------------------------------------------- MATLAB API
    def setVolume(self, vol):
        """setVolume (MultiGPUGridder_Matlab_Class.m:272-275) + the CAS preparation."""
        self.Volume = _own(vol)
        n = self.VolumeSize
        if self.Volume.shape != (n, n, n):
            raise ValueError("Volume must be %d^3 (got %s)" % (n, self.Volume.shape))
        dims = (ctypes.c_int * 3)(n, n, n)
        self._call("gg_set_volume", _ptr(self.Volume), dims)
        self._cas_from_volume = True

    def setCASVolume(self, cas):
        c = _f32(cas)
        dims = (ctypes.c_int * 3)(*c.shape)
        self._call("gg_set_cas_volume", _ptr(c), dims)
        self._cas_from_volume = False

    def _axes(self, axes):
        a = _f32(axes).reshape(-1, 9)
        return a

    def forwardProject(self, *args):
        """forwardProject(coordAxes) or forwardProject(Volume, coordAxes, MaskRadius)
        (MultiGPUGridder_Matlab_Class.m:198-243) -> images [n, N, N]."""
        if len(args) == 1:
            axes = self._axes(args[0])
        elif len(args) == 3:
            self.Volume = _own(args[0])
            axes = self._axes(args[1])
            self.setMaskRadius(args[2])
            self._cas_from_volume = False
        elif len(args) == 0:
            axes = self._axes(self.coordAxes)
        else:
            raise ValueError("forwardProject(): Unknown input")
        self.coordAxes = axes
        self.CheckParameters()
        if not self._cas_from_volume:
            self.setVolume(self.Volume)
        n = axes.shape[0]
        imgs = np.empty((n, self.VolumeSize, self.VolumeSize), dtype=np.float32)
        cas = np.empty((n, self.M, self.M), dtype=np.float32) if self.CASImages is not None else None
        self._call("gg_forward_project", _ptr(axes), n, _ptr(imgs), _ptr(cas))
        self.Images = imgs
        if cas is not None:
            self.CASImages = cas
        return imgs

    def backProject(self, images=None, axes=None):
        """backProject(images, coordAxes) (MultiGPUGridder_Matlab_Class.m:245-269):
        the CAS volume is zeroed and replaced by the back projection
        (gpuGridder.cpp:330-332)."""
        ax = self._axes(axes if axes is not None else self.coordAxes)
        if images is not None:
            self.Images = _own(images)
            self.coordAxes = ax
            self._call("gg_back_project", _ptr(ax), ax.shape[0], _ptr(self.Images), None, 0)
        elif not self.RunFFTOnGPU and self.CASImages is not None:
            # host-FFT mode without new images: back-project the stored CAS images
            ci = _f32(self.CASImages)
            self._call("gg_back_project", _ptr(ax), ax.shape[0], None, _ptr(ci), 0)
        else:
            self._call("gg_back_project", _ptr(ax), ax.shape[0], _ptr(_f32(self.Images)), None, 0)
        self._cas_from_volume = False

    def backProjectCAS(self, cas_images, axes, accumulate=False):
        """Back projection of CAS images (the reference's host-FFT mode)."""
        ci = _f32(cas_images)
        ax = self._axes(axes)
        self._call("gg_back_project", _ptr(ax), ax.shape[0], None, _ptr(ci), int(bool(accumulate)))
        self._cas_from_volume = False

    def forwardProjectCAS(self, axes):
        """Forward projection returning CAS images [n, M, M] (the kernel output)."""
        ax = self._axes(axes)
        cas = np.empty((ax.shape[0], self.M, self.M), dtype=np.float32)
        if not self._cas_from_volume and self.Volume is not None and np.any(self.Volume):
            self.setVolume(self.Volume)
        self._call("gg_forward_project", _ptr(ax), ax.shape[0], None, _ptr(cas))
        return cas

    def resetVolume(self):
        """resetVolume (MultiGPUGridder_Matlab_Class.m:277-282)."""
        self.Volume[...] = 0
        self.CASVolume[...] = 0
        self._call("gg_reset_volume")
        self._cas_from_volume = False

    def getCASVolume(self):
        out = np.empty((self.V,) * 3, dtype=np.float32)
        self._call("gg_get_cas_volume", _ptr(out))
        self.CASVolume = out
        return out

    def getVol(self):
        """getVol (MultiGPUGridder_Matlab_Class.m:314-327): CAS volume -> volume, on the GPU."""
        n = self.VolumeSize
        out = np.empty((n, n, n), dtype=np.float32)
        self._call("gg_get_volume", _ptr(out))
        self.Volume = out
        return out

    def reconstructVol(self, images=None, axes=None):
        """reconstructVol (MultiGPUGridder_Matlab_Class.m:284-312): back projection
        divided by the plane density (+1e-6), then getVol."""
        if images is not None:
            self.Images = _own(images)
            self.coordAxes = self._axes(axes)
        ax = self._axes(self.coordAxes)
        n = self.VolumeSize
        out = np.empty((n, n, n), dtype=np.float32)
        self._call("gg_reconstruct_volume", _ptr(ax), ax.shape[0], _ptr(self.Images), _ptr(out))
        self.Volume = out
        self._cas_from_volume = False
        return out

    def reconstructVolCTF(self, images, axes, defocus, voltage_kv=300.0, cs_mm=2.7, amp_contrast=0.1,
                          pixel_size=1.0, defocus_v=None, astig_angle=None):
        """reconstructVol with each image's weak-phase CTF applied before the
        back projection (the reference's unimplemented ApplyCTFs flag,
        src/Gridders/AbstractGridder.h:118-119): the CAS images are multiplied
        by the CTF and the plane density back-projects CTF^2.  defocus: one
        value per image in Å (underfocus positive; defocus U when astigmatic);
        defocus_v, astig_angle: per-image defocus V (Å) and the angle of the U
        axis from the image x axis (radians), both or neither; cs_mm in mm;
        pixel_size in Å per image pixel."""
        self.Images = _own(images)
        self.coordAxes = self._axes(axes)
        ax = self._axes(self.coordAxes)
        n_img = ax.shape[0]

        def per_image(x, name):
            v = np.ascontiguousarray(x, dtype=np.float32).reshape(-1)
            if v.size != n_img:
                raise ValueError("%s needs one value per image (%d), got %d" % (name, n_img, v.size))
            return v

        df = per_image(defocus, "defocus")
        if (defocus_v is None) != (astig_angle is None):
            raise ValueError("defocus_v and astig_angle go together")
        dv = per_image(defocus_v, "defocus_v") if defocus_v is not None else None
        an = per_image(astig_angle, "astig_angle") if astig_angle is not None else None
        n = self.VolumeSize
        out = np.empty((n, n, n), dtype=np.float32)
        self._call("gg_reconstruct_volume_ctf", _ptr(ax), n_img, _ptr(self.Images), _ptr(df), _ptr(dv), _ptr(an),
                   float(voltage_kv), float(cs_mm), float(amp_contrast), float(pixel_size), _ptr(out))
        self.Volume = out
        self._cas_from_volume = False
        return out

    def CheckParameters(self):
        """CheckParameters (MultiGPUGridder_Matlab_Class.m:329-344)."""
        a = np.asarray(self.coordAxes, dtype=np.float64).reshape(-1, 9)
        for j in range(3):
            nrm = np.linalg.norm(a[:, 3 * j:3 * j + 3], axis=1)
            if np.any(nrm - 1 > 0.0001):
                warnings.warn("Invalid coordAxes parameter: Each x, y, and z component of the coordinate axes "
                              "needs to have a norm of one")
                break
        if self.interpFactor <= 0:
            raise ValueError("Invalid Interp Factor parameter: must be a non-negative value")
