"""CPU oracle for the Kaiser-Bessel Fourier-slice projection path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by the cpu_baseline / reference arm of bench.py.  The
product package never imports it.

Restates in NumPy (FP64 unless stated) the MATLAB host math of
tagarelab/MultiGPUGridder and the stage order of its C++ engine, and wraps the
C restatement of the two CUDA projection kernels (gg_oracle.c).  Each function
cites the reference file:line it follows.

Array convention: the reference passes MATLAB column-major arrays, so element
(i, j, k) (1-based in MATLAB) sits at flat offset i + j*N + k*N*N.  Here arrays
are NumPy C-order indexed [k, j, i] (x fastest in memory), which is the same
memory layout.  Images are [n, j, i]; coordinate axes are [n, 9].
"""
import ctypes
import math
import os

import numpy as np

from . import build as _build

# --------------------------------------------------------------------------
# Kaiser-Bessel window and tables
# --------------------------------------------------------------------------


def matlab_colon(a, d, b):
    """MATLAB ``a:d:b`` (the count and the symmetric endpoint evaluation)."""
    n = int(math.floor((b - a) / d + 1e-10)) + 1
    k = np.arange(n, dtype=np.float64)
    out = a + k * d
    last = a + (n - 1) * d
    if abs(last - b) < 1e-9 * max(1.0, abs(b)):
        last = b
    # MATLAB evaluates the second half backwards from the last element
    half = n // 2
    out[half:] = last - (n - 1 - k[half:]) * d
    return out


def kernel_alpha(hw):
    """src/Matlab/utils/kernelAlpha.m:6-10 (alpha = 10 for half-width 2)."""
    alphavals = [5.5, 10.0, 10.2, 13, 17]
    if hw > 5 or hw < 1:
        raise ValueError("invalid kernel half-width %r" % (hw,))
    return alphavals[int(hw) - 1]


def bessel_i0(x):
    """Modified Bessel function I0 by its power series sum_k ((x/2)^k / k!)^2
    (Abramowitz & Stegun 9.6.10); converges to double precision for x <= 20."""
    x = np.asarray(x, dtype=np.float64)
    q = (x / 2.0) ** 2
    term = np.ones_like(x)
    total = np.ones_like(x)
    for k in range(1, 80):
        term = term * q / (k * k)
        total = total + term
    return total


def grid_lib_kaiser(n, alpha, k):
    """src/Matlab/utils/gridLibKaiser.m:5-15: I0(alpha*sqrt(1-(q/n)^2))/I0(alpha)."""
    k = np.asarray(k, dtype=np.float64)
    r0 = bessel_i0(alpha)
    w = np.zeros_like(k)
    inside = np.abs(k) <= n
    r = np.sqrt(1.0 - (k[inside] / n) ** 2)
    w[inside] = bessel_i0(alpha * r) / r0
    return w


def kb_table(hw=2, size=501):
    """src/Matlab/utils/getKernelFiltTable.m:1-22, in FP64.

    Unit-integral KB window on x in [-hw, hw] (size points), edge value
    subtracted, last value forced to 0, then scaled by (sum over the 5^3
    integer taps)^(-1/3).  The reference hands single(w) to the GPU
    (MultiGPUGridder_Matlab_Class.m:128); take .astype(np.float32) for that.
    """
    alpha = kernel_alpha(hw)
    delta = 2.0 * hw / (size - 1)
    x = matlab_colon(-hw, delta, hw)
    assert x.size == size
    w = grid_lib_kaiser(hw, alpha, x)
    w = w / np.sum(w * delta)
    w = w - w[0]
    w[-1] = 0.0
    center = (size + 1) / 2.0
    scale = (center - 1) / hw
    index = np.arange(-hw, hw + 1) * scale + center  # 1-based
    ker = w[np.round(index).astype(int) - 1]
    denom = np.sum(np.einsum("i,j,k->ijk", ker, ker, ker))
    return w / denom ** (1.0 / 3.0)


def precomp(M, hw=2):
    """src/Matlab/utils/getPreComp.m:1-28: deapodization vector of length M.

    KB sampled at 1/4 voxel (oversampling 4), edge value subtracted, placed at
    the centre of a 4M line, real(fftshift(fft(fftshift(.)))), the central M
    samples taken and normalised as fc0 ./ (.).
    """
    ovr = 4
    alpha = kernel_alpha(hw)
    x = matlab_colon(-hw, 1.0 / ovr, hw)
    w = grid_lib_kaiser(hw, alpha, x)
    w = w - w[0]
    w[-1] = 0.0
    whw = (x.size - 1) // 2
    L = M * ovr
    line = np.zeros(L)
    xc = L // 2  # 0-based position of MATLAB's numel/2+1
    line[xc - whw: xc + whw + 1] = w
    pc = np.real(np.fft.fftshift(np.fft.fft(np.fft.fftshift(line))))
    c = L // 2
    fc0 = pc[c]
    return fc0 / pc[c - M // 2: c + M // 2]


def get_sizes(N, interp, pad):
    """src/Matlab/utils/getSizes.m:1-16 (0-based begin offsets)."""
    M = int(round(N * interp))
    V = M + 2 * pad
    return {"N": N, "M": M, "V": V,
            "interp_origB": M // 2 - N // 2,  # where the N-box starts inside M
            "cas_interpB": V // 2 - M // 2}   # where the M-box starts inside V


def default_mask_radius(N, interp):
    """MaskRadius = N*interp/2 - 1 (MultiGPUGridder_Matlab_Class.m:101,
    AbstractGridder.cpp:13), truncated to int at RunKernel
    (gpuForwardProject.h:57, gpuBackProject.h:56)."""
    return int(np.float32(N) * np.float32(interp) / np.float32(2) - np.float32(1))


# --------------------------------------------------------------------------
# CAS conversions (src/Matlab/utils/ToCAS.m, FromCAS.m)
# --------------------------------------------------------------------------


def to_cas(c):
    """ToCAS.m:5: r = real(c) + imag(c)."""
    return np.real(c) + np.imag(c)


def from_cas(r, axes=None):
    """FromCAS.m:7-13 over the given axes (default: all): c = 0.5(r + r_flip)
    + 0.5i(r - r_flip) where r_flip pairs index m with s - m, and the first
    index along every converted axis is zero."""
    r = np.asarray(r, dtype=np.float64)
    if axes is None:
        axes = tuple(range(r.ndim))
    c = np.zeros(r.shape, dtype=np.complex128)
    sl_in = [slice(None)] * r.ndim
    sl_fl = [slice(None)] * r.ndim
    for ax in axes:
        sl_in[ax] = slice(1, None)
        sl_fl[ax] = slice(None, 0, -1)
    a = r[tuple(sl_in)]
    b = r[tuple(sl_fl)]
    c[tuple(sl_in)] = 0.5 * (a + b) + 0.5j * (a - b)
    return c


# --------------------------------------------------------------------------
# Volume <-> CAS volume (CASFromVol_Gridder.m, volFromCAS_Gridder.m)
# --------------------------------------------------------------------------


def _precomp3(M, hw):
    p = precomp(M, hw)
    return p[:, None, None] * p[None, :, None] * p[None, None, :]


def cas_from_vol(vol, hw=2, interp=2, pad=3):
    """CASFromVol_Gridder.m:25-60: zero-pad N^3 -> M^3 centred, multiply by
    the separable precomp, fftshift(fftn(fftshift())), Re+Im, zero-pad by
    `pad` on every side -> V^3.  FP64."""
    vol = np.asarray(vol)
    N = vol.shape[0]
    s = get_sizes(N, interp, pad)
    M, V = s["M"], s["V"]
    b = s["interp_origB"]
    iv = np.zeros((M, M, M))
    iv[b:b + N, b:b + N, b:b + N] = vol
    iv *= _precomp3(M, hw)
    F = np.fft.fftshift(np.fft.fftn(np.fft.fftshift(iv)))
    out = np.zeros((V, V, V))
    out[pad:pad + M, pad:pad + M, pad:pad + M] = to_cas(F)
    return out


def vol_from_cas(cas, N, hw=2, interp=2):
    """volFromCAS_Gridder.m:26-56: crop the padding, FromCAS, real(fftshift(
    ifftn(fftshift()))) (1/M^3), multiply by the precomp, crop N^3."""
    cas = np.asarray(cas, dtype=np.float64)
    V = cas.shape[0]
    M = int(round(N * interp))
    b = V // 2 - M // 2
    ic = cas[b:b + M, b:b + M, b:b + M]
    F = from_cas(ic)
    iv = np.real(np.fft.fftshift(np.fft.ifftn(np.fft.fftshift(F))))
    iv *= _precomp3(M, hw)
    ob = M // 2 - N // 2
    return iv[ob:ob + N, ob:ob + N, ob:ob + N]


# --------------------------------------------------------------------------
# CAS images <-> images (gpuGridder.cpp:432-518 and :520-596;
# imgsFromCASImgs.m:7-21, CASImgsFromImgs.m:3-10)
# --------------------------------------------------------------------------


def imgs_from_cas_imgs(cas_imgs, N):
    """CAS images [n, M, M] -> images [n, N, N]: FromCAS per slice (first row
    and column zero), fftshift2, inverse FFT normalised by 1/M^2 (the GPU path
    divides cuFFT's unnormalised result by ImgSize^2*interp^2,
    gpuGridder.cpp:509-517), fftshift2, real part, centred crop."""
    r = np.asarray(cas_imgs, dtype=np.float64)
    M = r.shape[-1]
    c = from_cas(r, axes=(1, 2))
    y = np.real(np.fft.fftshift(np.fft.ifft2(np.fft.fftshift(c, axes=(1, 2))), axes=(1, 2)))
    b = (M - N) // 2
    return y[:, b:b + N, b:b + N]


def cas_imgs_from_imgs(imgs, M):
    """Images [n, N, N] -> CAS images [n, M, M]: centred zero-pad, fftshift2,
    forward FFT (unnormalised), fftshift2, Re+Im."""
    x = np.asarray(imgs, dtype=np.float64)
    n, N = x.shape[0], x.shape[-1]
    b = (M - N) // 2
    p = np.zeros((n, M, M))
    p[:, b:b + N, b:b + N] = x
    F = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(p, axes=(1, 2))), axes=(1, 2))
    return to_cas(F)


# --------------------------------------------------------------------------
# The C restatement of the kernels
# --------------------------------------------------------------------------

_LIB = None
_f = ctypes.POINTER(ctypes.c_float)
_d = ctypes.POINTER(ctypes.c_double)


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        sig32 = [_f, ctypes.c_int, _f, ctypes.c_int, _f, ctypes.c_int, ctypes.c_int, _f, ctypes.c_int, ctypes.c_float]
        sig64 = [_d, ctypes.c_int, _d, ctypes.c_int, _d, ctypes.c_int, ctypes.c_int, _f, ctypes.c_int, ctypes.c_double]
        for name, sig in (("gg_oracle_fp_ref_f32", sig32), ("gg_oracle_bp_ref_f32", sig32),
                          ("gg_oracle_fp_f64", sig64), ("gg_oracle_bp_ref_f64", sig64),
                          ("gg_oracle_bp_adjoint_f64", sig64)):
            fn = getattr(L, name)
            fn.argtypes = sig
            fn.restype = None
        L.gg_oracle_num_threads.restype = ctypes.c_int
        L.gg_oracle_set_num_threads.argtypes = [ctypes.c_int]
        _LIB = L
    return _LIB


def _p32(a):
    return a.ctypes.data_as(_f)


def _p64(a):
    return a.ctypes.data_as(_d)


def _axes(axes, dtype):
    a = np.ascontiguousarray(np.asarray(axes, dtype=dtype).reshape(-1, 9))
    return a


def set_threads(n):
    lib().gg_oracle_set_num_threads(int(n))


def num_threads():
    return int(lib().gg_oracle_num_threads())


def fp_ref_f32(cas_vol, axes, M, mask_radius, ker, ker_hw=2.0):
    """gpuForwardProjectKernel restated in FP32 -> CAS images [n, M, M]."""
    vol = np.ascontiguousarray(cas_vol, dtype=np.float32)
    V = vol.shape[0]
    ax = _axes(axes, np.float32)
    ker = np.ascontiguousarray(ker, dtype=np.float32)
    out = np.zeros((ax.shape[0], M, M), dtype=np.float32)
    lib().gg_oracle_fp_ref_f32(_p32(vol), V, _p32(out), M, _p32(ax), ax.shape[0], int(mask_radius),
                               _p32(ker), ker.size, float(ker_hw))
    return out


def bp_ref_f32(cas_imgs, axes, V, mask_radius, ker, ker_hw=2.0, out=None):
    """gpuBackProjectKernel restated in FP32 -> CAS volume [V, V, V] (accumulates into out)."""
    img = np.ascontiguousarray(cas_imgs, dtype=np.float32)
    M = img.shape[-1]
    ax = _axes(axes, np.float32)
    ker = np.ascontiguousarray(ker, dtype=np.float32)
    if out is None:
        out = np.zeros((V, V, V), dtype=np.float32)
    lib().gg_oracle_bp_ref_f32(_p32(out), V, _p32(img), M, _p32(ax), ax.shape[0], int(mask_radius),
                               _p32(ker), ker.size, float(ker_hw))
    return out


def fp_f64(cas_vol, axes, M, mask_radius, ker, ker_hw=2.0):
    vol = np.ascontiguousarray(cas_vol, dtype=np.float64)
    V = vol.shape[0]
    ax = _axes(axes, np.float64)
    ker = np.ascontiguousarray(ker, dtype=np.float32)
    out = np.zeros((ax.shape[0], M, M), dtype=np.float64)
    lib().gg_oracle_fp_f64(_p64(vol), V, _p64(out), M, _p64(ax), ax.shape[0], int(mask_radius),
                           _p32(ker), ker.size, float(ker_hw))
    return out


def bp_ref_f64(cas_imgs, axes, V, mask_radius, ker, ker_hw=2.0):
    img = np.ascontiguousarray(cas_imgs, dtype=np.float64)
    M = img.shape[-1]
    ax = _axes(axes, np.float64)
    ker = np.ascontiguousarray(ker, dtype=np.float32)
    out = np.zeros((V, V, V), dtype=np.float64)
    lib().gg_oracle_bp_ref_f64(_p64(out), V, _p64(img), M, _p64(ax), ax.shape[0], int(mask_radius),
                               _p32(ker), ker.size, float(ker_hw))
    return out


def bp_adjoint_f64(cas_imgs, axes, V, mask_radius, ker, ker_hw=2.0):
    img = np.ascontiguousarray(cas_imgs, dtype=np.float64)
    M = img.shape[-1]
    ax = _axes(axes, np.float64)
    ker = np.ascontiguousarray(ker, dtype=np.float32)
    out = np.zeros((V, V, V), dtype=np.float64)
    lib().gg_oracle_bp_adjoint_f64(_p64(out), V, _p64(img), M, _p64(ax), ax.shape[0], int(mask_radius),
                                   _p32(ker), ker.size, float(ker_hw))
    return out


# --------------------------------------------------------------------------
# Whole-path restatements (MultiGPUGridder_Matlab_Class.m)
# --------------------------------------------------------------------------


class Params:
    """Object parameters with the reference defaults: kerHWidth 2, table 501,
    extraPadding 3 (MultiGPUGridder_Matlab_Class.m:23-25, :101)."""

    def __init__(self, N, interp=2.0, pad=3, hw=2, table_size=501, mask_radius=None):
        self.N = int(N)
        self.interp = float(interp)
        self.pad = int(pad)
        self.hw = hw
        s = get_sizes(self.N, self.interp, self.pad)
        self.M, self.V = s["M"], s["V"]
        self.ker = kb_table(hw, table_size).astype(np.float32)
        self.mask_radius = default_mask_radius(self.N, self.interp) if mask_radius is None else int(mask_radius)


def forward_project(vol, axes, p, precision="f64"):
    """forwardProject (MultiGPUGridder_Matlab_Class.m:198-243 with the GPU FFT
    path): CAS volume prep, forward projection, CAS images -> images.
    Returns (images [n,N,N], cas_images [n,M,M])."""
    cas = cas_from_vol(vol, p.hw, p.interp, p.pad)
    if precision == "f32":
        ci = fp_ref_f32(cas.astype(np.float32), axes, p.M, p.mask_radius, p.ker, p.hw).astype(np.float64)
    else:
        ci = fp_f64(cas, axes, p.M, p.mask_radius, p.ker, p.hw)
    return imgs_from_cas_imgs(ci, p.N), ci


def back_project(imgs, axes, p, precision="f64", mode="ref"):
    """backProject (gpuGridder.cpp:307-430): images -> CAS images -> CAS volume."""
    ci = cas_imgs_from_imgs(imgs, p.M)
    return back_project_cas(ci, axes, p, precision, mode)


def back_project_cas(ci, axes, p, precision="f64", mode="ref"):
    if mode == "adjoint":
        return bp_adjoint_f64(ci, axes, p.V, p.mask_radius, p.ker, p.hw)
    if precision == "f32":
        return bp_ref_f32(ci.astype(np.float32), axes, p.V, p.mask_radius, p.ker, p.hw).astype(np.float64)
    return bp_ref_f64(ci, axes, p.V, p.mask_radius, p.ker, p.hw)


def reconstruct_vol(imgs, axes, p, precision="f64"):
    """reconstructVol (MultiGPUGridder_Matlab_Class.m:284-312): back project
    the images, back project all-ones CAS images (plane density), divide
    CAS ./ (PD + 1e-6), volFromCAS."""
    cas = back_project(imgs, axes, p, precision)
    ones = np.ones((np.asarray(axes).reshape(-1, 9).shape[0], p.M, p.M))
    pd = back_project_cas(ones, axes, p, precision)
    return vol_from_cas(cas / (pd + 1e-6), p.N, p.hw, p.interp), cas, pd


def electron_wavelength(voltage_kv):
    """Relativistic electron wavelength in Å at the accelerating voltage:
    h / sqrt(2 m e U (1 + e U / (2 m c^2))) = 12.2643247 / sqrt(U (1 + 0.978466e-6 U))."""
    U = float(voltage_kv) * 1e3
    return 12.2643247 / math.sqrt(U * (1.0 + 0.978466e-6 * U))


def ctf_cas(M, defocus, voltage_kv, cs_mm, amp_contrast, pixel_size, defocus_v=None, astig_angle=None):
    """Weak-phase CTF on the CAS-image grid, FP64, shape (n, M, M), DC at
    (M/2, M/2).  No reference counterpart (the reference declares only the
    ApplyCTFs flag, src/Gridders/AbstractGridder.h:118-119):
    CTF = -(sqrt(1 - A^2) sin chi + A cos chi),
    chi = pi lambda df s^2 - pi/2 Cs lambda^3 s^4, s = |(i, j) - M/2| / (M px).
    Astigmatic (defocus_v, astig_angle given): defocus is U and
    df = (U + V)/2 + (U - V)/2 cos 2(theta - angle), theta the angle of the
    frequency (i - M/2, j - M/2) from the x axis."""
    lam = electron_wavelength(voltage_kv)
    f = (np.arange(M) - M // 2) / (M * float(pixel_size))
    fx, fy = f[None, :], f[:, None]
    s2 = fx ** 2 + fy ** 2
    du = np.asarray(defocus, dtype=np.float64).reshape(-1, 1, 1)
    if defocus_v is None:
        df = du
    else:
        dv = np.asarray(defocus_v, dtype=np.float64).reshape(-1, 1, 1)
        ang = np.asarray(astig_angle, dtype=np.float64).reshape(-1, 1, 1)
        theta = np.arctan2(np.broadcast_to(fy, s2.shape), np.broadcast_to(fx, s2.shape))[None]
        df = 0.5 * (du + dv) + 0.5 * (du - dv) * np.cos(2.0 * (theta - ang))
    chi = math.pi * lam * df * s2 - 0.5 * math.pi * (cs_mm * 1e7) * lam ** 3 * s2 ** 2
    A = float(amp_contrast)
    return -(math.sqrt(1.0 - A * A) * np.sin(chi) + A * np.cos(chi))


def reconstruct_vol_ctf(imgs, axes, p, defocus, voltage_kv, cs_mm, amp_contrast, pixel_size, precision="f64",
                        defocus_v=None, astig_angle=None):
    """reconstructVol with the CTF applied to each CAS image before the back
    projection and CTF^2 images as the plane density:
    volFromCAS(BP(CTF . CAS(img)) ./ (BP(CTF^2) + 1e-6))."""
    c = ctf_cas(p.M, defocus, voltage_kv, cs_mm, amp_contrast, pixel_size, defocus_v, astig_angle)
    if precision == "f32":
        c = c.astype(np.float32).astype(np.float64)
    ci = cas_imgs_from_imgs(imgs, p.M) * c
    cas = back_project_cas(ci, axes, p, precision)
    pd = back_project_cas(c * c, axes, p, precision)
    return vol_from_cas(cas / (pd + 1e-6), p.N, p.hw, p.interp), cas, pd


def forward_operator(vol, axes, p):
    """The whole forward operator in FP64, volume -> images (linear in vol)."""
    return forward_project(vol, axes, p, "f64")[0]


def forward_adjoint(y, axes, p):
    """Exact adjoint of forward_operator, images -> volume, in FP64 (no
    reference counterpart).  By stage:
      images -> CAS images: pad, shift, FFT, shift, Re+Im (FromCAS^T of a
        Hermitian spectrum), first row and column zeroed, / M^2;
      CAS images -> CAS volume: bp_adjoint_f64;
      CAS volume -> volume: inner crop, shift, FFT, shift, Re+Im, * precomp,
        centred crop (ToCAS^T maps g to (1+i) g and the unnormalised FFT's
        adjoint of a real input is conj(FFT), so Re((1+i) conj(F)) = Re F + Im F)."""
    M, N = p.M, p.N
    ci = cas_imgs_from_imgs(y, M)
    ci[:, 0, :] = 0
    ci[:, :, 0] = 0
    ci /= float(M) * M
    G = bp_adjoint_f64(ci, axes, p.V, p.mask_radius, p.ker, p.hw)
    b = p.V // 2 - M // 2
    F = np.fft.fftshift(np.fft.fftn(np.fft.fftshift(G[b:b + M, b:b + M, b:b + M])))
    R = to_cas(F) * _precomp3(M, p.hw)
    ob = M // 2 - N // 2
    return R[ob:ob + N, ob:ob + N, ob:ob + N]


# --------------------------------------------------------------------------
# Fixture generators
# --------------------------------------------------------------------------


def fuzzymask(n, dims, r0, risetime, origin=None):
    """src/Matlab/utils/fuzzymask.m (3-D and 2-D cases): 0.5*(1-erf(k(r-r0)))
    with k = 1.782/risetime; origin is 1-based, default floor(n/2)+1."""
    from scipy.special import erf
    if origin is None:
        origin = [n // 2 + 1] * dims
    origin = np.broadcast_to(np.asarray(origin, dtype=np.float64), (dims,))
    grids = [np.arange(1, n + 1) - origin[d] for d in range(dims)]
    # MATLAB ndgrid: first index is x (fastest in memory) -> numpy [k, j, i]
    mesh = np.meshgrid(*grids[::-1], indexing="ij")
    r = np.sqrt(sum(g ** 2 for g in mesh))
    if risetime == 0:
        return (r < r0).astype(np.float64)
    k = 1.782 / risetime
    return 0.5 * (1.0 - erf(k * (r - r0)))


def get_axes_from_n_rot(nvec, phi_r):
    """src/Matlab/utils/get_axes_from_n_rot.m:1-37 -> 9 floats [x; y; z] columns."""
    nvec = np.asarray(nvec, dtype=np.float64)
    a = np.cross([0.0, 0.0, 1.0], nvec)
    if np.sqrt(np.sum(a * a)) < 0.0001:
        T1 = np.eye(3)
        T2 = np.eye(3)
    else:
        phi = math.atan2(nvec[1], nvec[0])
        T1 = np.array([[math.cos(phi), -math.sin(phi), 0], [math.sin(phi), math.cos(phi), 0], [0, 0, 1]])
        theta = math.atan2(math.sqrt(nvec[0] ** 2 + nvec[1] ** 2), nvec[2])
        T2 = np.array([[math.cos(theta), 0, math.sin(theta)], [0, 1, 0], [-math.sin(theta), 0, math.cos(theta)]])
    T3 = np.array([[math.cos(phi_r), -math.sin(phi_r), 0], [math.sin(phi_r), math.cos(phi_r), 0], [0, 0, 1]])
    T = (T1 @ T2) @ T3
    return np.concatenate([T[:, 0], T[:, 1], T[:, 2]])


def create_uniform_axes(ntheta, nphi):
    """src/Matlab/utils/create_uniform_axes.m:16-28 -> [ntheta*nphi, 9]."""
    out = []
    alpha = math.pi / 180.0
    for theta in matlab_colon(90.0 / ntheta, 90.0 / ntheta, 90.0):
        for phi in matlab_colon(0.0, 360.0 / nphi, 360.0 - 0.1):
            z = [math.sin(theta * alpha) * math.cos(phi * alpha), math.sin(theta * alpha) * math.sin(phi * alpha),
                 math.cos(theta * alpha)]
            out.append(get_axes_from_n_rot(z, 30 * alpha))
    return np.array(out)


def grid_axes(n_az=100, n_pol=100, psi_deg=30.0):
    """Uniform axis grid: azimuth phi_a = 2*pi*a/n_az, cos-polar
    cos(theta_b) = -1 + (2b+1)/n_pol, in-plane rotation psi, built with the
    get_axes_from_n_rot convention.  Polar index outer."""
    out = []
    for b in range(n_pol):
        ct = -1.0 + (2 * b + 1) / n_pol
        st = math.sqrt(max(0.0, 1.0 - ct * ct))
        for a in range(n_az):
            ph = 2 * math.pi * a / n_az
            out.append(get_axes_from_n_rot([st * math.cos(ph), st * math.sin(ph), ct], math.radians(psi_deg)))
    return np.array(out)


def quaternion_axes(n, seed):
    """Directions from uniformly random unit quaternions (Shoemake): rotation
    matrix R, coordAxes = [R[:,0]; R[:,1]; R[:,2]]."""
    rng = np.random.default_rng(seed)
    u = rng.random((n, 3))
    q1 = np.sqrt(1 - u[:, 0]) * np.sin(2 * np.pi * u[:, 1])
    q2 = np.sqrt(1 - u[:, 0]) * np.cos(2 * np.pi * u[:, 1])
    q3 = np.sqrt(u[:, 0]) * np.sin(2 * np.pi * u[:, 2])
    q0 = np.sqrt(u[:, 0]) * np.cos(2 * np.pi * u[:, 2])
    w, x, y, z = q0, q1, q2, q3
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return np.concatenate([R[:, :, 0], R[:, :, 1], R[:, :, 2]], axis=1)


def blob_volume(N, n_blobs, seed, dtype=np.float32):
    """Seeded sum of isotropic Gaussian blobs: centres U[0.2N, 0.8N]^3, sigma
    U(2, 6) voxels, amplitude U(0.5, 1.5); evaluated in FP64, x fastest."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.2 * N, 0.8 * N, size=(n_blobs, 3))
    s = rng.uniform(2.0, 6.0, size=n_blobs)
    a = rng.uniform(0.5, 1.5, size=n_blobs)
    x = np.arange(N, dtype=np.float64)
    gx = np.exp(-(x[None, :] - c[:, 0:1]) ** 2 / (2 * s[:, None] ** 2))  # [b, i]
    gy = np.exp(-(x[None, :] - c[:, 1:2]) ** 2 / (2 * s[:, None] ** 2))  # [b, j]
    gz = np.exp(-(x[None, :] - c[:, 2:3]) ** 2 / (2 * s[:, None] ** 2)) * a[:, None]  # [b, k]
    vol = np.empty((N, N, N), dtype=np.float64)
    for k in range(N):
        vol[k] = (gy * gz[:, k:k + 1]).T @ gx
    return vol.astype(dtype)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return float(d / n) if n > 0 else float(d)
