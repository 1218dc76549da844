"""Timed CPU restatement of the whole reference path (TEST / BENCH INFRASTRUCTURE ONLY).

Used by bench.py as the CPU baseline and as its reference arm.  The reference
has no CPU implementation of the gridding kernels (its RunFFTOnGPU=false mode
still runs both kernels on the GPU, and src/Gridders/CPU is a different,
real-space projector), so the CPU path is the reference's own host math in
single precision -- CASFromVol_Gridder.m, volFromCAS_Gridder.m,
CASImgsFromImgs.m / imgsFromCASImgs.m, the plane-density division of
MultiGPUGridder_Matlab_Class.m:308 -- around the C restatement of its two CUDA
kernels (gg_oracle.c, OpenMP over all host threads).  FFTs use scipy.fft with
every worker thread.

One bench step of the GPU path processes D directions (forward projection,
back projection, plane-density back projection).  On the CPU one step runs
the same path on a bounded sample of S of those directions: the
direction-independent work (CAS volume preparation, getVol) and the
per-direction work of the S directions.  Its measured duration is
t_sample_step = t_fixed + t_sample(S); the D-direction step it stands for is
extrapolated as t_step(D) = t_fixed + (D / S) * t_sample(S) and reported
apart.
"""
import os
import time

import numpy as np
import scipy.fft as sfft

from . import oracle as O


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _pc3(M, hw):
    p = O.precomp(M, hw).astype(np.float32)
    return p[:, None, None] * p[None, :, None] * p[None, None, :]


def cas_from_vol_f32(vol, p, workers):
    """CASFromVol_Gridder.m in single precision."""
    N, M, V, pad = p.N, p.M, p.V, p.pad
    b = M // 2 - N // 2
    iv = np.zeros((M, M, M), np.float32)
    iv[b:b + N, b:b + N, b:b + N] = vol
    iv *= _pc3(M, p.hw)
    F = sfft.fftshift(sfft.fftn(sfft.fftshift(iv), workers=workers))
    out = np.zeros((V, V, V), np.float32)
    out[pad:pad + M, pad:pad + M, pad:pad + M] = (F.real + F.imag).astype(np.float32)
    return out


def vol_from_cas_f32(cas, p, workers):
    """volFromCAS_Gridder.m in single precision."""
    N, M, V = p.N, p.M, p.V
    b = V // 2 - M // 2
    ic = cas[b:b + M, b:b + M, b:b + M]
    r2 = ic[:0:-1, :0:-1, :0:-1]
    F = np.zeros((M, M, M), np.complex64)
    F[1:, 1:, 1:] = 0.5 * (ic[1:, 1:, 1:] + r2) + 0.5j * (ic[1:, 1:, 1:] - r2)
    iv = np.real(sfft.fftshift(sfft.ifftn(sfft.fftshift(F), workers=workers))).astype(np.float32)
    iv *= _pc3(M, p.hw)
    ob = M // 2 - N // 2
    return iv[ob:ob + N, ob:ob + N, ob:ob + N]


def imgs_from_cas_imgs_f32(r, N, workers):
    M = r.shape[-1]
    c = np.zeros(r.shape, np.complex64)
    a, f = r[:, 1:, 1:], r[:, :0:-1, :0:-1]
    c[:, 1:, 1:] = 0.5 * (a + f) + 0.5j * (a - f)
    y = np.real(sfft.fftshift(sfft.ifft2(sfft.fftshift(c, axes=(1, 2)), workers=workers), axes=(1, 2)))
    b = (M - N) // 2
    return np.ascontiguousarray(y[:, b:b + N, b:b + N], dtype=np.float32)


def cas_imgs_from_imgs_f32(x, M, workers):
    n, N = x.shape[0], x.shape[-1]
    b = (M - N) // 2
    pimg = np.zeros((n, M, M), np.float32)
    pimg[:, b:b + N, b:b + N] = x
    F = sfft.fftshift(sfft.fft2(sfft.fftshift(pimg, axes=(1, 2)), workers=workers), axes=(1, 2))
    return (F.real + F.imag).astype(np.float32)


def time_step(vol, axes_sample, p, n_directions, threads=None):
    """Time one step on the sample; returns (measured seconds, details with
    the extrapolated full-step time t_step_extrapolated_s)."""
    threads = threads or host_threads()
    O.set_threads(threads)
    t0 = time.perf_counter()
    cas = cas_from_vol_f32(vol, p, threads)
    t_prep = time.perf_counter() - t0

    t0 = time.perf_counter()
    ci = O.fp_ref_f32(cas, axes_sample, p.M, p.mask_radius, p.ker)
    t_fp = time.perf_counter() - t0
    t0 = time.perf_counter()
    imgs = imgs_from_cas_imgs_f32(ci, p.N, threads)
    t_ifft = time.perf_counter() - t0
    t0 = time.perf_counter()
    ci2 = cas_imgs_from_imgs_f32(imgs, p.M, threads)
    t_fft = time.perf_counter() - t0
    t0 = time.perf_counter()
    bp = O.bp_ref_f32(ci2, axes_sample, p.V, p.mask_radius, p.ker)
    t_bp = time.perf_counter() - t0
    t0 = time.perf_counter()
    pd = O.bp_ref_f32(np.ones_like(ci2), axes_sample, p.V, p.mask_radius, p.ker)
    t_pd = time.perf_counter() - t0
    t0 = time.perf_counter()
    rec = vol_from_cas_f32(bp / (pd + np.float32(1e-6)), p, threads)
    t_get = time.perf_counter() - t0

    S = len(axes_sample)
    per_dir = (t_fp + t_ifft + t_fft + t_bp + t_pd) / S
    t_fixed = t_prep + t_get
    t_measured = t_fixed + per_dir * S
    details = {"threads": threads, "sample_directions": S, "t_fixed_s": t_fixed, "t_per_direction_s": per_dir,
               "t_fp_s": t_fp, "t_bp_s": t_bp, "t_density_s": t_pd, "t_fft2_s": t_ifft + t_fft,
               "t_step_extrapolated_s": t_fixed + n_directions * per_dir, "finite": bool(np.isfinite(rec).all())}
    return t_measured, details
