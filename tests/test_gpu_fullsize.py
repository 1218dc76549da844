"""Size-independent properties at the benchmark's full sizes, where the oracle
is too slow for whole workloads: linearity of forwardProject and the exact
adjoint identity at 128^3 (CAS images of 256^2 through the fused FFT
kernels), and forwardProject at 256^3 (CAS images of 512^2 through cuFFT)
against the oracle's FP32 restatement on a few directions.

Tolerances: FP32, relative 1e-5 (the parity bound); the adjoint identity in
FP64 dot products of the FP32 results, relative 1e-5."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def test_forward_projection_is_linear_at_128(cuda):
    import multigpugridder_gb300 as gg

    N = 128
    rng = np.random.default_rng(3)
    v1 = O.blob_volume(N, 100, seed=31)
    v2 = rng.standard_normal((N,) * 3).astype(np.float32)
    a, b = np.float32(0.75), np.float32(-1.25)
    axes = O.quaternion_axes(24, seed=32).astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(v1)
        p1 = g.forwardProject(axes).astype(np.float64)
        g.setVolume(v2)
        p2 = g.forwardProject(axes).astype(np.float64)
        g.setVolume(a * v1 + b * v2)
        p12 = g.forwardProject(axes).astype(np.float64)
    assert O.rel_l2(p12, float(a) * p1 + float(b) * p2) < TOL


def test_adjoint_identity_at_128(cuda):
    import torch

    from multigpugridder_gb300.autograd import ForwardProjector

    N = 128
    rng = np.random.default_rng(4)
    axes = torch.from_numpy(O.quaternion_axes(64, seed=33).astype(np.float32)).to(cuda)
    x = torch.from_numpy(rng.standard_normal((N,) * 3).astype(np.float32)).to(cuda)
    y = torch.from_numpy(rng.standard_normal((64, N, N)).astype(np.float32)).to(cuda)
    proj = ForwardProjector(N, 2.0)
    try:
        lhs = torch.sum(proj.project(x, axes).double() * y.double()).item()
        rhs = torch.sum(x.double() * proj.adjoint(y, axes).double()).item()
    finally:
        proj.close()
    assert abs(lhs - rhs) <= TOL * abs(lhs)


def test_forward_projection_at_256_matches_oracle(cuda):
    import multigpugridder_gb300 as gg

    N = 256
    p = O.Params(N)
    vol = O.blob_volume(N, 400, seed=3)
    axes = O.quaternion_axes(3, seed=34).astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        cas = g.forwardProjectCAS(axes)
    ref_cas = O.fp_ref_f32(O.cas_from_vol(vol).astype(np.float32), axes, p.M, p.mask_radius, p.ker)
    assert O.rel_l2(cas, ref_cas) < TOL
    ref = O.imgs_from_cas_imgs(ref_cas.astype(np.float64), N)
    assert O.rel_l2(imgs, ref) < TOL


def test_benchmark_workload_matches_oracle(cuda):
    """The benchmark's own configuration through the device-pointer calls it
    times: 128^3 (100 blobs, seed 2), interpFactor 2 (CAS images 256^2, CAS
    volume 262^3), the 100 x 100 azimuth x cos-polar direction grid,
    MaxAxesToAllocate 2000.  forwardProject of all 10,000 directions (five
    device batches) is checked on a fixed subset of 500 directions against
    the oracle's FP32 restatement; reconstructVol of those 500 images is
    checked against the oracle's FP32 reconstructVol (plane density and
    a / (b + 1e-6), MultiGPUGridder_Matlab_Class.m:284-312).  Relative L2
    <= 1e-5."""
    import ctypes

    import torch

    import multigpugridder_gb300 as gg
    from multigpugridder_gb300 import synthetic
    from multigpugridder_gb300._lib import check, lib

    N, n, S = 128, 10000, 500
    p = O.Params(N)
    vol = synthetic.blob_volume(N, 100, seed=2)
    axes = synthetic.grid_axes(100, 100).astype(np.float32)
    sub = np.linspace(0, n - 1, S).round().astype(int)
    L = lib()
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    g = gg.MultiGPUGridder(N, n, 2.0, MaxAxesToAllocate=2000)
    try:
        h = g.handle
        s = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
        d_vol = torch.from_numpy(vol).to(cuda)
        d_ax = torch.from_numpy(axes).to(cuda)
        d_img = torch.full((n, N, N), float("nan"), device=cuda)
        check(L.gg_set_volume_dev(h, vp(d_vol), s), h)
        check(L.gg_forward_project_dev(h, vp(d_ax), n, vp(d_img), None, s), h)
        d_sub_ax = d_ax[torch.from_numpy(sub).to(cuda)].contiguous()
        d_sub_img = d_img[torch.from_numpy(sub).to(cuda)].contiguous()
        d_rec = torch.full((N, N, N), float("nan"), device=cuda)
        check(L.gg_reconstruct_volume_dev(h, vp(d_sub_ax), S, vp(d_sub_img), vp(d_rec), s), h)
        torch.cuda.synchronize()
        imgs = d_sub_img.cpu().numpy()
        rec = d_rec.cpu().numpy()
    finally:
        g.close()
    assert np.all(np.isfinite(imgs)) and np.all(np.isfinite(rec))
    ref_imgs, _ = O.forward_project(vol, axes[sub], p, precision="f32")
    e_img = O.rel_l2(imgs, ref_imgs)
    ref_rec, _, _ = O.reconstruct_vol(imgs, axes[sub], p, precision="f32")
    e_rec = O.rel_l2(rec, ref_rec)
    print("benchmark workload, %d of %d directions: images rel-L2 %.2e, reconstructVol rel-L2 %.2e"
          % (S, n, e_img, e_rec))
    assert e_img < TOL
    assert e_rec < TOL
