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
