"""GPU: the CTF applied to the images before the back projection (the
reference's ApplyCTFs flag, src/Gridders/AbstractGridder.h:118-119, which it
declares and never implements).

Tolerances: the CTF within 1e-6 absolute of the FP64 formula (chi is formed
in float-float arithmetic and reduced mod 2 pi before sincosf); the
CTF-corrected reconstruction within relative L2 1e-5 of the oracle (the FP32
back-projection restatement fed the FP64 CTF rounded to FP32), the bound of
the FP32 parity tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5
# the parameters cross the C ABI as FP32: the FP64 formula is evaluated at
# the FP32 values (2.7 -> 2.70000005 alone moves chi by 1.4e-6 rad at 80 rad)
KV, CS, AMP = (float(np.float32(v)) for v in (300.0, 2.7, 0.1))


def dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def to_dev(a, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


@pytest.mark.parametrize("M,px", [(64, 1.5), (256, 1.0)])
def test_ctf_filter_matches_formula(cuda, gglib, M, px):
    import torch

    df = np.array([0.0, 8000.0, 15000.0, 30000.0, 60000.0, -12000.0], np.float32)
    n = len(df)
    d_df = to_dev(df, cuda)
    ref = O.ctf_cas(M, df, KV, CS, AMP, px)
    for power in (1, 2):
        out = torch.full((n, M, M), float("nan"), device=cuda)
        assert gglib.gg_filter_apply_ctf(dptr(out), M, n, dptr(d_df), None, None, KV, CS, AMP, px, power, 1, None) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(got - ref ** power)) < 1e-6
    # multiply mode: the same CTF values times the images
    img = np.random.default_rng(M).standard_normal((n, M, M)).astype(np.float32)
    d_img = to_dev(img, cuda)
    gen = torch.empty_like(d_img)
    assert gglib.gg_filter_apply_ctf(dptr(d_img), M, n, dptr(d_df), None, None, KV, CS, AMP, px, 1, 0, None) == 0
    assert gglib.gg_filter_apply_ctf(dptr(gen), M, n, dptr(d_df), None, None, KV, CS, AMP, px, 1, 1, None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_img.cpu().numpy(), img * gen.cpu().numpy())


def test_ctf_filter_rejects_bad_parameters(cuda, gglib):
    import torch

    from multigpugridder_gb300._lib import GG_ERR_INVALID_ARG

    x = torch.zeros((1, 8, 8), device=cuda)
    d = torch.zeros(1, device=cuda)
    assert gglib.gg_filter_apply_ctf(dptr(x), 8, 1, dptr(d), None, None, 0.0, CS, AMP, 1.0, 1, 0, None) == GG_ERR_INVALID_ARG
    assert gglib.gg_filter_apply_ctf(dptr(x), 8, 1, dptr(d), None, None, KV, CS, 1.5, 1.0, 1, 0, None) == GG_ERR_INVALID_ARG
    assert gglib.gg_filter_apply_ctf(dptr(x), 8, 1, dptr(d), None, None, KV, CS, AMP, 0.0, 1, 0, None) == GG_ERR_INVALID_ARG
    assert gglib.gg_filter_apply_ctf(dptr(x), 8, 1, dptr(d), None, None, KV, CS, AMP, 1.0, 3, 0, None) == GG_ERR_INVALID_ARG
    assert gglib.gg_filter_apply_ctf(dptr(x), 8, 0, None, None, None, KV, CS, AMP, 1.0, 1, 0, None) == 0


def _data(N, n, seed):
    vol = O.blob_volume(N, 10, seed=seed)
    axes = np.concatenate([O.quaternion_axes(n, seed + 1), O.create_uniform_axes(2, 4)]).astype(np.float32)
    return vol, axes


def test_ctf_reconstruction_without_aberration_is_minus_plain(cuda):
    """defocus 0, Cs 0, A = 1: CTF = -1 at every pixel and CTF^2 = 1, so the
    one-pass back projection of (CTF . image, CTF^2) must give minus the
    plain reconstruction bit for bit (negation is exact and 1 * w + s rounds
    as w + s)."""
    import multigpugridder_gb300 as gg

    N = 32
    vol, axes = _data(N, 30, 40)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        plain = g.reconstructVol(imgs, axes)
        ctf = g.reconstructVolCTF(imgs, axes, np.zeros(len(axes)), KV, 0.0, 1.0, 1.0)
    assert np.array_equal(ctf, -plain)


@pytest.mark.parametrize("N", [16, 32])
def test_ctf_reconstruction_matches_oracle(cuda, N):
    import multigpugridder_gb300 as gg

    p = O.Params(N)
    vol, axes = _data(N, 30, 50 + N)
    df = np.random.default_rng(N).uniform(5000.0, 25000.0, len(axes)).astype(np.float32)
    px = 2.0
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        rec = g.reconstructVolCTF(imgs, axes, df, KV, CS, AMP, px)
    ref = O.reconstruct_vol_ctf(imgs, axes, p, df, KV, CS, AMP, px, precision="f32")[0]
    assert np.all(np.isfinite(rec))
    assert O.rel_l2(rec, ref) < TOL


@pytest.mark.parametrize("prec", ["bf16", "f16"])
def test_ctf_reconstruction_reduced_precision(cuda, prec):
    """FP16 / BF16 storage: the two stacks take separate back projections;
    the result stays within 1e-3 relative L2 of the FP64 oracle."""
    import multigpugridder_gb300 as gg

    N = 32
    p = O.Params(N)
    vol, axes = _data(N, 30, 70)
    df = np.random.default_rng(7).uniform(5000.0, 25000.0, len(axes)).astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        g.set_precision(prec)
        rec = g.reconstructVolCTF(imgs, axes, df, KV, CS, AMP, 2.0)
    ref = O.reconstruct_vol_ctf(imgs, axes, p, df, KV, CS, AMP, 2.0)[0]
    assert O.rel_l2(rec, ref) < 1e-3


def test_ctf_reconstruction_device_form_equals_host_form(cuda):
    import torch

    import multigpugridder_gb300 as gg
    from multigpugridder_gb300._lib import check, lib

    N = 32
    vol, axes = _data(N, 40, 60)
    df = np.linspace(6000.0, 22000.0, len(axes)).astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        host = g.reconstructVolCTF(imgs, axes, df, KV, CS, AMP, 1.2)
        out = torch.empty((N, N, N), device=cuda)
        d_ax, d_im, d_df = to_dev(axes, cuda), to_dev(imgs, cuda), to_dev(df, cuda)
        s = torch.cuda.current_stream(cuda)
        check(lib().gg_reconstruct_volume_ctf_dev(g.handle, dptr(d_ax), len(axes), dptr(d_im), dptr(d_df), None,
                                                  None, KV, CS, AMP, 1.2, dptr(out), ctypes.c_void_p(s.cuda_stream)),
              g.handle)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), host)
        with pytest.raises(ValueError):
            g.reconstructVolCTF(imgs, axes, df[:-1])


@pytest.mark.parametrize("M,px", [(64, 1.5), (256, 1.0)])
def test_astigmatic_ctf_filter_matches_formula(cuda, gglib, M, px):
    import torch

    rng = np.random.default_rng(M + 1)
    n = 6
    du = rng.uniform(5000.0, 40000.0, n).astype(np.float32)
    dv = (du - rng.uniform(-3000.0, 3000.0, n)).astype(np.float32)
    ang = rng.uniform(-np.pi, np.pi, n).astype(np.float32)
    ref = O.ctf_cas(M, du, KV, CS, AMP, px, dv, ang)
    out = torch.full((n, M, M), float("nan"), device=cuda)
    d_u, d_v, d_a = to_dev(du, cuda), to_dev(dv, cuda), to_dev(ang, cuda)
    assert gglib.gg_filter_apply_ctf(dptr(out), M, n, dptr(d_u), dptr(d_v), dptr(d_a), KV, CS, AMP, px, 1, 1,
                                     None) == 0
    torch.cuda.synchronize()
    assert np.max(np.abs(out.cpu().numpy().astype(np.float64) - ref)) < 1e-6
    # V without an angle is refused
    from multigpugridder_gb300._lib import GG_ERR_INVALID_ARG
    assert gglib.gg_filter_apply_ctf(dptr(out), M, n, dptr(d_u), dptr(d_v), None, KV, CS, AMP, px, 1, 1,
                                     None) == GG_ERR_INVALID_ARG


def test_astigmatic_ctf_reconstruction_matches_oracle(cuda):
    import multigpugridder_gb300 as gg

    N = 32
    p = O.Params(N)
    vol, axes = _data(N, 30, 90)
    rng = np.random.default_rng(91)
    du = rng.uniform(6000.0, 25000.0, len(axes)).astype(np.float32)
    dv = (du - rng.uniform(-2000.0, 2000.0, len(axes))).astype(np.float32)
    ang = rng.uniform(0.0, np.pi, len(axes)).astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        rec = g.reconstructVolCTF(imgs, axes, du, KV, CS, AMP, 2.0, defocus_v=dv, astig_angle=ang)
        with pytest.raises(ValueError):
            g.reconstructVolCTF(imgs, axes, du, defocus_v=dv)
    ref = O.reconstruct_vol_ctf(imgs, axes, p, du, KV, CS, AMP, 2.0, precision="f32", defocus_v=dv,
                                astig_angle=ang)[0]
    assert O.rel_l2(rec, ref) < TOL

