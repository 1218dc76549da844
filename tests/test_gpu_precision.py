"""Reduced-precision storage (FP16 / BF16 CAS volume and CAS images, FP32
window accumulation) against the FP64 oracle.

Bound: relative L2 <= 1e-3 against FP64 for every stored form; the FP32 path
is also checked against FP64 (it differs only by FP32 rounding, which can move
a nearest-index table lookup: ~1e-5 forward, ~1e-4 back)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_REDUCED = 1e-3


@pytest.fixture(scope="module")
def case():
    N = 64
    p = O.Params(N)
    vol = O.blob_volume(N, 20, seed=31)
    axes = O.quaternion_axes(24, seed=32).astype(np.float32)
    imgs64, cas64 = O.forward_project(vol.astype(np.float64), axes, p, "f64")
    return N, p, vol, axes, imgs64, cas64


@pytest.mark.parametrize("prec", ["f32", "bf16", "f16"])
def test_forward_projection_precision(cuda, case, prec):
    import multigpugridder_gb300 as gg

    N, p, vol, axes, imgs64, cas64 = case
    with gg.MultiGPUGridder(N, len(axes), precision=prec, adjustInterpFactor=False) as g:
        g.setVolume(vol)
        cas = g.forwardProjectCAS(axes)
        imgs = g.forwardProject(axes)
    e_cas, e_img = O.rel_l2(cas, cas64), O.rel_l2(imgs, imgs64)
    print("%s: CAS images rel-L2 %.2e, images rel-L2 %.2e vs FP64" % (prec, e_cas, e_img))
    bound = 1e-4 if prec == "f32" else TOL_REDUCED
    assert e_cas < bound and e_img < bound


@pytest.mark.parametrize("prec", ["f32", "bf16", "f16"])
def test_back_projection_precision(cuda, case, prec):
    import multigpugridder_gb300 as gg

    N, p, vol, axes, imgs64, cas64 = case
    ref = O.back_project(imgs64, axes, p, "f64")
    with gg.MultiGPUGridder(N, len(axes), precision=prec, adjustInterpFactor=False) as g:
        g.backProject(imgs64.astype(np.float32), axes)
        got = g.getCASVolume()
    e = O.rel_l2(got, ref)
    print("%s: back projection rel-L2 %.2e vs FP64" % (prec, e))
    assert e < (1e-3 if prec == "f32" else TOL_REDUCED)


@pytest.mark.parametrize("prec", ["bf16", "f16"])
def test_reconstruct_precision(cuda, case, prec):
    import multigpugridder_gb300 as gg

    N, p, vol, axes, imgs64, cas64 = case
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        ref = g.reconstructVol(imgs64.astype(np.float32), axes)
    with gg.MultiGPUGridder(N, len(axes), precision=prec, adjustInterpFactor=False) as g:
        got = g.reconstructVol(imgs64.astype(np.float32), axes)
    e = O.rel_l2(got, ref)
    print("%s: reconstruction rel-L2 %.2e vs FP32 path" % (prec, e))
    assert e < TOL_REDUCED


def test_f16_scaling_handles_large_values(cuda, case):
    """CAS values far above the FP16 range (65504) are scaled by a power of
    two on the device, so nothing overflows."""
    import multigpugridder_gb300 as gg

    N, p, vol, axes, imgs64, cas64 = case
    big = vol * np.float32(1e6)
    with gg.MultiGPUGridder(N, len(axes), precision="f16", adjustInterpFactor=False) as g:
        g.setVolume(big)
        imgs = g.forwardProject(axes)
        g.backProject(imgs, axes)
        cas = g.getCASVolume()
    assert np.all(np.isfinite(imgs)) and np.all(np.isfinite(cas))
    assert O.rel_l2(imgs, imgs64 * 1e6) < TOL_REDUCED


def test_image_precision_knob(cuda, case):
    """BF16 volume with FP32 CAS images for the back projection
    (gg_set_image_precision): the back projection equals the FP32 mode's bit
    for bit (it does not read the volume), the forward projection equals the
    BF16 mode's, and None restores the volume's precision for the images."""
    import multigpugridder_gb300 as gg

    N, p, vol, axes, imgs64, cas64 = case
    imgs = imgs64.astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), precision="f32", adjustInterpFactor=False) as g:
        g.backProject(imgs, axes)
        bp32 = g.getCASVolume()
    with gg.MultiGPUGridder(N, len(axes), precision="bf16", adjustInterpFactor=False) as g:
        g.setVolume(vol)
        fp16b = g.forwardProject(axes)
        g.backProject(imgs, axes)
        bp16b = g.getCASVolume()
    with gg.MultiGPUGridder(N, len(axes), precision="bf16", adjustInterpFactor=False) as g:
        g.set_image_precision("f32")
        g.setVolume(vol)
        assert np.array_equal(g.forwardProject(axes), fp16b)
        g.backProject(imgs, axes)
        assert np.array_equal(g.getCASVolume(), bp32)
        g.set_image_precision(None)
        g.backProject(imgs, axes)
        assert np.array_equal(g.getCASVolume(), bp16b)
