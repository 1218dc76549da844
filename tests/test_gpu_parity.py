"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerance: relative L2 <= 1e-5 for the FP32 path (the bound the reference
parity is stated in; back-projection summation order differs, so exactness is
by tolerance).  Pixels outside the mask must be exactly zero.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def to_dev(a, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def test_axes(n, seed):
    """Random quaternion directions plus the reference's own axis grid, whose
    30 degree in-plane rotation puts exact 0.5 entries in the axes (table
    index ties)."""
    return np.concatenate([O.quaternion_axes(n, seed), O.create_uniform_axes(2, 4)]).astype(np.float32)


test_axes.__test__ = False


@pytest.mark.parametrize("N", [16, 32, 64])
def test_forward_kernel_matches_oracle(cuda, gglib, N):
    import torch

    p = O.Params(N)
    rng = np.random.default_rng(100 + N)
    cas = rng.standard_normal((p.V,) * 3).astype(np.float32)
    axes = test_axes(12, seed=N)
    ref = O.fp_ref_f32(cas, axes, p.M, p.mask_radius, p.ker)
    out = torch.full((len(axes), p.M, p.M), float("nan"), device=cuda)
    d_cas, d_ker, d_axes = to_dev(cas, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda)
    rc = gglib.gg_forward_project_kernel(dptr(d_cas), dptr(out), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V, p.M,
                                         3, p.mask_radius, p.ker.size, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert O.rel_l2(got, ref) < TOL
    assert np.all(got[ref == 0] == 0)  # outside the mask


@pytest.mark.parametrize("N", [2, 4, 6, 21, 50, 100])
def test_forward_kernel_other_sizes(cuda, gglib, N):
    """The forward projection at tiny volume edges (tap windows that leave the
    CAS volume: the reference's linear-index rule), at an odd edge (M = 42) and
    at edges whose CAS images are not a multiple of the 16-pixel tile: within
    the FP32 parity bound, and exactly zero outside the mask."""
    import torch

    p = O.Params(N)
    rng = np.random.default_rng(400 + N)
    cas = rng.standard_normal((p.V,) * 3).astype(np.float32)
    axes = test_axes(6, seed=N + 7)
    ref = O.fp_ref_f32(cas, axes, p.M, p.mask_radius, p.ker)
    out = torch.full((len(axes), p.M, p.M), float("nan"), device=cuda)
    d_cas, d_ker, d_axes = to_dev(cas, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda)
    rc = gglib.gg_forward_project_kernel(dptr(d_cas), dptr(out), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V, p.M,
                                         3, p.mask_radius, p.ker.size, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert O.rel_l2(got, ref) < TOL
    assert np.all(got[ref == 0] == 0)


@pytest.mark.parametrize("N", [16, 32, 64])
def test_back_kernel_matches_oracle(cuda, gglib, N):
    import torch

    p = O.Params(N)
    rng = np.random.default_rng(200 + N)
    # full-frame random CAS images: border pixels exercise the reference's
    # row-wrap of windows that cross an image edge (gpuBackProject.cu:99)
    img = rng.standard_normal((14, p.M, p.M)).astype(np.float32)
    axes = test_axes(6, seed=N + 1)[:14]
    ref = O.bp_ref_f32(img, axes, p.V, p.mask_radius, p.ker)
    vol = torch.zeros((p.V,) * 3, device=cuda)
    d_img, d_ker, d_axes = to_dev(img, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda)
    rc = gglib.gg_back_project_kernel(dptr(vol), dptr(d_img), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V, p.M,
                                      p.mask_radius, p.ker.size, 3, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = vol.cpu().numpy()
    assert O.rel_l2(got, ref) < TOL
    assert np.all(got[ref == 0] == 0)


def _table(kind):
    """KB tables of other lengths (getKernelFiltTable's size argument), and a
    raw window whose edge entries are not zero."""
    if kind == "raw":
        x = np.linspace(-2.0, 2.0, 501)
        return (O.grid_lib_kaiser(2, O.kernel_alpha(2), x) + 0.05).astype(np.float32)
    return O.kb_table(2, int(kind)).astype(np.float32)


@pytest.mark.parametrize("kind", ["1000", "513", "101", "raw"])
def test_back_kernel_other_tables_bit_exact(cuda, gglib, kind):
    """The back projection's saturating table index and its interleaved table
    copies (P = 512 or 1024 entries, 32 or 16 copies) for tables of other
    lengths, and the clamp to the edge entries for a table whose edges are not
    zero: equal to the oracle's FP32 restatement bit for bit."""
    import torch

    N = 32
    p = O.Params(N)
    ker = _table(kind)
    rng = np.random.default_rng(11)
    axes = test_axes(6, seed=3)[:10]
    img = rng.standard_normal((len(axes), p.M, p.M)).astype(np.float32)
    ref = O.bp_ref_f32(img, axes, p.V, p.mask_radius, ker)
    vol = torch.zeros((p.V,) * 3, device=cuda)
    d_img, d_ker, d_axes = to_dev(img, cuda), to_dev(ker, cuda), to_dev(axes, cuda)
    rc = gglib.gg_back_project_kernel(dptr(vol), dptr(d_img), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V, p.M,
                                      p.mask_radius, ker.size, 3, None)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(vol.cpu().numpy(), ref)


@pytest.mark.parametrize("N", [2, 4, 6, 21, 50, 100])
def test_back_kernel_other_sizes_bit_exact(cuda, gglib, N):
    """Tiny volumes (CAS images of 4-12 pixels, narrower than a footprint,
    bricks that overhang the whole volume), volume edges whose CAS images are
    not a multiple of 4 wide (M = 42: footprints staged pixel by pixel), and
    brick grids that do not divide the CAS volume (V = 48, 106, 206): equal to
    the oracle bit for bit."""
    import torch

    p = O.Params(N)
    rng = np.random.default_rng(300 + N)
    axes = test_axes(5, seed=N)[:8]
    img = rng.standard_normal((len(axes), p.M, p.M)).astype(np.float32)
    ref = O.bp_ref_f32(img, axes, p.V, p.mask_radius, p.ker)
    vol = torch.zeros((p.V,) * 3, device=cuda)
    d_img, d_ker, d_axes = to_dev(img, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda)
    rc = gglib.gg_back_project_kernel(dptr(vol), dptr(d_img), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V, p.M,
                                      p.mask_radius, p.ker.size, 3, None)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(vol.cpu().numpy(), ref)


def test_back_kernel_deep_blocks_bit_exact(cuda, gglib):
    """CAS images of 512^2 (N = 256) take the 8-voxel-deep warp blocks: the
    back projection equals the oracle's FP32 restatement bit for bit."""
    import torch

    N = 256
    p = O.Params(N)
    rng = np.random.default_rng(7)
    axes = test_axes(3, seed=5)[:4]
    img = rng.standard_normal((len(axes), p.M, p.M)).astype(np.float32)
    ref = O.bp_ref_f32(img, axes, p.V, p.mask_radius, p.ker)
    vol = torch.zeros((p.V,) * 3, device=cuda)
    d_img, d_ker, d_axes = to_dev(img, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda)
    rc = gglib.gg_back_project_kernel(dptr(vol), dptr(d_img), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V, p.M,
                                      p.mask_radius, p.ker.size, 3, None)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(vol.cpu().numpy(), ref)


def test_reconstruct_deep_blocks(cuda):
    """reconstructVol at N = 256 (the fused back projection + plane density
    with 8-deep blocks): the resident divided CAS volume against the oracle's
    BP(images) / (BP(ones) + 1e-6)."""
    import multigpugridder_gb300 as gg

    N = 256
    p = O.Params(N)
    rng = np.random.default_rng(8)
    axes = test_axes(3, seed=6)[:4]
    imgs = rng.standard_normal((len(axes), N, N)).astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.reconstructVol(imgs, axes)
        got = g.getCASVolume()
    ci = O.cas_imgs_from_imgs(imgs, p.M).astype(np.float32)
    num = O.bp_ref_f32(ci, axes, p.V, p.mask_radius, p.ker)
    den = O.bp_ref_f32(np.ones_like(ci), axes, p.V, p.mask_radius, p.ker)
    ref = num / (den + np.float32(1e-6))
    assert O.rel_l2(got, ref) < TOL


@pytest.mark.parametrize("N", [16, 32])
def test_adjoint_kernel_is_exact_adjoint(cuda, gglib, N):
    import torch

    p = O.Params(N)
    rng = np.random.default_rng(300 + N)
    x = rng.standard_normal((p.V,) * 3).astype(np.float32)
    axes = test_axes(8, seed=N + 2)
    n = len(axes)
    y = rng.standard_normal((n, p.M, p.M)).astype(np.float32)
    d_ker, d_axes, d_x, d_y = to_dev(p.ker, cuda), to_dev(axes, cuda), to_dev(x, cuda), to_dev(y, cuda)
    px = torch.zeros((n, p.M, p.M), device=cuda)
    assert gglib.gg_forward_project_kernel(dptr(d_x), dptr(px), dptr(d_ker), dptr(d_axes), 2.0, n, p.V,
                                           p.M, 3, p.mask_radius, p.ker.size, None) == 0
    bty = torch.zeros((p.V,) * 3, device=cuda)
    assert gglib.gg_back_project_adjoint_kernel(dptr(bty), dptr(d_y), dptr(d_ker), dptr(d_axes), 2.0, n,
                                                p.V, p.M, p.mask_radius, p.ker.size, None) == 0
    torch.cuda.synchronize()
    px, bty = px.cpu().numpy().astype(np.float64), bty.cpu().numpy().astype(np.float64)
    lhs = float(np.sum(px * y))
    rhs = float(np.sum(x * bty))
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), np.linalg.norm(px) * np.linalg.norm(y) * 1e-3)
    # against the FP64 adjoint: the same pairs and weights up to FP32
    # rounding, which can move a nearest-index table lookup (~1e-4)
    ref = O.bp_adjoint_f64(y.astype(np.float64), axes, p.V, p.mask_radius, p.ker)
    assert O.rel_l2(bty, ref) < 1e-3


def test_reference_rule_is_not_adjoint(cuda, gglib):
    """The reference's BP window differs from the forward window at general
    orientations: the two modes must give different volumes."""
    import torch

    p = O.Params(16)
    rng = np.random.default_rng(7)
    axes = O.quaternion_axes(6, seed=8).astype(np.float32)
    y = rng.standard_normal((6, p.M, p.M)).astype(np.float32)
    d = [torch.zeros((p.V,) * 3, device=cuda) for _ in range(2)]
    keep = (to_dev(y, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda))
    args = (dptr(keep[0]), dptr(keep[1]), dptr(keep[2]), 2.0, 6, p.V, p.M, p.mask_radius, p.ker.size)
    assert gglib.gg_back_project_kernel(dptr(d[0]), *args, 3, None) == 0
    assert gglib.gg_back_project_adjoint_kernel(dptr(d[1]), *args, None) == 0
    torch.cuda.synchronize()
    assert O.rel_l2(d[0].cpu().numpy(), d[1].cpu().numpy()) > 1e-3


# ---------------------------------------------------------------------------
# Whole-path calls through the gridder object
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("N", [16, 32])
def test_set_volume_cas_prep(cuda, N):
    import multigpugridder_gb300 as gg

    vol = O.blob_volume(N, 8, seed=N)
    with gg.MultiGPUGridder(N, 4, adjustInterpFactor=False) as g:
        g.setVolume(vol)
        cas = g.getCASVolume()
    ref = O.cas_from_vol(vol.astype(np.float64))
    assert O.rel_l2(cas, ref) < TOL
    p = O.Params(N)
    border = np.ones((p.V,) * 3, bool)
    border[3:-3, 3:-3, 3:-3] = False
    assert np.all(cas[border] == 0)


@pytest.mark.parametrize("N", [16, 32])
def test_get_volume_inverts_cas_prep(cuda, N):
    import multigpugridder_gb300 as gg

    vol = O.blob_volume(N, 8, seed=N + 5)
    rng = np.random.default_rng(N)
    p = O.Params(N)
    cas = rng.standard_normal((p.V,) * 3).astype(np.float32)
    with gg.MultiGPUGridder(N, 4, adjustInterpFactor=False) as g:
        g.setCASVolume(cas)
        got = g.getVol()
        g.setVolume(vol)
        rt = g.getVol()
    assert O.rel_l2(got, O.vol_from_cas(cas, N)) < TOL
    assert O.rel_l2(rt, O.vol_from_cas(O.cas_from_vol(vol), N)) < TOL


@pytest.mark.parametrize("N,batch", [(32, 1000), (32, 7)])
def test_forward_project_images(cuda, N, batch):
    import multigpugridder_gb300 as gg

    p = O.Params(N)
    vol = O.blob_volume(N, 10, seed=N + 3)
    axes = test_axes(17, seed=N + 4)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False, MaxAxesToAllocate=batch) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        cas = g.forwardProjectCAS(axes)
    ref_cas = O.fp_ref_f32(O.cas_from_vol(vol).astype(np.float32), axes, p.M, p.mask_radius, p.ker)
    assert O.rel_l2(cas, ref_cas) < TOL
    ref = O.imgs_from_cas_imgs(ref_cas.astype(np.float64), N)
    assert O.rel_l2(imgs, ref) < TOL


@pytest.mark.parametrize("pinned", [False, True])
def test_back_project_images(cuda, pinned):
    import torch

    import multigpugridder_gb300 as gg

    N = 32
    p = O.Params(N)
    rng = np.random.default_rng(5)
    axes = test_axes(20, seed=9)
    imgs = rng.standard_normal((len(axes), N, N)).astype(np.float32)
    if pinned:
        t = torch.from_numpy(imgs).pin_memory()
        imgs_in = t.numpy()
    else:
        imgs_in = imgs
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False, MaxAxesToAllocate=9) as g:
        g.backProject(imgs_in, axes)
        got = g.getCASVolume()
    ref = O.bp_ref_f32(O.cas_imgs_from_imgs(imgs, p.M).astype(np.float32), axes, p.V, p.mask_radius, p.ker)
    assert O.rel_l2(got, ref) < TOL


def test_forward_project_pinned_outputs(cuda):
    import torch

    import multigpugridder_gb300 as gg
    from multigpugridder_gb300._lib import lib

    N = 16
    vol = O.blob_volume(N, 5, seed=1)
    axes = test_axes(9, seed=2)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False, MaxAxesToAllocate=4) as g:
        g.setVolume(vol)
        ref = g.forwardProject(axes)
        out = torch.empty((len(axes), N, N), dtype=torch.float32).pin_memory()
        cas = torch.empty((len(axes), g.M, g.M), dtype=torch.float32).pin_memory()
        a = np.ascontiguousarray(axes, dtype=np.float32)
        rc = lib().gg_forward_project(g.handle, ctypes.c_void_p(a.ctypes.data), len(axes),
                                      ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(cas.data_ptr()))
        assert rc == 0
        assert np.array_equal(out.numpy(), ref)
        assert np.array_equal(cas.numpy(), g.forwardProjectCAS(axes))


@pytest.mark.parametrize("N", [32, 50])
def test_reconstruct_volume(cuda, N):
    import multigpugridder_gb300 as gg

    p = O.Params(N)
    vol = O.blob_volume(N, 10, seed=21)
    axes = test_axes(30, seed=22)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        rec = g.reconstructVol(imgs, axes)
    ref, _, _ = O.reconstruct_vol(imgs, axes, p, precision="f32")
    assert O.rel_l2(rec, ref) < TOL


def test_cpu_runnable_workload(cuda):
    """The reference's CPU-runnable configuration at full size: 64^3, 20
    Gaussian blobs (seed 1), 1,000 random-quaternion directions (seed 1),
    interpFactor 2 (CAS images 128^2, CAS volume 134^3): forwardProject and
    reconstructVol against the oracle's FP32 restatement."""
    import multigpugridder_gb300 as gg

    N = 64
    p = O.Params(N)
    vol = O.blob_volume(N, 20, seed=1)
    axes = O.quaternion_axes(1000, seed=1).astype(np.float32)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        rec = g.reconstructVol(imgs, axes)
    ref_imgs, _ = O.forward_project(vol, axes, p, precision="f32")
    assert O.rel_l2(imgs, ref_imgs) < TOL
    ref_rec, _, _ = O.reconstruct_vol(imgs, axes, p, precision="f32")
    assert O.rel_l2(rec, ref_rec) < TOL


def test_fp_sphere_known_answer(cuda):
    """ForwardProjectTests.m:28-69: a fuzzy sphere projects to sum(V, 3) in
    every direction; max |mean(image - GT)| <= 1."""
    import multigpugridder_gb300 as gg

    N = 64
    vol = O.fuzzymask(N, 3, N * 0.25, 2, (N // 2 + 1) * np.ones(3)).astype(np.float32)
    axes = O.create_uniform_axes(10, 50)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
    gt = vol.astype(np.float64).sum(axis=0)
    md = (imgs - gt[None]).reshape(len(axes), -1).mean(axis=1)
    assert np.max(np.abs(md)) <= 1.0
    assert np.max(np.abs(imgs - gt[None])) < 0.1


def test_reconstruction_known_answer(cuda):
    """BackProjectTests.m:25-66: 128^3 fuzzy sphere, 100x50 directions,
    forward project -> reconstructVol; max |recon - V| <= 1."""
    import multigpugridder_gb300 as gg

    N = 128
    vol = O.fuzzymask(N, 3, N * 0.25, 2, (N // 2 + 1) * np.ones(3)).astype(np.float32)
    axes = O.create_uniform_axes(100, 50)
    with gg.MultiGPUGridder(N, len(axes), adjustInterpFactor=False) as g:
        g.setVolume(vol)
        imgs = g.forwardProject(axes)
        g.resetVolume()
        rec = g.reconstructVol(imgs, axes)
    assert np.max(np.abs(rec - vol)) <= 1.0


def test_zero_axes_and_errors(cuda):
    import multigpugridder_gb300 as gg
    from multigpugridder_gb300._lib import GG_ERR_INVALID_ARG, GG_ERR_STATE, GridderError, lib

    N = 16
    with gg.MultiGPUGridder(N, 4, adjustInterpFactor=False) as g:
        # forward projection before any volume: state error, not a crash
        with pytest.raises(GridderError) as e:
            g._call("gg_forward_project", ctypes.c_void_p(np.zeros(9, np.float32).ctypes.data), 1,
                    ctypes.c_void_p(np.zeros(N * N, np.float32).ctypes.data), None)
        assert e.value.code == GG_ERR_STATE
        g.setVolume(O.blob_volume(N, 3, seed=1))
        out = g.forwardProject(np.zeros((0, 9), np.float32))
        assert out.shape == (0, N, N)
        bad = np.zeros((N + 2,) * 3, np.float32)
        dims = (ctypes.c_int * 3)(N + 2, N + 2, N + 2)
        assert lib().gg_set_volume(g.handle, ctypes.c_void_p(bad.ctypes.data), dims) == GG_ERR_INVALID_ARG
        assert b"must be" in lib().gg_last_error(g.handle)
        with pytest.raises(GridderError):
            g.set_precision(7)
    h = ctypes.c_void_p()
    assert lib().gg_create(15, 1, ctypes.c_float(2.0), 3, 1, None, 1, 0, ctypes.byref(h)) == GG_ERR_INVALID_ARG


# ---------------------------------------------------------------------------
# The reference's own kernels (compiled from its sources into oracle/_ref)
# ---------------------------------------------------------------------------


def _ref():
    from oracle import ref_kernels

    if not ref_kernels.available():
        pytest.skip("reference cubins not present")
    return ref_kernels.RefKernels()


@pytest.mark.parametrize("N", [32, 64])
def test_forward_matches_reference_kernel(cuda, gglib, N):
    import torch

    rk = _ref()
    p = O.Params(N)
    vol = O.blob_volume(N, 12, seed=N + 40)
    cas = O.cas_from_vol(vol).astype(np.float32)
    axes = test_axes(24, seed=N + 41)
    d_cas, d_ker, d_axes = to_dev(cas, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda)
    ref = torch.zeros((len(axes), p.M, p.M), device=cuda)
    rk.forward_project(d_cas.data_ptr(), p.V, ref.data_ptr(), p.M, d_axes.data_ptr(), len(axes), p.mask_radius,
                       d_ker.data_ptr(), p.ker.size)
    got = torch.full_like(ref, float("nan"))
    assert gglib.gg_forward_project_kernel(dptr(d_cas), dptr(got), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V,
                                           p.M, 3, p.mask_radius, p.ker.size, None) == 0
    torch.cuda.synchronize()
    ref, got = ref.cpu().numpy(), got.cpu().numpy()
    assert O.rel_l2(got, ref) < TOL
    # and the oracle restatement agrees with the reference kernel
    assert O.rel_l2(O.fp_ref_f32(cas, axes, p.M, p.mask_radius, p.ker), ref) < TOL


@pytest.mark.parametrize("N", [32, 64])
def test_back_matches_reference_kernel(cuda, gglib, N):
    import torch

    rk = _ref()
    p = O.Params(N)
    rng = np.random.default_rng(N + 50)
    img = rng.standard_normal((16, p.M, p.M)).astype(np.float32)
    axes = test_axes(8, seed=N + 51)[:16]
    d_img, d_ker, d_axes = to_dev(img, cuda), to_dev(p.ker, cuda), to_dev(axes, cuda)
    ref = torch.zeros((p.V,) * 3, device=cuda)
    rk.back_project(ref.data_ptr(), p.V, d_img.data_ptr(), p.M, d_axes.data_ptr(), len(axes), p.mask_radius,
                    d_ker.data_ptr(), p.ker.size)
    got = torch.zeros_like(ref)
    assert gglib.gg_back_project_kernel(dptr(got), dptr(d_img), dptr(d_ker), dptr(d_axes), 2.0, len(axes), p.V, p.M,
                                        p.mask_radius, p.ker.size, 3, None) == 0
    torch.cuda.synchronize()
    ref, got = ref.cpu().numpy(), got.cpu().numpy()
    assert O.rel_l2(got, ref) < TOL
    assert O.rel_l2(O.bp_ref_f32(img, axes, p.V, p.mask_radius, p.ker), ref) < TOL


def test_l2_read_probe(cuda, gglib):
    """gg_measure_l2_read_gbs: the L2 read bandwidth the roofline is taken
    against; a GB300 reads its L2 well above its HBM rate and below 100 TB/s."""
    gbs = ctypes.c_double()
    assert gglib.gg_measure_l2_read_gbs(3, ctypes.byref(gbs)) == 0
    print("L2 read %.0f GB/s" % gbs.value)
    assert 2000.0 < gbs.value < 100000.0
    assert gglib.gg_measure_l2_read_gbs(0, ctypes.byref(gbs)) != 0
