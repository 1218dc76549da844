"""GPU parity of the filter building blocks and the 2-D image stages against
the reference's own kernels.

The reference pins each filter with an exact-equality known-answer test
(src/Tests/Filter_Unit_Tests.m:1-86; ComplexToCASTest.m:12-14,
CASToComplexTest.m:15-22, FFTShift2DTest.m:15-20, FFTShift3DTest.m:15-17,
PadVolumeTest.m:14-21, CropVolumeTest.m:15-17, DivideVolumeTest.m:8-20).  Here
each gg_filter_* runs beside the reference's filter kernel (compiled
unmodified from src/Filters/*Filter.cu into oracle/_ref/, launched with its
UpdateFilter geometry by oracle/ref_kernels.py) on the same seeded inputs,
and the outputs must be equal bit for bit.

The image stages (gpuGridder::CASImgsToImgs / ::ImgsToCASImgs,
gpuGridder.cpp:432-596) are checked through the gridder's own calls against
the reference's chain of those filters with one cuFFT C2C per image, at
relative L2 <= 1e-5 (different FFT algorithms round differently).
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def vp(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def ref(cuda):
    from oracle import ref_kernels

    if not ref_kernels.filters_available():
        pytest.skip("reference filter cubins not built (oracle/build.py build_ref)")
    return ref_kernels.RefFilters()


def _rand(shape, seed, dev, zeros=0.0):
    import torch

    rng = np.random.default_rng(seed)
    a = rng.standard_normal(shape).astype(np.float32)
    if zeros:
        a[rng.random(shape) < zeros] = 0.0
    return torch.from_numpy(a).to(dev)


def _equal(a, b):
    import torch

    torch.cuda.synchronize()
    return np.array_equal(a.cpu().numpy(), b.cpu().numpy())


# (size, n_slices): stacks of 2-D slices, and n_slices = 0 for a size^3 volume
SLICE_CASES = [(16, 3), (64, 5), (100, 2), (16, 0), (34, 0)]


@pytest.mark.parametrize("size,ns", SLICE_CASES)
def test_complex_to_cas_and_back(cuda, gglib, ref, size, ns):
    import torch

    nsl = ns or size
    c = _rand((nsl, size, size, 2), 1 + size, cuda)
    mine, theirs = (torch.full((nsl, size, size), float("nan"), device=cuda) for _ in range(2))
    assert gglib.gg_filter_complex_to_cas(vp(c), vp(mine), size, ns, None) == 0
    ref.complex_to_cas(c.data_ptr(), theirs.data_ptr(), size, ns)
    assert _equal(mine, theirs)
    r = _rand((nsl, size, size), 2 + size, cuda)
    mine_c, theirs_c = (torch.full((nsl, size, size, 2), float("nan"), device=cuda) for _ in range(2))
    assert gglib.gg_filter_cas_to_complex(vp(r), vp(mine_c), size, ns, None) == 0
    ref.cas_to_complex(r.data_ptr(), theirs_c.data_ptr(), size, ns)
    assert _equal(mine_c, theirs_c)


@pytest.mark.parametrize("size,ns", SLICE_CASES)
def test_real_complex_conversions(cuda, gglib, ref, size, ns):
    import torch

    nsl = ns or size
    r = _rand((nsl, size, size), 3 + size, cuda)
    mine, theirs = (torch.full((nsl, size, size, 2), float("nan"), device=cuda) for _ in range(2))
    assert gglib.gg_filter_real_to_complex(vp(r), vp(mine), size, ns, None) == 0
    ref.real_to_complex(r.data_ptr(), theirs.data_ptr(), size, ns)
    assert _equal(mine, theirs)
    c = _rand((nsl, size, size, 2), 4 + size, cuda)
    mine_r, theirs_r = (torch.full((nsl, size, size), float("nan"), device=cuda) for _ in range(2))
    assert gglib.gg_filter_complex_to_real(vp(c), vp(mine_r), size, ns, None) == 0
    ref.complex_to_real(c.data_ptr(), theirs_r.data_ptr(), size, ns)
    assert _equal(mine_r, theirs_r)


@pytest.mark.parametrize("complex_elems", [0, 1])
@pytest.mark.parametrize("size,ns", [(16, 3), (64, 2), (256, 1)])
def test_fftshift_2d(cuda, gglib, ref, size, ns, complex_elems):
    shape = (ns, size, size, 2) if complex_elems else (ns, size, size)
    a = _rand(shape, 5 + size, cuda)
    b = a.clone()
    assert gglib.gg_filter_fftshift_2d(vp(a), complex_elems, size, ns, None) == 0
    ref.fftshift_2d(b.data_ptr(), size, ns, bool(complex_elems))
    assert _equal(a, b)


@pytest.mark.parametrize("complex_elems", [0, 1])
@pytest.mark.parametrize("size", [8, 32, 66])
def test_fftshift_3d(cuda, gglib, ref, size, complex_elems):
    shape = (size, size, size, 2) if complex_elems else (size, size, size)
    a = _rand(shape, 6 + size, cuda)
    b = a.clone()
    assert gglib.gg_filter_fftshift_3d(vp(a), complex_elems, size, None) == 0
    ref.fftshift_3d(b.data_ptr(), size, bool(complex_elems))
    assert _equal(a, b)


@pytest.mark.parametrize("dims,pads", [((16, 16, 5), (8, 8, 0)), ((64, 64, 3), (32, 32, 0)),
                                       ((12, 10, 7), (3, 2, 1)), ((20, 20, 20), (4, 4, 4))])
def test_pad_and_crop(cuda, gglib, ref, dims, pads):
    import torch

    ix, iy, iz = dims
    px, py, pz = pads
    ox, oy, oz = ix + 2 * px, iy + 2 * py, iz + 2 * pz
    x = _rand((iz, iy, ix), 7 + ix, cuda)
    mine = torch.full((oz, oy, ox), float("nan"), device=cuda)
    theirs = torch.zeros((oz, oy, ox), device=cuda)  # the reference writes the interior only
    assert gglib.gg_filter_pad_volume(vp(x), vp(mine), ix, iy, iz, px, py, pz, None) == 0
    ref.pad_volume(x.data_ptr(), theirs.data_ptr(), ix, iy, iz, px, py, pz)
    assert _equal(mine, theirs)
    # crop the padded volume back (the inverse of the pad)
    y = _rand((oz, oy, ox), 8 + ix, cuda)
    mine_c, theirs_c = (torch.full((iz, iy, ix), float("nan"), device=cuda) for _ in range(2))
    assert gglib.gg_filter_crop_volume(vp(y), vp(mine_c), ox, oy, oz, px, py, pz, None) == 0
    ref.crop_volume(y.data_ptr(), theirs_c.data_ptr(), ox, oy, oz, px, py, pz)
    assert _equal(mine_c, theirs_c)


@pytest.mark.parametrize("size,ns", SLICE_CASES)
def test_volume_arithmetic(cuda, gglib, ref, size, ns):
    nsl = ns or size
    shape = (nsl, size, size)
    # divide with the zero guard: zeros in numerator and denominator
    a, b = _rand(shape, 9 + size, cuda, zeros=0.2), _rand(shape, 10 + size, cuda, zeros=0.2)
    a2 = a.clone()
    assert gglib.gg_filter_divide_volumes(vp(a), vp(b), size, ns, None) == 0
    ref.divide_volumes(a2.data_ptr(), b.data_ptr(), size, ns)
    assert _equal(a, a2)
    # multiply, real and complex first operand
    a, b = _rand(shape, 11 + size, cuda), _rand(shape, 12 + size, cuda)
    a2 = a.clone()
    assert gglib.gg_filter_multiply_volumes(vp(a), vp(b), 0, size, ns, None) == 0
    ref.multiply_volumes(a2.data_ptr(), b.data_ptr(), size, ns, False)
    assert _equal(a, a2)
    c = _rand(shape + (2,), 13 + size, cuda)
    c2 = c.clone()
    assert gglib.gg_filter_multiply_volumes(vp(c), vp(b), 1, size, ns, None) == 0
    ref.multiply_volumes(c2.data_ptr(), b.data_ptr(), size, ns, True)
    assert _equal(c, c2)
    # divide by a scalar (the image stage's 1/M^2 normalisation, gpuGridder.cpp:510-517)
    a = _rand(shape, 14 + size, cuda)
    a2 = a.clone()
    assert gglib.gg_filter_divide_scalar(vp(a), 65536.0, size, ns, None) == 0
    ref.divide_scalar(a2.data_ptr(), 65536.0, size, ns)
    assert _equal(a, a2)
    a = _rand(shape, 15 + size, cuda)
    a2 = a.clone()
    assert gglib.gg_filter_divide_scalar(vp(a), 3.0, size, ns, None) == 0
    ref.divide_scalar(a2.data_ptr(), 3.0, size, ns)
    assert _equal(a, a2)


@pytest.mark.parametrize("size,ns", [(16, 3), (64, 5), (34, 34)])
def test_add_volumes(cuda, gglib, ref, size, ns):
    # the reference's AddVolumeFilter needs n_slices > 0 (AddVolumeFilter.cu:42-46)
    shape = (ns, size, size)
    a, b = _rand(shape, 16 + size, cuda), _rand(shape, 17 + size, cuda)
    a2 = a.clone()
    assert gglib.gg_filter_add_volumes(vp(a), vp(b), size, ns, None) == 0
    ref.add_volumes(a2.data_ptr(), b.data_ptr(), size, ns)
    assert _equal(a, a2)


# ---------------------------------------------------------------------------
# The 2-D image stages against the reference's filter + cuFFT chain
# ---------------------------------------------------------------------------

def _gridder(N, n, batch):
    import multigpugridder_gb300 as gg

    return gg.MultiGPUGridder(N, n, 2.0, MaxAxesToAllocate=batch, adjustInterpFactor=False)


# N = 32, 64, 128 take the fused 2-D FFT kernels; N = 50 (M = 100) the cuFFT R2C/C2R path
@pytest.mark.parametrize("N,n,batch", [(32, 40, 16), (64, 12, 12), (128, 9, 4), (50, 10, 10)])
def test_cas_images_to_images_matches_reference_chain(cuda, ref, N, n, batch):
    """forwardProject's CAS images -> images (gpuGridder.cpp:432-518)."""
    import torch

    from multigpugridder_gb300._lib import check, lib

    L = lib()
    vol = O.blob_volume(N, 8, seed=200 + N)
    axes = O.quaternion_axes(n, seed=201 + N).astype(np.float32)
    g = _gridder(N, n, batch)
    try:
        g.setVolume(vol)
        M = g.M
        d_ax = torch.from_numpy(axes).to(cuda)
        imgs = torch.full((n, N, N), float("nan"), device=cuda)
        cas = torch.full((n, M, M), float("nan"), device=cuda)
        s = torch.cuda.current_stream(cuda)
        check(L.gg_forward_project_dev(g.handle, vp(d_ax), n, vp(imgs), vp(cas), ctypes.c_void_p(s.cuda_stream)),
              g.handle)
        torch.cuda.synchronize()
        work = cas.clone()
        out = torch.zeros((n, N, N), device=cuda)
        cplx = torch.zeros((n, M, M, 2), device=cuda)
        ref.cas_imgs_to_imgs(work.data_ptr(), out.data_ptr(), cplx.data_ptr(), M, N, n, 2.0)
        torch.cuda.synchronize()
    finally:
        g.close()
    got, want = imgs.cpu().numpy(), out.cpu().numpy()
    assert np.all(np.isfinite(got))
    err = O.rel_l2(got, want)
    print("CAS images -> images N=%d: rel-L2 %.2e against the reference chain" % (N, err))
    assert err < TOL


@pytest.mark.parametrize("N,n,batch", [(32, 40, 16), (64, 12, 12), (128, 9, 4), (50, 10, 10)])
def test_images_to_cas_images_matches_reference_chain(cuda, ref, N, n, batch):
    """backProject's images -> CAS images (gpuGridder.cpp:520-596): the
    gridder back-projects the images (its own image stage) and the reference
    chain's CAS images (the host-FFT interface); the back projection is the
    same bit-exact kernel, so the volumes differ only by the image stage."""
    import torch

    from multigpugridder_gb300._lib import check, lib

    L = lib()
    rng = np.random.default_rng(300 + N)
    imgs = rng.standard_normal((n, N, N)).astype(np.float32)
    axes = O.quaternion_axes(n, seed=301 + N).astype(np.float32)
    g = _gridder(N, n, batch)
    try:
        M, V = g.M, g.V
        d_img = torch.from_numpy(imgs).to(cuda)
        d_ax = torch.from_numpy(axes).to(cuda)
        cas = torch.zeros((n, M, M), device=cuda)
        cplx = torch.zeros((n, M, M, 2), device=cuda)
        ref.imgs_to_cas_imgs(d_img.data_ptr(), cas.data_ptr(), cplx.data_ptr(), M, N, n)
        torch.cuda.synchronize()
        s = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
        a = torch.empty((V, V, V), device=cuda)
        b = torch.empty((V, V, V), device=cuda)
        check(L.gg_back_project_dev(g.handle, vp(d_ax), n, vp(d_img), None, 0, s), g.handle)
        check(L.gg_get_cas_volume_dev(g.handle, vp(a), s), g.handle)
        check(L.gg_back_project_dev(g.handle, vp(d_ax), n, None, vp(cas), 0, s), g.handle)
        check(L.gg_get_cas_volume_dev(g.handle, vp(b), s), g.handle)
        torch.cuda.synchronize()
    finally:
        g.close()
    err = O.rel_l2(a.cpu().numpy(), b.cpu().numpy())
    print("images -> CAS images N=%d: rel-L2 %.2e (through the back projection) against the reference chain"
          % (N, err))
    assert err < TOL
