"""CPU checks of the oracle: the reference's known-answer tests, closed forms,
round trips, and the FFT formulation the CUDA kernels use (real-to-complex /
complex-to-real transforms with the fftshifts folded into index maps)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# ---------------------------------------------------------------------------
# KB table and pre-compensation
# ---------------------------------------------------------------------------


def test_kb_table_properties():
    t = O.kb_table(2, 501)
    assert t.shape == (501,)
    assert t[0] == 0.0 and t[-1] == 0.0  # getKernelFiltTable.m:12-13
    assert np.allclose(t, t[::-1], rtol=0, atol=1e-15)
    # normalised so the 5 integer taps sum to 1 (so the 5^3 kernel sums to 1)
    assert abs(t[[0, 125, 250, 375, 500]].sum() - 1.0) < 1e-14
    assert np.all(np.diff(t[:251]) > 0)


def test_kb_table_golden():
    g = np.load(os.path.join(GOLDEN, "kb_precomp.npz"))
    assert np.array_equal(O.kb_table(2, 501).astype(np.float32), g["kb_table_f32"])
    for M in (64, 128, 256):
        assert np.allclose(O.precomp(M, 2), g["precomp_%d" % M], rtol=1e-13, atol=0)


def test_precomp_is_cosine_sum():
    M = 128
    x = np.arange(-2, 2.0001, 0.25)
    w = O.grid_lib_kaiser(2, 10.0, x)
    w = w - w[0]
    w[-1] = 0
    m = np.arange(-8, 9)
    P = np.array([np.sum(w * np.cos(2 * np.pi * j * m / (4 * M))) for j in range(-M // 2, M // 2)])
    assert np.allclose(O.precomp(M), P[M // 2] / P, rtol=1e-13)
    assert O.precomp(M)[M // 2] == 1.0


def test_bessel_i0_matches_scipy():
    from scipy.special import i0

    x = np.linspace(0, 20, 101)
    assert np.allclose(O.bessel_i0(x), i0(x), rtol=1e-14)


# ---------------------------------------------------------------------------
# CAS conversions and round trips
# ---------------------------------------------------------------------------


def test_from_cas_is_hermitian_and_inverts_to_cas():
    rng = np.random.default_rng(1)
    r = rng.standard_normal((8, 8, 8))
    c = O.from_cas(r)
    # c[k] = conj(c[-k]) for all indices >= 1 (pairing m <-> s-m)
    inner = c[1:, 1:, 1:]
    assert np.allclose(inner, np.conj(inner[::-1, ::-1, ::-1]))
    assert np.allclose(O.to_cas(c)[1:, 1:, 1:], r[1:, 1:, 1:])
    assert np.all(c[0] == 0) and np.all(c[:, 0] == 0) and np.all(c[:, :, 0] == 0)


@pytest.mark.parametrize("N", [8, 16])
def test_volume_cas_round_trip(N):
    """volFromCAS(CASFromVol(v)): both directions multiply by the precomp
    (getPreComp is the inverse KB transform, applied once per gridding pass)
    and FromCAS drops the Nyquist planes, so the round trip is
    real(ifft(Nyquist-zeroed fft(v*pc^3))) * pc^3, cropped."""
    vol = O.blob_volume(N, 4, seed=N).astype(np.float64)
    cas = O.cas_from_vol(vol)
    assert cas.shape == (2 * N + 6,) * 3
    M = 2 * N
    b = M // 2 - N // 2
    iv = np.zeros((M,) * 3)
    iv[b:b + N, b:b + N, b:b + N] = vol
    pc = O.precomp(M)
    pc3 = pc[:, None, None] * pc[None, :, None] * pc[None, None, :]
    F = np.fft.fftshift(np.fft.fftn(np.fft.fftshift(iv * pc3)))
    F[0, :, :] = 0
    F[:, 0, :] = 0
    F[:, :, 0] = 0
    want = (np.real(np.fft.fftshift(np.fft.ifftn(np.fft.fftshift(F)))) * pc3)[b:b + N, b:b + N, b:b + N]
    assert np.allclose(O.vol_from_cas(cas, N), want, rtol=0, atol=1e-10 * np.abs(want).max())


def test_image_cas_round_trip():
    """imgsFromCASImgs(CASImgsFromImgs(x)) is x with the Nyquist row and
    column of the padded spectrum removed (FromCAS zeroes them)."""
    rng = np.random.default_rng(2)
    x = rng.standard_normal((3, 16, 16))
    p = np.zeros((3, 32, 32))
    p[:, 8:24, 8:24] = x
    F = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(p, axes=(1, 2))), axes=(1, 2))
    F[:, 0, :] = 0
    F[:, :, 0] = 0
    want = np.real(np.fft.fftshift(np.fft.ifft2(np.fft.fftshift(F, axes=(1, 2))), axes=(1, 2)))[:, 8:24, 8:24]
    assert np.allclose(O.imgs_from_cas_imgs(O.cas_imgs_from_imgs(x, 32), 16), want, atol=1e-12)


# ---------------------------------------------------------------------------
# The CUDA kernels' FFT formulation, modelled in NumPy
# ---------------------------------------------------------------------------


def _shift(q, M):
    return (q + M // 2) % M


def test_model_cas_prep_r2c_with_index_remaps():
    """vol_to_fft_input -> R2C -> spectrum_to_cas_volume (gg_cas.cu)."""
    N, M, pad = 8, 16, 3
    V = M + 2 * pad
    vol = O.blob_volume(N, 3, seed=3).astype(np.float64)
    pc = O.precomp(M)
    q = np.arange(M)
    src = _shift(q, M) - (M // 2 - N // 2)
    x = np.zeros((M, M, M))
    ok = (src >= 0) & (src < N)
    k, j, i = np.ix_(q[ok], q[ok], q[ok])
    x[k, j, i] = vol[np.ix_(src[ok], src[ok], src[ok])]
    sh = _shift(q, M)
    x *= (pc[sh][:, None, None] * pc[sh][None, :, None] * pc[sh][None, None, :])
    Y = np.fft.rfftn(x)  # [w][v][u], u <= M/2
    cas = np.zeros((V, V, V))
    ii = np.arange(M)
    u, v, w = _shift(ii, M)[None, None, :], _shift(ii, M)[None, :, None], _shift(ii, M)[:, None, None]
    u, v, w = np.broadcast_arrays(u, v, w)
    low = u <= M // 2
    val = np.empty((M, M, M))
    c = Y[w[low], v[low], u[low]]
    val[low] = c.real + c.imag
    w2, v2, u2 = (M - w[~low]) % M, (M - v[~low]) % M, M - u[~low]
    c = Y[w2, v2, u2]
    val[~low] = c.real - c.imag
    cas[pad:pad + M, pad:pad + M, pad:pad + M] = val
    assert np.allclose(cas, O.cas_from_vol(vol, 2, 2, pad), atol=1e-9)


def test_model_fp_image_path_c2r():
    """cas_images_to_spectrum -> C2R -> fft_output_to_images (gg_cas.cu)."""
    M, N = 16, 8
    rng = np.random.default_rng(4)
    r = rng.standard_normal((2, M, M))
    H = M // 2 + 1
    spec = np.zeros((2, M, H), complex)
    for v in range(M):
        for u in range(H):
            i, j = _shift(u, M), _shift(v, M)
            if i and j:
                a, b = r[:, j, i], r[:, M - j, M - i]
                spec[:, v, u] = 0.5 * (a + b) + 0.5j * (a - b)
    y = np.fft.irfft2(spec, s=(M, M)) * M * M  # cuFFT C2R is unnormalised
    ob = (M - N) // 2
    idx = _shift(np.arange(N) + ob, M)
    img = y[:, idx][:, :, idx] / (M * M)
    assert np.allclose(img, O.imgs_from_cas_imgs(r, N), atol=1e-12)


def test_model_bp_image_path_r2c():
    """images_to_fft_input -> R2C -> spectrum_to_cas_images (gg_cas.cu)."""
    M, N = 16, 8
    rng = np.random.default_rng(5)
    x = rng.standard_normal((2, N, N))
    b = (M - N) // 2
    q = np.arange(M)
    src = _shift(q, M) - b
    ok = (src >= 0) & (src < N)
    xin = np.zeros((2, M, M))
    xin[:, q[ok][:, None], q[ok][None, :]] = x[:, src[ok][:, None], src[ok][None, :]]
    Y = np.fft.rfft2(xin)
    cas = np.zeros((2, M, M))
    for j in range(M):
        for i in range(M):
            u, v = _shift(i, M), _shift(j, M)
            if u <= M // 2:
                c = Y[:, v, u]
                cas[:, j, i] = c.real + c.imag
            else:
                c = Y[:, (M - v) % M, M - u]
                cas[:, j, i] = c.real - c.imag
    assert np.allclose(cas, O.cas_imgs_from_imgs(x, M), atol=1e-10)


def test_model_get_volume_c2r():
    """cas_volume_to_spectrum -> C2R -> fft_output_to_vol (gg_cas.cu)."""
    N, M, pad = 8, 16, 3
    V = M + 2 * pad
    rng = np.random.default_rng(6)
    cas = rng.standard_normal((V, V, V))
    b = V // 2 - M // 2
    H = M // 2 + 1
    spec = np.zeros((M, M, H), complex)
    for w in range(M):
        for v in range(M):
            for u in range(H):
                i, j, k = _shift(u, M), _shift(v, M), _shift(w, M)
                if i and j and k:
                    r1 = cas[k + b, j + b, i + b]
                    r2 = cas[M - k + b, M - j + b, M - i + b]
                    spec[w, v, u] = 0.5 * (r1 + r2) + 0.5j * (r1 - r2)
    y = np.fft.irfftn(spec, s=(M, M, M), axes=(0, 1, 2)) * M ** 3
    pc = O.precomp(M)
    ob = M // 2 - N // 2
    idx = _shift(np.arange(N) + ob, M)
    p = pc[np.arange(N) + ob]
    vol = y[np.ix_(idx, idx, idx)] / M ** 3 * (p[:, None, None] * p[None, :, None] * p[None, None, :])
    assert np.allclose(vol, O.vol_from_cas(cas, N), atol=1e-12)


# ---------------------------------------------------------------------------
# Kernel restatements: the reference's known-answer tests
# ---------------------------------------------------------------------------


def test_forward_sphere_known_answer():
    """ForwardProjectTests.m:28-69 (smaller volume): max |mean(img - sum_z V)| <= 1."""
    N = 32
    p = O.Params(N)
    vol = O.fuzzymask(N, 3, N * 0.25, 2, (N // 2 + 1) * np.ones(3))
    axes = O.create_uniform_axes(4, 10)
    imgs, _ = O.forward_project(vol, axes, p, "f32")
    gt = vol.sum(axis=0)
    assert np.max(np.abs((imgs - gt[None]).reshape(len(axes), -1).mean(1))) <= 1.0
    assert np.max(np.abs(imgs - gt[None])) < 0.1


def test_reconstruction_known_answer():
    """BackProjectTests.m:25-66 (smaller volume): max |recon - V| <= 1."""
    N = 32
    p = O.Params(N)
    vol = O.fuzzymask(N, 3, N * 0.25, 2, (N // 2 + 1) * np.ones(3))
    axes = O.create_uniform_axes(20, 40)
    imgs, _ = O.forward_project(vol, axes, p, "f64")
    rec, _, _ = O.reconstruct_vol(imgs, axes, p, "f64")
    assert np.max(np.abs(rec - vol)) <= 1.0


def test_f32_restatement_close_to_f64():
    """Same operator, different rounding.  The nearest-index KB lookup
    (roundf(r*125 + 250)) flips a table index whenever rounding moves the
    argument across a half-integer, and the BP window (5x5 pixels around
    round(projection), |f_imgk| <= 2) has discontinuous edges, so FP32 and
    FP64 evaluations differ by ~1e-5 (forward) and ~1e-4 (back) in relative L2.
    Parity at 1e-5 therefore needs the same rounding as the reference kernels,
    which the FP32 restatement reproduces."""
    N = 16
    p = O.Params(N)
    vol = O.blob_volume(N, 5, seed=3)
    axes = O.quaternion_axes(10, seed=4)
    cas = O.cas_from_vol(vol)
    a = O.fp_ref_f32(cas.astype(np.float32), axes, p.M, p.mask_radius, p.ker)
    b = O.fp_f64(cas, axes, p.M, p.mask_radius, p.ker)
    assert O.rel_l2(a, b) < 1e-4
    y = np.random.default_rng(5).standard_normal((10, p.M, p.M))
    c = O.bp_ref_f32(y.astype(np.float32), axes, p.V, p.mask_radius, p.ker)
    d = O.bp_ref_f64(y, axes, p.V, p.mask_radius, p.ker)
    assert O.rel_l2(c, d) < 1e-3


def test_adjoint_exact_and_reference_rule_not():
    N = 16
    p = O.Params(N)
    rng = np.random.default_rng(9)
    axes = O.quaternion_axes(6, seed=10)
    x = rng.standard_normal((p.V,) * 3)
    y = rng.standard_normal((6, p.M, p.M))
    Px = O.fp_f64(x, axes, p.M, p.mask_radius, p.ker)
    lhs = np.sum(Px * y)
    assert abs(lhs - np.sum(x * O.bp_adjoint_f64(y, axes, p.V, p.mask_radius, p.ker))) < 1e-10 * abs(lhs)
    assert abs(lhs - np.sum(x * O.bp_ref_f64(y, axes, p.V, p.mask_radius, p.ker))) > 1e-3 * abs(lhs)


def test_whole_operator_adjoint():
    """forward_adjoint is the exact adjoint of volume -> images (CAS prep,
    forward projection, CAS images -> images)."""
    N = 12
    p = O.Params(N)
    rng = np.random.default_rng(21)
    axes = O.quaternion_axes(5, seed=22)
    x = rng.standard_normal((N, N, N))
    y = rng.standard_normal((5, N, N))
    lhs = np.sum(O.forward_operator(x, axes, p) * y)
    rhs = np.sum(x * O.forward_adjoint(y, axes, p))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


def test_axis_aligned_reference_rule_is_adjoint():
    """For axis-aligned directions the two windows coincide on voxels inside
    the mask sphere (the reference BP writes no voxel outside it, while the
    forward window reaches up to sqrt(3) voxels past it)."""
    N = 16
    p = O.Params(N)
    rng = np.random.default_rng(11)
    axes = np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1], [0, 1, 0, 0, 0, 1, 1, 0, 0]], float)
    x = rng.standard_normal((p.V,) * 3)
    c = np.arange(p.V) - p.V // 2
    x[(c[:, None, None] ** 2 + c[None, :, None] ** 2 + c[None, None, :] ** 2) > p.mask_radius ** 2] = 0
    y = rng.standard_normal((2, p.M, p.M))
    # and images supported on the forward mask disc (the reference BP reads
    # every pixel of its window, the forward projection writes only the disc)
    q = np.arange(p.M) - p.M // 2
    y[:, (q[:, None] ** 2 + q[None, :] ** 2) > p.mask_radius ** 2] = 0
    lhs = np.sum(O.fp_f64(x, axes, p.M, p.mask_radius, p.ker) * y)
    rhs = np.sum(x * O.bp_ref_f64(y, axes, p.V, p.mask_radius, p.ker))
    assert abs(lhs - rhs) < 1e-4 * abs(lhs)


def test_axes_generators():
    ax = O.create_uniform_axes(10, 50)
    assert ax.shape == (500, 9)
    R = ax.reshape(-1, 3, 3)
    assert np.allclose(np.einsum("nij,nkj->nik", R, R), np.eye(3), atol=1e-12)
    # the 30 degree in-plane rotation gives exact halves once cast to single
    assert np.any(ax.astype(np.float32) == 0.5)
    g = O.grid_axes(100, 100)
    assert g.shape == (10000, 9)
    q = O.quaternion_axes(100, seed=1).reshape(-1, 3, 3)
    assert np.allclose(np.linalg.det(np.transpose(q, (0, 2, 1))), 1.0)


def test_blob_volume_seeded():
    a = O.blob_volume(32, 20, seed=1)
    b = O.blob_volume(32, 20, seed=1)
    assert np.array_equal(a, b)
    assert a.dtype == np.float32 and a.max() > 0.4


# ---------------------------------------------------------------------------
# Pins against outputs of the reference's own kernels (generated on a GB300
# by tests/golden/make_golden.py from the cubins in oracle/_ref)
# ---------------------------------------------------------------------------

REF_GOLDEN = os.path.join(GOLDEN, "reference_kernels.npz")


@pytest.mark.skipif(not os.path.exists(REF_GOLDEN), reason="reference-kernel fixtures not generated")
def test_oracle_matches_reference_kernel_outputs():
    """The C restatement replays the reference kernels' own outputs."""
    g = np.load(REF_GOLDEN)
    keys = sorted({k.split("_")[0] for k in g.files})
    assert keys
    for key in keys:
        N, M, V, R = (int(x) for x in g[key + "_meta"])
        cas, axes, img, ker = (g[key + "_" + s] for s in ("cas", "axes", "img", "ker"))
        # bit for bit: same operation order and the same fused multiply-adds
        fp = O.fp_ref_f32(cas, axes, M, R, ker)
        ref_fp = g[key + "_fp"]
        assert np.array_equal(fp, ref_fp), key
        bp = O.bp_ref_f32(img, axes, V, R, ker)
        assert np.array_equal(bp, g[key + "_bp"]), key
        # the FP64 oracle is the same operator
        assert O.rel_l2(O.fp_f64(cas, axes, M, R, ker), ref_fp) < 1e-5, key


REF_FILTERS = os.path.join(GOLDEN, "reference_filters.npz")


@pytest.mark.skipif(not os.path.exists(REF_FILTERS), reason="reference-filter fixtures not generated")
def test_oracle_matches_reference_filter_outputs():
    """The oracle's NumPy forms of the filters and image stages against the
    reference's own filter kernels and cuFFT chain (tests/golden/make_golden.py
    filters): data movement bit for bit, the CAS -> complex halves within FP32
    rounding of (a + b) / 2, the two image-stage chains (FP32 cuFFT against the
    FP64 restatement) within relative L2 1e-5."""
    g = np.load(REF_FILTERS)
    c2 = g["c2"][..., 0] + 1j * g["c2"][..., 1]
    r2, r3 = g["r2"], g["r3"]

    def cplx(x):
        return x[..., 0] + 1j * x[..., 1]

    # ComplexToCASFilter.cu:3-26 / ToCAS.m:5
    assert np.array_equal(O.to_cas(c2.astype(np.complex64)), g["complex_to_cas_2d"])
    # CASToComplexFilter.cu:3-81 / FromCAS.m:7-13, 2-D slices and the 3-D volume
    assert np.allclose(O.from_cas(r2, axes=(1, 2)), cplx(g["cas_to_complex_2d"]), rtol=1e-6, atol=1e-6)
    assert np.allclose(O.from_cas(r3), cplx(g["cas_to_complex_3d"]), rtol=1e-6, atol=1e-6)
    # FFTShift2DFilter.cu / FFTShift3DFilter.cu: fftshift over the slice axes
    assert np.array_equal(np.fft.fftshift(r2, axes=(1, 2)), g["fftshift_2d_real"])
    assert np.array_equal(np.fft.fftshift(g["c2"], axes=(1, 2)), g["fftshift_2d_complex"])
    assert np.array_equal(np.fft.fftshift(r3), g["fftshift_3d_real"])
    # PadVolumeFilter.cu (into a zeroed output) / CropVolumeFilter.cu
    assert np.array_equal(np.pad(g["pad_in"], ((1, 1), (2, 2), (1, 1))), g["pad_out"])
    assert np.array_equal(g["crop_in"][1:-1, 2:-2, 1:-1], g["crop_out"])
    a, b = g["arith_a"], g["arith_b"]
    with np.errstate(divide="ignore", invalid="ignore"):
        # DivideVolumeFilter.cu:24-31: the zero guard
        assert np.array_equal(np.where((a != 0) & (b != 0), a / b, np.float32(0)), g["divide"])
    assert np.array_equal(a * b, g["multiply"])
    assert np.array_equal(g["c2"] * b[..., None], g["multiply_complex"])
    assert np.array_equal(a + b, g["add"])
    assert np.array_equal(a / np.float32(3.0), g["divide_scalar"])
    assert np.array_equal(np.stack([r2, np.zeros_like(r2)], -1), g["real_to_complex"])
    assert np.array_equal(g["c2"][..., 0], g["complex_to_real"])
    # the image stages (gpuGridder.cpp:432-518 and :520-596)
    assert O.rel_l2(O.imgs_from_cas_imgs(g["chain_cas_in"], 16), g["chain_imgs_out"]) < 1e-5
    assert O.rel_l2(O.cas_imgs_from_imgs(g["chain_imgs_in"], 32), g["chain_cas_out"]) < 1e-5
