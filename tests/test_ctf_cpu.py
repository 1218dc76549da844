"""The CTF formula of the CTF-corrected reconstruction (oracle side)."""
import math

import numpy as np

from oracle import oracle as O


def test_wavelength_300kv():
    # 300 kV electrons: 0.019687 Å
    assert abs(O.electron_wavelength(300.0) - 0.019687) < 2e-6


def test_ctf_zero_aberration_is_minus_one():
    c = O.ctf_cas(16, [0.0, 0.0], 300.0, 0.0, 1.0, 1.3)
    assert c.shape == (2, 16, 16)
    assert np.array_equal(c, -np.ones_like(c))


def test_ctf_dc_and_first_zero():
    M, px, A, df = 64, 1.5, 0.07, 15000.0
    c = O.ctf_cas(M, [df], 300.0, 0.0, A, px)[0]
    assert abs(c[M // 2, M // 2] + A) < 1e-12               # chi = 0 at DC
    h = M // 2
    assert np.array_equal(c[:, h + 1:], c[:, h - 1:0:-1])   # even in x about the centre
    assert np.array_equal(c[h + 1:], c[h - 1:0:-1])         # and in y
    # with Cs = 0 and A = 0 the first zero is at s^2 = 1 / (lambda df)
    lam = O.electron_wavelength(300.0)
    s0 = math.sqrt(1.0 / (lam * df))
    pure = O.ctf_cas(M, [df], 300.0, 0.0, 0.0, px)[0]
    r = np.hypot(*np.meshgrid(np.arange(M) - M // 2, np.arange(M) - M // 2)) / (M * px)
    near = np.abs(r - s0) < 0.2 / (M * px)
    if near.any():
        assert np.max(np.abs(pure[near])) < 0.2
    inside = r < 0.8 * s0
    assert np.all(pure[inside] <= 0)                        # negative before the first zero


def test_ctf_corrected_reconstruction_reduces_to_plain():
    # CTF = -1 everywhere: the result is minus reconstructVol's
    N = 16
    p = O.Params(N)
    vol = O.blob_volume(N, 4, seed=5)
    axes = O.quaternion_axes(6, seed=6)
    imgs = O.forward_project(vol, axes, p)[0]
    plain = O.reconstruct_vol(imgs, axes, p)[0]
    ctf = O.reconstruct_vol_ctf(imgs, axes, p, np.zeros(len(axes)), 300.0, 0.0, 1.0, 1.0)[0]
    assert np.allclose(ctf, -plain, rtol=0, atol=1e-12 * np.abs(plain).max())


def test_astigmatic_ctf_reduces_and_is_symmetric():
    M, px, A = 64, 1.2, 0.1
    u = [15000.0, 9000.0]
    v = [12000.0, 9000.0]
    ang = [0.3, -1.1]
    c = O.ctf_cas(M, u, 300.0, 2.7, A, px, v, ang)
    # V = U: the isotropic CTF
    assert np.array_equal(O.ctf_cas(M, u, 300.0, 2.7, A, px, u, ang), O.ctf_cas(M, u, 300.0, 2.7, A, px))
    # the angle is defined modulo pi, and (U, V, a) equals (V, U, a + pi/2)
    c_pi = O.ctf_cas(M, u, 300.0, 2.7, A, px, v, np.add(ang, math.pi))
    c_sw = O.ctf_cas(M, v, 300.0, 2.7, A, px, u, np.add(ang, math.pi / 2))
    assert np.allclose(c_pi, c, rtol=0, atol=1e-9) and np.allclose(c_sw, c, rtol=0, atol=1e-9)
    # along the U axis the defocus is U: pixel (M/2 + 10, M/2) with angle 0
    cu = O.ctf_cas(M, [u[0]], 300.0, 2.7, A, px, [v[0]], [0.0])[0]
    iso = O.ctf_cas(M, [u[0]], 300.0, 2.7, A, px)[0]
    assert abs(cu[M // 2, M // 2 + 10] - iso[M // 2, M // 2 + 10]) < 1e-12
