"""Seeded synthetic inputs for benchmarks and examples (no dataset is needed).

* blob_volume: a sum of isotropic Gaussian blobs, centres uniform in the
  inner 60% of the box, sigma uniform in 2-6 voxels, amplitude uniform in
  0.5-1.5, evaluated in FP64 and stored FP32, x fastest.
* quaternion_axes: directions from uniformly random unit quaternions
  (Shoemake's method), 9 floats each: the x, y, z columns of the rotation.
* grid_axes: a uniform direction grid, azimuth phi_a = 2 pi a / n_az and
  cos-polar cos(theta_b) = -1 + (2b + 1) / n_pol, each turned by an in-plane
  angle psi; the rotation is built as get_axes_from_n_rot does
  (src/Matlab/utils/get_axes_from_n_rot.m:19-36): Rz(phi) Ry(theta) Rz(psi).
"""
import math

import numpy as np


def blob_volume(N, n_blobs, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.2 * N, 0.8 * N, size=(n_blobs, 3))
    s = rng.uniform(2.0, 6.0, size=n_blobs)
    a = rng.uniform(0.5, 1.5, size=n_blobs)
    x = np.arange(N, dtype=np.float64)
    inv = 1.0 / (2.0 * s[:, None] ** 2)
    gx = np.exp(-((x[None, :] - c[:, 0:1]) ** 2) * inv)
    gy = np.exp(-((x[None, :] - c[:, 1:2]) ** 2) * inv)
    gz = np.exp(-((x[None, :] - c[:, 2:3]) ** 2) * inv) * a[:, None]
    # vol[k, j, i] = sum_b gz[b, k] gy[b, j] gx[b, i]; einsum may return any
    # memory order, and callers hand the buffer to the C ABI (x fastest)
    vol = np.einsum("bk,bj,bi->kji", gz, gy, gx, optimize=True)
    return np.ascontiguousarray(vol, dtype=dtype)


def quaternion_axes(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.random((n, 3))
    r1, r2 = np.sqrt(1.0 - u[:, 0]), np.sqrt(u[:, 0])
    t1, t2 = 2.0 * np.pi * u[:, 1], 2.0 * np.pi * u[:, 2]
    x, y = r1 * np.sin(t1), r1 * np.cos(t1)
    z, w = r2 * np.sin(t2), r2 * np.cos(t2)
    R = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)], -1),   # column 0
        np.stack([2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)], -1),   # column 1
        np.stack([2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)], -1),   # column 2
    ], 1)
    return R.reshape(n, 9)


def _rz(a):
    return np.array([[math.cos(a), -math.sin(a), 0.0], [math.sin(a), math.cos(a), 0.0], [0.0, 0.0, 1.0]])


def _ry(a):
    return np.array([[math.cos(a), 0.0, math.sin(a)], [0.0, 1.0, 0.0], [-math.sin(a), 0.0, math.cos(a)]])


def grid_axes(n_az=100, n_pol=100, psi_deg=30.0):
    psi = _rz(math.radians(psi_deg))
    out = np.empty((n_az * n_pol, 9))
    k = 0
    for b in range(n_pol):
        ct = -1.0 + (2 * b + 1) / n_pol
        st = math.sqrt(max(0.0, 1.0 - ct * ct))
        for a in range(n_az):
            ph = 2 * math.pi * a / n_az
            nx, ny = st * math.cos(ph), st * math.sin(ph)
            if math.hypot(nx, ny) < 1e-4:  # along z: no azimuth or polar turn
                T = psi
            else:
                T = (_rz(math.atan2(ny, nx)) @ _ry(math.atan2(math.hypot(nx, ny), ct))) @ psi
            out[k] = T.T.reshape(9)  # columns x, y, z
            k += 1
    return out
