"""The differentiable form: exact adjoint of the whole forward operator,
checked by the adjoint identity, against the FP64 oracle, and against FP64
finite differences of the loss ||P(V) - Y||^2 (32^3, 64 directions, step 1e-6,
50 random voxels)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_adjoint_identity_fp32(cuda):
    import torch

    from multigpugridder_gb300.autograd import ForwardProjector

    N = 32
    rng = np.random.default_rng(41)
    axes = torch.from_numpy(O.quaternion_axes(16, seed=42).astype(np.float32)).to(cuda)
    x = torch.from_numpy(rng.standard_normal((N,) * 3).astype(np.float32)).to(cuda)
    y = torch.from_numpy(rng.standard_normal((16, N, N)).astype(np.float32)).to(cuda)
    proj = ForwardProjector(N, 2.0)
    px = proj.project(x, axes)
    pty = proj.adjoint(y, axes)
    lhs = torch.sum(px.double() * y.double()).item()
    rhs = torch.sum(x.double() * pty.double()).item()
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
    proj.close()


def test_adjoint_matches_fp64_oracle(cuda):
    import torch

    from multigpugridder_gb300.autograd import ForwardProjector

    N = 24
    p = O.Params(N)
    rng = np.random.default_rng(43)
    axes_np = O.quaternion_axes(12, seed=44)
    y = rng.standard_normal((12, N, N))
    ref = O.forward_adjoint(y, axes_np, p)
    proj = ForwardProjector(N, 2.0)
    got = proj.adjoint(torch.from_numpy(y.astype(np.float32)).to(cuda),
                       torch.from_numpy(axes_np.astype(np.float32)).to(cuda)).cpu().numpy()
    proj.close()
    # FP32 rounding can move a nearest-index table lookup
    assert O.rel_l2(got, ref) < 1e-3


def test_gradient_matches_fp64_finite_differences(cuda):
    """Configuration of the differentiation workload: 32^3, 64 random
    directions, Y = P(V_true) + noise at SNR 0.1, loss ||P(V) - Y||^2."""
    import torch

    from multigpugridder_gb300.autograd import ForwardProjector

    N = 32
    p = O.Params(N)
    axes_np = O.quaternion_axes(64, seed=45)
    v_true = O.blob_volume(N, 8, seed=46).astype(np.float64)
    v0 = O.blob_volume(N, 8, seed=47).astype(np.float32)
    clean = O.forward_operator(v_true, axes_np, p)
    rng = np.random.default_rng(48)
    Y = clean + rng.normal(0.0, np.sqrt(np.var(clean) / 0.1), clean.shape)

    proj = ForwardProjector(N, 2.0)
    vol = torch.from_numpy(v0).to(cuda).requires_grad_(True)
    axes = torch.from_numpy(axes_np.astype(np.float32)).to(cuda)
    Yt = torch.from_numpy(Y.astype(np.float32)).to(cuda)
    loss = torch.sum((proj.project(vol, axes) - Yt) ** 2)
    loss.backward()
    g_gpu = vol.grad.double().cpu().numpy()
    proj.close()

    def L(v):
        r = O.forward_operator(v, axes_np, p) - Y
        return float(np.sum(r * r))

    h = 1e-6
    base = v0.astype(np.float64)
    idx = rng.choice(N ** 3, size=50, replace=False)
    fd = []
    for i in idx:
        e = np.zeros(N ** 3)
        e[i] = h
        e = e.reshape(base.shape)
        fd.append((L(base + e) - L(base - e)) / (2 * h))
    fd = np.array(fd)
    got = g_gpu.ravel()[idx]
    err = np.max(np.abs(got - fd)) / np.max(np.abs(fd))
    print("gradient vs FP64 finite differences: max rel %.2e" % err)
    assert err < 1e-3


def test_adjoint_equals_reference_rule_for_axis_aligned_directions(cuda, gglib):
    """The reference BP window and the forward window pick the same pairs for
    axis-aligned directions (inside the mask); elsewhere they differ."""
    import ctypes

    import torch

    p = O.Params(16)
    rng = np.random.default_rng(49)
    axes = np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1], [0, 1, 0, 0, 0, 1, 1, 0, 0]], np.float32)
    y = rng.standard_normal((2, p.M, p.M)).astype(np.float32)
    q = np.arange(p.M) - p.M // 2
    y[:, (q[:, None] ** 2 + q[None, :] ** 2) > p.mask_radius ** 2] = 0
    dy, dk, da = (torch.from_numpy(a).to(cuda) for a in (y, p.ker, axes))
    ref = torch.zeros((p.V,) * 3, device=cuda)
    adj = torch.zeros_like(ref)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    assert gglib.gg_back_project_kernel(vp(ref), vp(dy), vp(dk), vp(da), 2.0, 2, p.V, p.M, p.mask_radius, 501, 3,
                                        None) == 0
    assert gglib.gg_back_project_adjoint_kernel(vp(adj), vp(dy), vp(dk), vp(da), 2.0, 2, p.V, p.M, p.mask_radius,
                                                501, None) == 0
    torch.cuda.synchronize()
    c = np.arange(p.V) - p.V // 2
    inside = (c[:, None, None] ** 2 + c[None, :, None] ** 2 + c[None, None, :] ** 2) <= p.mask_radius ** 2
    r, a = ref.cpu().numpy(), adj.cpu().numpy()
    assert O.rel_l2(a[inside], r[inside]) < 1e-5
