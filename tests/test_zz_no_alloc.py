"""gg_back_project_normalized_noalloc, the entry point that allocates no
memory, through the C ABI.  Each call is compared with the existing stateless
back projection, gg_back_project_kernel on the images and on all-ones images,
divided as reconstructVol divides (MultiGPUGridder_Matlab_Class.m:308), on two
calls in a row.  Tolerance: relative L2 <= 1e-6 (both sides run the same
window rule and sums; only the quotient is formed in different code).

The file name makes pytest collect it last, so it runs both alone and after
every other GPU test."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _dev(a, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def _existing(gglib, img, ker, axes, p):
    """BP(images) / (BP(ones) + 1e-6) from two calls of gg_back_project_kernel."""
    import torch

    n = axes.numel() // 9
    bp = torch.zeros((p.V,) * 3, device=img.device)
    pd = torch.zeros_like(bp)
    ones = torch.ones_like(img)
    for out, src in ((bp, img), (pd, ones)):
        assert gglib.gg_back_project_kernel(_vp(out), _vp(src), _vp(ker), _vp(axes), 2.0, n, p.V, p.M, p.mask_radius,
                                            p.ker.size, 3, None) == 0
    return bp / (pd + 1e-6)


def _noalloc(gglib, out, img, ker, axes, p):
    n = axes.numel() // 9
    rc = gglib.gg_back_project_normalized_noalloc(_vp(out), _vp(img), _vp(ker), _vp(axes), 2.0, n, p.V, p.M,
                                                  p.mask_radius, p.ker.size, None)
    assert rc == 0, gglib.gg_global_error()


def _case(p, n, seed, dev):
    rng = np.random.default_rng(seed)
    img = rng.standard_normal((n, p.M, p.M)).astype(np.float32)
    axes = np.concatenate([O.quaternion_axes(n - 4, seed + 1), O.create_uniform_axes(2, 2)]).astype(np.float32)[:n]
    return _dev(img, dev), _dev(axes, dev)


@pytest.mark.parametrize("N", [16, 64])
def test_noalloc_matches_existing_entry_two_calls_in_a_row(cuda, gglib, N):
    import torch

    p = O.Params(N)  # N = 64: cas_vol_size 134, near the 161 limit
    ker = _dev(p.ker, cuda)
    cases = [_case(p, 40, 500 + N, cuda), _case(p, 23, 600 + N, cuda)]
    for img, axes in cases:
        # the output need not start at zero: start from NaN
        out = torch.full((p.V,) * 3, float("nan"), device=cuda)
        _noalloc(gglib, out, img, ker, axes, p)
        ref = _existing(gglib, img, ker, axes, p)
        torch.cuda.synchronize()
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(got))
        err = O.rel_l2(got, want)
        print("noalloc N=%d n=%d: rel-L2 %.2e vs gg_back_project_kernel" % (N, axes.numel() // 9, err))
        assert err <= TOL


def test_noalloc_leaves_free_device_memory_unchanged(cuda, gglib):
    import torch

    p = O.Params(32)
    ker = _dev(p.ker, cuda)
    img, axes = _case(p, 30, 700, cuda)
    out = torch.empty((p.V,) * 3, device=cuda)
    _noalloc(gglib, out, img, ker, axes, p)  # the first call in the context may load the module
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        _noalloc(gglib, out, img, ker, axes, p)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_volumes_beyond_the_scratch(cuda, gglib):
    import torch

    V, M = 162, 162  # 162^3 > 4,194,304
    out = torch.zeros((V,) * 3, device=cuda)
    img = torch.zeros((2, M, M), device=cuda)
    ker = _dev(O.Params(16).ker, cuda)
    axes = _dev(O.create_uniform_axes(2, 1)[:2], cuda)
    rc = gglib.gg_back_project_normalized_noalloc(_vp(out), _vp(img), _vp(ker), _vp(axes), 2.0, 2, V, M, 70, 501,
                                                  None)
    assert rc == 1  # GG_ERR_INVALID_ARG
    assert b"4,194,304" in gglib.gg_global_error()
