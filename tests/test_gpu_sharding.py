"""reconstruct_sharded with the library's CUDA backend on one rank (no
process group): the back projections of the images and of all-ones CAS images,
the division and getVol give gg_reconstruct_volume's volume within relative L2
1e-6 (the fused kernel forms the same two sums in one pass)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_sharded_reconstruct_single_rank_equals_reconstruct_volume(cuda):
    import torch

    import multigpugridder_gb300 as gg
    from multigpugridder_gb300.sharding import GridderBackend, reconstruct_sharded

    N = 32
    axes = O.quaternion_axes(60, 91).astype(np.float32)
    imgs = np.random.default_rng(92).standard_normal((60, N, N)).astype(np.float32)
    g = gg.MultiGPUGridder(N, 60, 2.0, adjustInterpFactor=False)
    got = reconstruct_sharded(GridderBackend(g), axes, imgs).cpu().numpy()
    torch.cuda.synchronize()
    ref = np.empty((N, N, N), np.float32)
    L = gg.lib()
    assert L.gg_reconstruct_volume(g.handle, axes.ctypes.data, 60, imgs.ctypes.data, ref.ctypes.data) == 0
    g.close()
    assert np.all(np.isfinite(got))
    assert O.rel_l2(got, ref) < 1e-6
