"""The serving loop (gg_server_*): results of a mix of forward and back
requests on resident volumes of two sizes, submitted all at once so that they
overlap, equal the same requests run one at a time bit for bit, and equal the
plain gridder calls (gg_forward_project, gg_back_project + gg_get_cas_volume)
within relative L2 1e-6 (cuFFT may pick other kernels for other batch
sizes).  Admission by footprint: a request larger than the HBM budget fails
with GG_ERR_OUT_OF_MEMORY, and a budget that fits one request at a time runs
them one at a time.  Chunked scheduling: requests split into chunks that
interleave across lanes give the same results; short requests overtake a long
one between its chunks; a backlog bound refuses submissions with GG_ERR_BUSY."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _requests(vols, seed, count=24):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        vid = list(vols)[k % len(vols)]
        N = vols[vid].shape[0]
        n = int(np.exp(rng.uniform(np.log(1), np.log(300))))
        op = "back" if rng.random() < 0.5 else "forward"
        axes = O.quaternion_axes(n, seed * 1000 + k).astype(np.float32)
        imgs = rng.standard_normal((n, N, N)).astype(np.float32) if op == "back" else None
        reqs.append((vid, op, axes, imgs))
    return reqs


def _plain(L, vol, op, axes, imgs):
    N = vol.shape[0]
    h = ctypes.c_void_p()
    dev = (ctypes.c_int * 1)(0)
    assert L.gg_create(N, 0, ctypes.c_float(2.0), 3, 1, dev, 1, 0, ctypes.byref(h)) == 0
    dims = (ctypes.c_int * 3)(N, N, N)
    n = len(axes)
    try:
        if op == "forward":
            assert L.gg_set_volume(h, vol.ctypes.data, dims) == 0
            out = np.empty((n, N, N), np.float32)
            assert L.gg_forward_project(h, axes.ctypes.data, n, out.ctypes.data, None) == 0
        else:
            Nn, M, V, R = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            L.gg_get_sizes(h, ctypes.byref(Nn), ctypes.byref(M), ctypes.byref(V), ctypes.byref(R))
            assert L.gg_back_project(h, axes.ctypes.data, n, imgs.ctypes.data, None, 0) == 0
            out = np.empty((V.value,) * 3, np.float32)
            assert L.gg_get_cas_volume(h, out.ctypes.data) == 0
    finally:
        L.gg_destroy(h)
    return out


def test_mix_equals_alone_and_plain_path(cuda, gglib):
    from multigpugridder_gb300.serve import Server

    vols = {}
    with Server(lanes=4) as srv:
        for N, seed in ((16, 61), (24, 62)):
            v = O.blob_volume(N, 6, seed=seed).astype(np.float32)
            vols[srv.add_volume(v)] = v
        reqs = _requests(vols, seed=63)
        # all at once: they overlap on the lanes
        handles = [srv.submit(vid, op, axes, imgs) for vid, op, axes, imgs in reqs]
        mixed = [srv.wait(h)[0].copy() for h in handles]
        st = srv.stats()
        assert st["completed"] == len(reqs)
        assert st["peak_inflight"] > 1
        # one at a time
        alone = []
        for vid, op, axes, imgs in reqs:
            alone.append(srv.wait(srv.submit(vid, op, axes, imgs))[0].copy())
    for (vid, op, axes, imgs), a, b in zip(reqs, mixed, alone):
        assert np.array_equal(a, b), (op, len(axes))
        assert np.all(np.isfinite(a))
    for k in (0, 1, 2, 3, 5, 8):
        vid, op, axes, imgs = reqs[k]
        ref = _plain(gglib, vols[vid], op, axes, imgs)
        assert O.rel_l2(mixed[k], ref) < 1e-6, (op, len(axes))


def test_admission_by_footprint(cuda):
    from multigpugridder_gb300 import _lib
    from multigpugridder_gb300._lib import GridderError
    from multigpugridder_gb300.serve import Server

    v = O.blob_volume(24, 6, seed=64).astype(np.float32)
    axes = O.quaternion_axes(64, 65).astype(np.float32)
    imgs = np.random.default_rng(66).standard_normal((64, 24, 24)).astype(np.float32)
    # a budget that holds the volume and one back request (~3.5 MB), not two
    with Server(hbm_budget_gb=0.0045, lanes=4) as srv:
        vid = srv.add_volume(v)
        hs = [srv.submit(vid, "back", axes, imgs) for _ in range(4)]
        outs = [srv.wait(h)[0].copy() for h in hs]
        assert srv.stats()["peak_inflight"] == 1
        for o in outs[1:]:
            assert np.array_equal(o, outs[0])
        big = srv.submit(vid, "back", O.quaternion_axes(4096, 67).astype(np.float32),
                         np.zeros((4096, 24, 24), np.float32))
        with pytest.raises(GridderError) as e:
            srv.wait(big)
        assert e.value.code == _lib.GG_ERR_OUT_OF_MEMORY
        # the server keeps serving
        out, _ = srv.wait(srv.submit(vid, "forward", axes[:5]))
        assert out.shape == (5, 24, 24) and np.all(np.isfinite(out))


def test_large_volume_equals_plain_path(cuda, gglib):
    """A 256^3 volume (CAS images of 512^2: the serving loop's back projection
    with 8-deep warp blocks and one brick group per CTA): a back and a forward
    request equal the plain gridder calls within relative L2 1e-6."""
    from multigpugridder_gb300.serve import Server

    N = 256
    v = O.blob_volume(N, 40, seed=71).astype(np.float32)
    axes = O.quaternion_axes(5, 72).astype(np.float32)
    imgs = np.random.default_rng(73).standard_normal((len(axes), N, N)).astype(np.float32)
    with Server(lanes=2) as srv:
        vid = srv.add_volume(v)
        back = srv.wait(srv.submit(vid, "back", axes, imgs))[0].copy()
        fwd = srv.wait(srv.submit(vid, "forward", axes))[0].copy()
    assert O.rel_l2(back, _plain(gglib, v, "back", axes, imgs)) < 1e-6
    assert O.rel_l2(fwd, _plain(gglib, v, "forward", axes, None)) < 1e-6


def test_chunked_mix_equals_alone_and_plain_path(cuda, gglib):
    """A quantum small enough that every request runs in chunks of 16
    directions, whose chunks of different requests interleave across the
    lanes: the mix equals the same requests one at a time bit for bit, and the
    plain gridder calls within relative L2 1e-6 (a chunked back projection sums
    its chunks' sums in another grouping)."""
    from multigpugridder_gb300.serve import Server

    vols = {}
    with Server(lanes=3, quantum_ms=1e-6) as srv:
        for N, seed in ((16, 81), (24, 82)):
            v = O.blob_volume(N, 6, seed=seed).astype(np.float32)
            vols[srv.add_volume(v)] = v
        reqs = _requests(vols, seed=83, count=16)
        assert max(len(a) for _, _, a, _ in reqs) > 64
        handles = [srv.submit(vid, op, axes, imgs) for vid, op, axes, imgs in reqs]
        mixed = [srv.wait(h)[0].copy() for h in handles]
        assert srv.stats()["peak_inflight"] > 1
        alone = [srv.wait(srv.submit(vid, op, axes, imgs))[0].copy() for vid, op, axes, imgs in reqs]
    for (vid, op, axes, imgs), a, b in zip(reqs, mixed, alone):
        assert np.array_equal(a, b), (op, len(axes))
    for k, (vid, op, axes, imgs) in enumerate(reqs):
        if len(axes) > 32:
            ref = _plain(gglib, vols[vid], op, axes, imgs)
            assert O.rel_l2(mixed[k], ref) < 1e-6, (op, len(axes))


def test_short_requests_overtake_a_long_one(cuda):
    """One lane, a long request submitted first and short ones after it: the
    long request runs in chunks and the short ones, with less work left, take
    the lane between its chunks and finish first."""
    from multigpugridder_gb300.serve import Server

    v = O.blob_volume(32, 6, seed=84).astype(np.float32)
    long_axes = O.quaternion_axes(2048, 85).astype(np.float32)
    short_axes = O.quaternion_axes(16, 86).astype(np.float32)
    with Server(lanes=1, quantum_ms=0.01) as srv:
        vid = srv.add_volume(v)
        srv.wait(srv.submit(vid, "forward", short_axes))  # plans and kernels warm
        big = srv.submit(vid, "forward", long_axes)
        small = [srv.submit(vid, "forward", short_axes) for _ in range(8)]
        lat_small = [srv.wait(h)[1] for h in small]
        lat_big = srv.wait(big)[1]
        ref = srv.wait(srv.submit(vid, "forward", short_axes))[0].copy()
    assert max(lat_small) < lat_big, (lat_small, lat_big)
    assert np.all(np.isfinite(ref))


def test_backlog_bound_sheds_load(cuda):
    """With a bound on the queued work, submissions beyond it fail with
    GG_ERR_BUSY at once, every accepted request completes, and the server
    keeps serving."""
    from multigpugridder_gb300 import _lib
    from multigpugridder_gb300._lib import GridderError
    from multigpugridder_gb300.serve import Server

    v = O.blob_volume(32, 6, seed=87).astype(np.float32)
    axes = O.quaternion_axes(512, 88).astype(np.float32)
    with Server(lanes=1, max_backlog_s=1e-6) as srv:
        vid = srv.add_volume(v)
        ok, busy = [], 0
        for _ in range(64):
            try:
                ok.append(srv.submit(vid, "forward", axes))
            except GridderError as e:
                assert e.code == _lib.GG_ERR_BUSY
                busy += 1
        assert busy > 0 and ok
        assert srv.load()["rejected"] == busy
        outs = [srv.wait(h)[0] for h in ok]
        for o in outs[1:]:
            assert np.array_equal(o, outs[0])
        srv.set_max_backlog(0)
        out, _ = srv.wait(srv.submit(vid, "forward", axes[:5]))
        assert np.array_equal(out, outs[0][:5])


def test_default_quantum_chunks_equal_plain_path(cuda, gglib):
    """A 64^3 volume (CAS images of 128^2) with the default quantum: a
    1,500-direction back request runs as chunks of 1,024 and 476 directions,
    a forward request as chunks too, beside short requests; both equal the
    plain gridder calls within relative L2 1e-6 and the same requests alone
    bit for bit."""
    from multigpugridder_gb300.serve import Server

    N = 64
    v = O.blob_volume(N, 20, seed=91).astype(np.float32)
    axes = O.quaternion_axes(1500, 92).astype(np.float32)
    imgs = np.random.default_rng(93).standard_normal((len(axes), N, N)).astype(np.float32)
    with Server(lanes=4) as srv:
        vid = srv.add_volume(v)
        hb = srv.submit(vid, "back", axes, imgs)
        hf = srv.submit(vid, "forward", axes)
        hs = [srv.submit(vid, "forward", axes[k * 16:(k + 1) * 16]) for k in range(8)]
        back = srv.wait(hb)[0].copy()
        fwd = srv.wait(hf)[0].copy()
        for h in hs:
            srv.wait(h)
        back_alone = srv.wait(srv.submit(vid, "back", axes, imgs))[0].copy()
    assert np.array_equal(back, back_alone)
    assert O.rel_l2(back, _plain(gglib, v, "back", axes, imgs)) < 1e-6
    assert O.rel_l2(fwd, _plain(gglib, v, "forward", axes, None)) < 1e-6
