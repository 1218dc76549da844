"""Python face of the serving loop (gg_server_* in include/gg_gridder.h).

    srv = Server(lanes=8)
    vid = srv.add_volume(volume_np, interp=2.0)          # CAS volume prepared once, resident
    req = srv.submit(vid, "forward", axes)               # returns at once
    images, latency_ms = srv.wait(req)                   # n x N x N

A back request returns the V^3 CAS volume of its images back-projected into
zeros.  Requests run in chunks of about `quantum_ms` of device time on `lanes`
lanes; a free lane takes the chunk of the request with the least work left, and
a request starts once its device buffers fit the HBM budget, so requests that
arrive while others run overlap with them and short ones overtake long ones.
With `max_backlog_s` set, a submission beyond that much queued work raises
GridderError with code GG_ERR_BUSY.  For copies that overlap, pass pinned host
buffers (`pinned_empty`).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import GG_OK, GridderError

OPS = {"forward": _lib.GG_OP_FORWARD, "back": _lib.GG_OP_BACK}


def pinned_empty(shape):
    """A pinned (page-locked) float32 host array, through torch's allocator."""
    import torch

    t = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    return t.numpy()


class Request:
    __slots__ = ("id", "op", "out", "_keep")

    def __init__(self, rid, op, out, keep):
        self.id = rid
        self.op = op
        self.out = out
        self._keep = keep


class Server:
    def __init__(self, device=0, hbm_budget_gb=0.0, lanes=8, quantum_ms=None, max_backlog_s=None):
        self._L = _lib.lib()
        h = ctypes.c_void_p()
        rc = self._L.gg_server_create(int(device), float(hbm_budget_gb), int(lanes), ctypes.byref(h))
        if rc != GG_OK:
            raise GridderError(rc, self._L.gg_global_error().decode(errors="replace"))
        self._h = h
        self._sizes = {}
        if quantum_ms is not None:
            self.set_quantum(quantum_ms)
        if max_backlog_s is not None:
            self.set_max_backlog(max_backlog_s)

    def set_quantum(self, quantum_ms):
        """Estimated device time of one chunk, for requests submitted afterwards."""
        self._check(self._L.gg_server_set_quantum(self._h, float(quantum_ms)))

    def set_max_backlog(self, seconds):
        """Refuse submissions (GG_ERR_BUSY) beyond this much queued work; 0: no bound."""
        self._check(self._L.gg_server_set_max_backlog(self._h, float(seconds)))

    def load(self):
        """Requests queued and admitted, seconds of queued work, submissions refused."""
        q, a, r = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        sec = ctypes.c_double()
        self._check(self._L.gg_server_load(self._h, ctypes.byref(q), ctypes.byref(a), ctypes.byref(sec),
                                           ctypes.byref(r)))
        return {"queued": q.value, "active": a.value, "queued_seconds": sec.value, "rejected": r.value}

    def _check(self, rc):
        if rc != GG_OK:
            raise GridderError(rc, (self._L.gg_server_last_error(self._h) or b"").decode(errors="replace"))

    def close(self):
        if getattr(self, "_h", None):
            self._L.gg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_volume(self, volume, interp=2.0):
        """volume: N^3 float32 (numpy on the host, or a CUDA torch tensor)."""
        vid = ctypes.c_int()
        if hasattr(volume, "is_cuda") and volume.is_cuda:
            v = volume.detach().contiguous().float()
            self._check(self._L.gg_server_add_volume(self._h, v.data_ptr(), v.shape[0], float(interp), 1,
                                                     ctypes.byref(vid)))
        else:
            v = np.ascontiguousarray(volume, dtype=np.float32)
            self._check(self._L.gg_server_add_volume(self._h, v.ctypes.data, v.shape[0], float(interp), 0,
                                                     ctypes.byref(vid)))
        N, M, V = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self._L.gg_server_volume_sizes(self._h, vid.value, ctypes.byref(N), ctypes.byref(M),
                                                   ctypes.byref(V)))
        self._sizes[vid.value] = (N.value, M.value, V.value)
        return vid.value

    def remove_volume(self, vid):
        self._check(self._L.gg_server_remove_volume(self._h, int(vid)))
        self._sizes.pop(vid, None)

    def sizes(self, vid):
        """(N, M, V) of a resident volume."""
        return self._sizes[vid]

    def submit(self, vid, op, axes, images=None, out=None):
        """Queue a request; `out` (optional) receives the result."""
        code = OPS[op]
        N, _, V = self._sizes[vid]
        ax = np.ascontiguousarray(axes, dtype=np.float32).reshape(-1)
        n = ax.size // 9
        keep = [ax]
        img_ptr = None
        if code == _lib.GG_OP_BACK:
            im = np.ascontiguousarray(images, dtype=np.float32)
            if im.size != n * N * N:
                raise ValueError("images must hold n*N*N floats")
            keep.append(im)
            img_ptr = im.ctypes.data
            shape = (V, V, V)
        else:
            shape = (n, N, N)
        if out is None:
            out = np.empty(shape, dtype=np.float32)
        elif out.size != int(np.prod(shape)) or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array of %d elements" % int(np.prod(shape)))
        rid = ctypes.c_longlong()
        self._check(self._L.gg_server_submit(self._h, int(vid), code, ax.ctypes.data if n else None, n, img_ptr,
                                             out.ctypes.data, ctypes.byref(rid)))
        return Request(rid.value, op, out.reshape(shape), keep)

    def wait(self, req, timeout=-1.0):
        """(result, latency in ms from submission to completion)."""
        lat = ctypes.c_double()
        self._check(self._L.gg_server_wait(self._h, req.id, float(timeout), ctypes.byref(lat)))
        req._keep = None
        return req.out, lat.value

    def stats(self):
        c, mx = ctypes.c_longlong(), ctypes.c_longlong()
        p50, p99, mean, gb = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self._L.gg_server_stats(self._h, ctypes.byref(c), ctypes.byref(p50), ctypes.byref(p99),
                                            ctypes.byref(mean), ctypes.byref(mx), ctypes.byref(gb)))
        return {"completed": c.value, "p50_ms": p50.value, "p99_ms": p99.value, "mean_ms": mean.value,
                "peak_inflight": mx.value, "peak_gb": gb.value}

    def reset_stats(self):
        self._check(self._L.gg_server_reset_stats(self._h))
