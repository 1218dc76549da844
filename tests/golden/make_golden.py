"""Generates the committed fixtures under tests/golden/.

  python tests/golden/make_golden.py tables      # kb_precomp.npz (CPU)
  python tests/golden/make_golden.py reference   # reference_kernels.npz (GPU)

kb_precomp.npz holds the FP32 KB lookup table the reference hands to its
kernels (single(getKernelFiltTable(2, 501)), MultiGPUGridder_Matlab_Class.m:128)
and the FP64 pre-compensation vectors for M = 64, 128, 256, from the oracle.

reference_kernels.npz holds inputs and the outputs of the reference's OWN
kernels -- gpuForwardProjectKernel and gpuBackProjectKernel compiled unmodified
from tagarelab/MultiGPUGridder's sources into oracle/_ref/*.cubin and launched
with their RunKernel geometry by oracle/ref_kernels.py -- on small seeded
cases.  It must be generated on a GPU (the GB300 machine); the inputs are stored
with the outputs so the CPU test replays exactly the same bits.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def make_tables(out_dir=HERE):
    d = {"kb_table_f32": O.kb_table(2, 501).astype(np.float32)}
    for M in (64, 128, 256):
        d["precomp_%d" % M] = O.precomp(M, 2)
    np.savez(os.path.join(out_dir, "kb_precomp.npz"), **d)


def golden_cases():
    """Small seeded cases: a realistic CAS volume (blob volume) with random
    quaternion directions, and full-frame random CAS images with the
    reference's own axis grid (exact 0.5 entries; row-wrapping windows)."""
    cases = {}
    for key, N, seed in (("n16a", 16, 1), ("n16b", 16, 2)):
        p = O.Params(N)
        rng = np.random.default_rng(seed)
        vol = O.blob_volume(N, 6, seed=seed)
        cas = O.cas_from_vol(vol).astype(np.float32)
        if key.endswith("a"):
            axes = O.quaternion_axes(10, seed=seed + 10)
        else:
            axes = O.create_uniform_axes(2, 5)
        axes = np.ascontiguousarray(axes, dtype=np.float32)
        img = rng.standard_normal((len(axes), p.M, p.M)).astype(np.float32)
        cases[key] = {"N": N, "cas": cas, "axes": axes, "img": img, "ker": p.ker,
                      "mask_radius": p.mask_radius, "M": p.M, "V": p.V}
    return cases


def make_reference(out_path):
    import torch

    from oracle.ref_kernels import RefKernels

    dev = torch.device("cuda:0")
    torch.cuda.init()
    rk = RefKernels()
    out = {}
    for key, c in golden_cases().items():
        d_cas = torch.from_numpy(c["cas"]).to(dev)
        d_ax = torch.from_numpy(c["axes"]).to(dev)
        d_ker = torch.from_numpy(c["ker"]).to(dev)
        d_img = torch.from_numpy(c["img"]).to(dev)
        fp = torch.zeros((len(c["axes"]), c["M"], c["M"]), device=dev)
        rk.forward_project(d_cas.data_ptr(), c["V"], fp.data_ptr(), c["M"], d_ax.data_ptr(), len(c["axes"]),
                           c["mask_radius"], d_ker.data_ptr(), c["ker"].size)
        bp = torch.zeros((c["V"],) * 3, device=dev)
        rk.back_project(bp.data_ptr(), c["V"], d_img.data_ptr(), c["M"], d_ax.data_ptr(), len(c["axes"]),
                        c["mask_radius"], d_ker.data_ptr(), c["ker"].size)
        torch.cuda.synchronize()
        for name in ("cas", "axes", "img", "ker"):
            out["%s_%s" % (key, name)] = c[name]
        out[key + "_meta"] = np.array([c["N"], c["M"], c["V"], c["mask_radius"]], np.int32)
        out[key + "_fp"] = fp.cpu().numpy()
        out[key + "_bp"] = bp.cpu().numpy()
    np.savez_compressed(out_path, **out)
    return out_path


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "tables"
    if what == "tables":
        make_tables()
    elif what == "reference":
        dst = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, "reference_kernels.npz")
        print(make_reference(dst))
    else:
        raise SystemExit("usage: make_golden.py tables|reference [out.npz]")
