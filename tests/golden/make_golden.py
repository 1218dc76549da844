"""Generates the committed fixtures under tests/golden/.

  python tests/golden/make_golden.py tables      # kb_precomp.npz (CPU)
  python tests/golden/make_golden.py reference   # reference_kernels.npz (GPU)
  python tests/golden/make_golden.py filters     # reference_filters.npz (GPU)

reference_filters.npz holds small seeded inputs and the outputs of the
reference's own filter kernels (src/Filters/*Filter.cu, compiled unmodified
into oracle/_ref/ and launched with their UpdateFilter geometry by
oracle/ref_kernels.py: RefFilters), and of its two image-stage chains
(gpuGridder::CASImgsToImgs / ::ImgsToCASImgs, gpuGridder.cpp:432-596:
those filters and one cuFFT C2C per image).  It must be generated on a GPU.

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


def make_filters(out_path):
    import torch

    from oracle.ref_kernels import RefFilters

    dev = torch.device("cuda:0")
    torch.cuda.init()
    rf = RefFilters()
    rng = np.random.default_rng(77)
    out = {}

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)

    def put(name, x):
        torch.cuda.synchronize()
        out[name] = x.cpu().numpy() if hasattr(x, "cpu") else x

    S, NS = 8, 3
    c2 = rng.standard_normal((NS, S, S, 2)).astype(np.float32)
    r2 = rng.standard_normal((NS, S, S)).astype(np.float32)
    r3 = rng.standard_normal((S, S, S)).astype(np.float32)
    out.update(c2=c2, r2=r2, r3=r3)
    y = torch.zeros((NS, S, S), device=dev)
    rf.complex_to_cas(t(c2).data_ptr(), y.data_ptr(), S, NS)
    put("complex_to_cas_2d", y)
    y = torch.zeros((NS, S, S, 2), device=dev)
    rf.cas_to_complex(t(r2).data_ptr(), y.data_ptr(), S, NS)
    put("cas_to_complex_2d", y)
    y = torch.zeros((S, S, S, 2), device=dev)
    rf.cas_to_complex(t(r3).data_ptr(), y.data_ptr(), S, 0)
    put("cas_to_complex_3d", y)
    for nm, a, cplx in (("fftshift_2d_real", r2, False), ("fftshift_2d_complex", c2, True)):
        x = t(a)
        rf.fftshift_2d(x.data_ptr(), S, NS, cplx)
        put(nm, x)
    x = t(r3)
    rf.fftshift_3d(x.data_ptr(), S, False)
    put("fftshift_3d_real", x)
    pin = rng.standard_normal((2, 5, 6)).astype(np.float32)
    out["pad_in"] = pin
    y = torch.zeros((2 + 2, 5 + 4, 6 + 2), device=dev)
    rf.pad_volume(t(pin).data_ptr(), y.data_ptr(), 6, 5, 2, 1, 2, 1)
    put("pad_out", y)
    cin = rng.standard_normal((6, 9, 10)).astype(np.float32)
    out["crop_in"] = cin
    y = torch.zeros((6 - 2, 9 - 4, 10 - 2), device=dev)
    rf.crop_volume(t(cin).data_ptr(), y.data_ptr(), 10, 9, 6, 1, 2, 1)
    put("crop_out", y)
    a = rng.standard_normal((NS, S, S)).astype(np.float32)
    b = rng.standard_normal((NS, S, S)).astype(np.float32)
    a[rng.random(a.shape) < 0.2] = 0.0
    b[rng.random(b.shape) < 0.2] = 0.0
    out.update(arith_a=a, arith_b=b)
    for nm, fn in (("divide", lambda x: rf.divide_volumes(x.data_ptr(), t(b).data_ptr(), S, NS)),
                   ("multiply", lambda x: rf.multiply_volumes(x.data_ptr(), t(b).data_ptr(), S, NS, False)),
                   ("add", lambda x: rf.add_volumes(x.data_ptr(), t(b).data_ptr(), S, NS)),
                   ("divide_scalar", lambda x: rf.divide_scalar(x.data_ptr(), 3.0, S, NS))):
        x = t(a)
        fn(x)
        put(nm, x)
    x = t(c2)
    rf.multiply_volumes(x.data_ptr(), t(b).data_ptr(), S, NS, True)
    put("multiply_complex", x)
    y = torch.zeros((NS, S, S, 2), device=dev)
    rf.real_to_complex(t(r2).data_ptr(), y.data_ptr(), S, NS)
    put("real_to_complex", y)
    y = torch.zeros((NS, S, S), device=dev)
    rf.complex_to_real(t(c2).data_ptr(), y.data_ptr(), S, NS)
    put("complex_to_real", y)
    # the image stages: CAS images of edge M = 32 <-> images of edge N = 16
    M, N, n = 32, 16, 3
    cas = rng.standard_normal((n, M, M)).astype(np.float32)
    imgs = rng.standard_normal((n, N, N)).astype(np.float32)
    out.update(chain_cas_in=cas, chain_imgs_in=imgs)
    w = t(cas)
    y = torch.zeros((n, N, N), device=dev)
    cx = torch.zeros((n, M, M, 2), device=dev)
    rf.cas_imgs_to_imgs(w.data_ptr(), y.data_ptr(), cx.data_ptr(), M, N, n, 2.0)
    put("chain_imgs_out", y)
    y = torch.zeros((n, M, M), device=dev)
    cx = torch.zeros((n, M, M, 2), device=dev)
    rf.imgs_to_cas_imgs(t(imgs).data_ptr(), y.data_ptr(), cx.data_ptr(), M, N, n)
    put("chain_cas_out", y)
    np.savez_compressed(out_path, **out)
    return out_path


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "tables"
    if what == "tables":
        make_tables()
    elif what == "reference":
        dst = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, "reference_kernels.npz")
        print(make_reference(dst))
    elif what == "filters":
        dst = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, "reference_filters.npz")
        print(make_filters(dst))
    else:
        raise SystemExit("usage: make_golden.py tables|reference|filters [out.npz]")
