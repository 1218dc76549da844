#!/usr/bin/env python
"""Benchmark: forward + back projections per second at 128^3, interpFactor 2.

Workload (one step): a seeded 128^3 Gaussian-blob volume (100 blobs) and
10,000 directions on a 100 x 100 azimuth x cos-polar grid.  setVolume (CAS
volume prepared on the device) -> forwardProject to 10,000 128^2 images ->
reconstructVol of those images (back projection of the images, back
projection of all-ones CAS images for the plane density, division, getVol).
One step = 10,000 forward+back projection pairs.

  value   device-resident inputs, timed with CUDA events on the stream the
          library runs on (*_dev entry points), L2 flushed between steps.
  e2e     the same step through the host-pointer C ABI with pinned host
          buffers: volume and axes in, 10,000 images out, images back in,
          volume out -- every host<->device copy inside the timed region.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "fwd+back projections/s at 128^3 x interp 2 (10,000 directions)"
UNIT = "projection pairs/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="f32", choices=["f32", "f16", "bf16"])
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--directions", type=int, default=10000)
    ap.add_argument("--batch", type=int, default=2000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=1024,
                    help="directions timed by the CPU baseline / reference arm per step (one core: 1/8 of it)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="arrival window of the serving workload (0: skip it)")
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="offered requests/s (Poisson)")
    ap.add_argument("--serve-lanes", type=int, default=8)
    ap.add_argument("--serve-closed", type=int, default=200,
                    help="requests in the closed-loop served vs sequential plain-path comparison")
    ap.add_argument("--serve-repeats", type=int, default=5, help="repeats of the closed-loop comparison")
    ap.add_argument("--serve-quantum-ms", type=float, default=8.0,
                    help="estimated device time of one chunk of a served request")
    ap.add_argument("--serve-backlog", type=float, default=2.0,
                    help="queued work (estimated seconds) beyond which the offered-rate run sheds arrivals")
    ap.add_argument("--serve-legs", default="closed,offered,load70",
                    help="serving runs: closed (served vs sequential), offered (the offered rate), "
                         "load70 (70%% of the capacity the offered run measured, or of --serve-capacity)")
    ap.add_argument("--serve-capacity", type=float, default=0.0,
                    help="requests/s taken as the capacity when the offered run is not among the legs")
    ap.add_argument("--no-precision", action="store_true", help="skip the 256^3 storage-precision comparison")
    ap.add_argument("--no-autograd", action="store_true", help="skip the gradient-descent timing")
    ap.add_argument("--no-ctf", action="store_true", help="skip the CTF-corrected reconstruction timing")
    return ap.parse_args()


def workload(args, rank=0, world=1):
    """The volume and this rank's directions.  One GPU: the 100 x 100 grid
    (in-plane angle 30 degrees).  World W > 1 (weak scaling): W x 10,000
    directions, shard r being the same grid turned in-plane by 360 r / W
    degrees more."""
    from multigpugridder_gb300 import synthetic

    N = args.size
    n_blobs = {64: 20, 128: 100, 256: 400}.get(N, max(10, N // 2))
    vol = synthetic.blob_volume(N, n_blobs, seed=2)
    side = int(round(args.directions ** 0.5))
    if side * side == args.directions:
        axes = synthetic.grid_axes(side, side, psi_deg=30.0 + 360.0 * rank / world).astype(np.float32)
    else:
        axes = synthetic.quaternion_axes(args.directions, seed=2 + rank).astype(np.float32)
    return vol, axes


FLUSH_BYTES = 512 << 20  # untimed write between steps: 4x the 126 MB L2

# From a one-launch ncu capture of the fused back projection at 128^3 x 2,
# 1,024 directions per launch (profiles/bp_ref_compact_kernel_density_128cubed_1024dirs.md):
# DRAM bytes (read + write) and L2 bytes (lts__t_bytes) per direction, and the
# fraction of cycles the schedulers issued.
NCU_BP_DRAM_PER_DIR = 545.2e6 / 1024
NCU_BP_LTS_PER_DIR = 5.488e9 / 1024
NCU_BP_ISSUE_ACTIVE = 0.720


def sizes(args):
    """(N, M, V) of the workload: interpFactor 2, extra padding 3."""
    N = args.size
    return N, 2 * N, 2 * N + 6


def bench_config(args, world):
    """The `config` both arms print (the same dict, so the two lines compare)."""
    N, M, V = sizes(args)
    return {"workload": "%d^3 volume, interpFactor 2 (CAS volume %d^3, CAS images %d^2), %d directions: "
                        "setVolume + forwardProject + reconstructVol" % (N, V, M, args.directions),
            "N": N, "M": M, "V": V, "directions": args.directions, "batch": args.batch,
            "precision": args.precision,
            "parallelism": ("orientation shards x%d, one all-reduce" % world) if world > 1 else "single",
            "l2": "inputs larger than L2 (%d images = %d MB per step) and an untimed %d MB write between steps"
                  % (args.directions, args.directions * N * N * 4 >> 20, FLUSH_BYTES >> 20)}


def p_in(M, R):
    c = M // 2
    i = np.arange(M) - c
    return int(np.sum((i[:, None] ** 2 + i[None, :] ** 2) <= R * R))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(vol, axes, args, threads=None, sample=None):
    """One CPU step of the restated reference path on a bounded sample of the
    directions; returns (pairs/s measured on the sample, details, S)."""
    from oracle import cpu_path, oracle as O

    p = O.Params(args.size)
    S = min(sample or args.cpu_sample, len(axes))
    idx = np.linspace(0, len(axes) - 1, S).round().astype(int)
    t, det = cpu_path.time_step(vol, axes[idx], p, len(axes), threads=threads)
    det["t_step_s"] = t
    return S / t, det, S


def run_reference(args):
    """The reference's gridding path on the host cores (the restatement in
    oracle/: the reference has no CPU implementation of it).  Each step is
    setVolume + forwardProject + reconstructVol of a bounded sample of the
    workload's directions (evenly spaced); value = sample directions / the
    measured step time.  The full-workload step it stands for is extrapolated
    and reported apart."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    vol, axes = workload(args)
    times, dets = [], []
    S = 0
    for s in range(args.warmup + args.steps):
        _, det, S = cpu_baseline(vol, axes, args)
        if s >= args.warmup:
            times.append(det["t_step_s"])
            dets.append(det)
    t_step = statistics.mean(times)
    value = S / t_step
    det = dets[-1]
    t_full = statistics.mean(d["t_step_extrapolated_s"] for d in dets)
    cores = det["threads"]
    sample = ("each step: %d of the %d directions (evenly spaced) through the restated reference path: FP32 CAS "
              "prep (scipy.fft), forward-projection kernel, 2-D FFTs, back projection and plane density "
              "(gg_oracle.c, OpenMP), getVol; value = %d / measured step time" % (S, len(axes), S))
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
           "data": "synthetic (seeded Gaussian-blob volume, 100x100 direction grid)",
           "config": bench_config(args, world),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "directions_per_step": S,
           "full_step_extrapolated": {"ms": t_full * 1e3, "value": len(axes) / t_full, "unit": UNIT,
                                      "how": "t_fixed + D/S * t_sample, D = %d" % len(axes)},
           "details": det}
    print(json.dumps(out), flush=True)


def run_gb300(args):
    import torch
    import torch.distributed as dist

    import multigpugridder_gb300 as gg
    from multigpugridder_gb300._lib import (GG_KERNEL_BACK, GG_KERNEL_DENSITY, GG_KERNEL_FORWARD, check, lib)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = lib()

    vol, axes = workload(args, rank, world)
    n = len(axes)
    N = args.size
    g = gg.MultiGPUGridder(N, n, 2.0, GPUs=[local], MaxAxesToAllocate=args.batch, precision=args.precision)
    h = g.handle
    M, V, R = g.M, g.V, int(g.MaskRadius)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    d_vol = torch.from_numpy(np.ascontiguousarray(vol)).to(dev)
    d_axes = torch.from_numpy(np.ascontiguousarray(axes)).to(dev)
    d_imgs = torch.empty((n, N, N), dtype=torch.float32, device=dev)
    d_out = torch.empty((N, N, N), dtype=torch.float32, device=dev)
    d_sums = torch.empty((2, V, V, V), dtype=torch.float32, device=dev) if world > 1 else None
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def vp(t):
        return ctypes.c_void_p(t.data_ptr())

    def step():
        check(L.gg_set_volume_dev(h, vp(d_vol), sp), h)
        check(L.gg_forward_project_dev(h, vp(d_axes), n, vp(d_imgs), None, sp), h)
        if world == 1:
            check(L.gg_reconstruct_volume_dev(h, vp(d_axes), n, vp(d_imgs), vp(d_out), sp), h)
        else:
            # the reference's split (MultiGPUGridder.cpp:37-96, 376-411): this rank's
            # sums, one all-reduce of CAS volume + plane density, division and getVol
            check(L.gg_back_project_sums_dev(h, vp(d_axes), n, vp(d_imgs), vp(d_sums), sp), h)
            dist.all_reduce(d_sums)
            check(L.gg_volume_from_sums_dev(h, vp(d_sums), vp(d_out), sp), h)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
            flush.fill_(1.0)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    check(L.gg_profile_enable(h, 1), h)
    launches0 = L.gg_kernel_launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
            flush.fill_(float(k))  # untimed L2 flush between steps
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches = L.gg_kernel_launch_count() - launches0
    ms_steps = [a.elapsed_time(b) for a, b in ev]
    prof = {}
    for name, kid in (("forward", GG_KERNEL_FORWARD), ("back", GG_KERNEL_BACK), ("density", GG_KERNEL_DENSITY)):
        tot = ctypes.c_double()
        cnt = ctypes.c_longlong()
        check(L.gg_profile_read(h, kid, ctypes.byref(tot), ctypes.byref(cnt)), h)
        prof[name] = (tot.value, cnt.value)
    check(L.gg_profile_enable(h, 0), h)
    clk = clocks.stop()
    from multigpugridder_gb300.sharding import max_over_ranks

    ms = max_over_ranks(sum(ms_steps), device=dev)  # the slowest rank's time
    ms_per_step = ms / args.steps
    value = world * n / (ms_per_step / 1e3)

    # roofline of the dominant kernel: algorithmic bytes per unit (one image)
    #   forward  4*P_in*125 + 4*M^2   (taps gathered + CAS image written)
    #   back     4*P_in*125 + s*M^2   (taps accumulated + CAS image read)
    #   density  4*P_in*125           (all-ones images are not read)
    # reconstructVol runs back projection and plane density in one fused
    # kernel (no separate density launches): both volumes are accumulated.
    s = 4 if args.precision == "f32" else 2
    pin = p_in(M, R)
    fused = prof["density"][1] == 0
    bpu = {"forward": s * pin * 125 + 4 * M * M,
           "back": (2 if fused else 1) * 4 * pin * 125 + s * M * M, "density": 4 * pin * 125}
    dom = max(prof, key=lambda k: prof[k][0])
    tot_ms, cnt = prof[dom]
    units_per_launch = n * args.steps / max(cnt, 1)
    achieved = bpu[dom] * units_per_launch / (tot_ms / max(cnt, 1) / 1e3) / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs") or 6800.0
    # the L2 read bandwidth of this GPU, measured here (the bound SURVEY-style
    # accounting names for 128^3: the 72 MB CAS volume stays in the 126 MB L2)
    l2 = ctypes.c_double()
    check(L.gg_measure_l2_read_gbs(10, ctypes.byref(l2)))
    # per-launch DRAM and L2 bytes of the dominant kernel from one-launch ncu
    # captures of this workload (profiles/), scaled by directions per launch
    traffic = lts = issue = None
    if dom == "back" and fused and N == 128 and args.precision == "f32":
        traffic = NCU_BP_DRAM_PER_DIR * units_per_launch
        lts = NCU_BP_LTS_PER_DIR * units_per_launch
        issue = NCU_BP_ISSUE_ACTIVE
    roofline = {"bound": "l2", "kernel": dom, "achieved": achieved, "peak": l2.value, "unit": "GB/s",
                "frac": achieved / l2.value, "peak_source": "measured in this run (gg_measure_l2_read_gbs, best of 10)",
                "traffic": traffic, "lts_bytes": lts, "bytes_per_unit": bpu[dom], "units_per_launch": units_per_launch,
                "hbm": {"peak": hbm, "frac": achieved / hbm,
                        "peak_source": "measured (MEASURED_PEAKS.json)" if peaks.get("hbm_gbs") else "fallback"},
                "issue_active": issue,
                "kernel_ms": {k: v[0] / args.steps for k, v in prof.items()}}

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, g, vol, axes, world, dev)

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, det, S = cpu_baseline(vol, axes, args)
        base = {"value": v, "unit": UNIT, "cores": det["threads"], "kind": "port",
                "sample": "one step of setVolume + forwardProject + reconstructVol on %d of the %d directions "
                          "(evenly spaced); value = %d / measured step time" % (S, n, S),
                "full_step_extrapolated": n / det["t_step_extrapolated_s"]}
        # the same port on one core, on a smaller sample
        v1, _, S1 = cpu_baseline(vol, axes, args, threads=1, sample=max(1, args.cpu_sample // 8))
        base["one_core"] = {"value": v1, "cores": 1,
                            "sample": "one step on %d of %d directions, one thread" % (S1, n)}

    g.close()
    serve = prec = grad = ctf = None
    if rank == 0 and world == 1 and args.serve_seconds > 0:
        serve = run_serve(args)
    prec128 = None
    if rank == 0 and world == 1 and not args.no_precision and args.size == 128:
        prec, keep = run_precision(args, "256")
        prec128, keep128 = run_precision(args, "128")
        if not args.no_cpu_baseline:
            # CPU leg: the FP64 oracle as the checker of the reduced-precision results
            prec["vs_f64"] = check_precision_vs_f64(keep, "256")
            prec128["vs_f64"] = check_precision_vs_f64(keep128, "128")
        del keep, keep128
    if rank == 0 and world == 1 and not args.no_autograd and args.size == 128:
        grad = run_autograd(args)
    if rank == 0 and world == 1 and not args.no_ctf:
        ctf = run_ctf(args, vol, axes)
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": args.precision,
               "data": "synthetic (seeded Gaussian-blob volume, 100x100 direction grid)",
               "config": bench_config(args, world),
               "roofline": roofline, "cpu_baseline": base, "e2e": e2e, "gpu_launches": launches,
               "clocks": clk, "step_ms": ms_steps, "serve": serve, "precision": prec, "precision_128": prec128,
               "autograd": grad,
               "ctf": ctf}
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---- serving workload ---------------------------------------------------------
SERVE_SIZES = (64, 128, 192, 256)
SERVE_WEIGHTS = (0.4, 0.3, 0.2, 0.1)
SERVE_BLOBS = (20, 100, 200, 400)


def serve_schedule(seconds, rate, seed=5, count=None):
    """(arrival s, size index, op, directions, request seed): Poisson arrivals,
    sizes 64/128/192/256 with weights .4/.3/.2/.1, forward/back 50/50,
    directions log-uniform in 16..4096."""
    rng = np.random.default_rng(seed)
    out, t, k = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if (count is None and t >= seconds) or (count is not None and k >= count):
            break
        si = int(rng.choice(4, p=SERVE_WEIGHTS))
        op = "forward" if rng.random() < 0.5 else "back"
        n = int(np.exp(rng.uniform(np.log(16), np.log(4096))))
        out.append((t, si, op, n, 1000 + k))
        k += 1
    return out


def run_serve(args):
    """Open-loop Poisson serving at the offered rate and at 70% of the
    measured capacity, and a closed-loop comparison with sequential
    plain-path calls (gg_forward_project / gg_back_project + gg_get_cas_volume)."""
    from multigpugridder_gb300 import synthetic
    from multigpugridder_gb300._lib import GG_ERR_BUSY, GridderError, check, lib
    from multigpugridder_gb300.serve import Server, pinned_empty

    L = lib()
    offered = serve_schedule(args.serve_seconds, args.serve_rate)
    closed = offered[:args.serve_closed]
    # request k takes the first n directions of direction set k mod 64 (4,096
    # random-quaternion directions each): a bounded host footprint for any run length
    pool = [synthetic.quaternion_axes(4096, 1000 + k).astype(np.float32) for k in range(64)]
    axes = {seed: pool[(seed - 1000) % len(pool)] for _, _, _, _, seed in offered}
    vols = [synthetic.blob_volume(N, b, seed=50 + i) for i, (N, b) in enumerate(zip(SERVE_SIZES, SERVE_BLOBS))]
    legs = set(args.serve_legs.split(","))
    srv = Server(lanes=args.serve_lanes, quantum_ms=args.serve_quantum_ms)
    vids = [srv.add_volume(v) for v in vols]
    sizes = [srv.sizes(v) for v in vids]
    rng = np.random.default_rng(7)
    img_in, fp_out, bp_out = [], [], []
    for (N, M, V) in sizes:
        block = rng.standard_normal((64, N, N)).astype(np.float32)
        buf = pinned_empty((4096, N, N))
        buf[:] = np.resize(block, buf.shape)
        img_in.append(buf.reshape(-1))
        fp_out.append(pinned_empty((4096 * N * N,)))
        bp_out.append(pinned_empty((V * V * V,)))

    def submit(si, op, n, seed):
        N, M, V = sizes[si]
        ax = axes[seed][:n]
        if op == "forward":
            return srv.submit(vids[si], op, ax, out=fp_out[si][:n * N * N])
        return srv.submit(vids[si], op, ax, images=img_in[si][:n * N * N], out=bp_out[si])

    def open_loop(sched, scale=1.0, backlog=0.0):
        """Arrivals at their scheduled times; with a backlog bound, arrivals that
        find that much work queued are refused (GG_ERR_BUSY) and counted."""
        srv.set_max_backlog(backlog)
        srv.reset_stats()
        t0 = time.perf_counter()
        hs, kept = [], []
        for req in sched:
            t, si, op, n, seed = req
            t = t * scale
            while True:
                dt = t - (time.perf_counter() - t0)
                if dt <= 0:
                    break
                if dt > 2e-3:
                    time.sleep(dt - 1e-3)
            try:
                hs.append(submit(si, op, n, seed))
                kept.append(req)
            except GridderError as e:
                if e.code != GG_ERR_BUSY:
                    raise
        lats = [srv.wait(h)[1] for h in hs]
        el = time.perf_counter() - t0
        srv.set_max_backlog(0.0)
        st = srv.stats()
        dirs = sum(x[3] for x in kept)
        # latency percentiles per request class: small (n < 256) and large (n >= 1024)
        # requests on 64^3/128^3 and on 192^3/256^3 volumes
        classes = {}
        for (t, si, op, n, seed), lat in zip(kept, lats):
            key = "%s_%s" % ("vol64_128" if si < 2 else "vol192_256",
                             "n_lt_256" if n < 256 else ("n_ge_1024" if n >= 1024 else "n_256_1023"))
            classes.setdefault(key, []).append(lat)
        by_class = {k: {"requests": len(v), "p50_ms": float(np.percentile(v, 50)),
                        "p99_ms": float(np.percentile(v, 99))} for k, v in sorted(classes.items())}
        return {"offered_rps": len(sched) / (sched[-1][0] * scale) if sched else 0.0, "offered": len(sched),
                "requests": len(kept), "refused": len(sched) - len(kept), "backlog_bound_s": backlog,
                "seconds": el, "throughput_rps": len(kept) / el, "directions_per_s": dirs / el,
                "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
                "peak_inflight": st["peak_inflight"], "peak_gb": st["peak_gb"], "by_class": by_class}

    # warm the lanes, then the closed loop: all requests queued at once
    for h in [submit(si, op, min(n, 64), seed) for _, si, op, n, seed in closed[:16]]:
        srv.wait(h)

    def served_once():
        t0 = time.perf_counter()
        hs = [submit(si, op, n, seed) for _, si, op, n, seed in closed]
        for h in hs:
            srv.wait(h)
        return len(closed) / (time.perf_counter() - t0)
    # the same requests one at a time through the plain gridder calls
    grids = []
    for v, (N, M, V) in zip(vols, sizes):
        h = ctypes.c_void_p()
        dev = (ctypes.c_int * 1)(0)
        check(L.gg_create(N, 0, ctypes.c_float(2.0), 3, 1, dev, 1, 0, ctypes.byref(h)))
        check(L.gg_set_max_axes_to_allocate(h, 4096), h)
        dims = (ctypes.c_int * 3)(N, N, N)
        check(L.gg_set_volume(h, v.ctypes.data, dims), h)
        grids.append(h)

    def plain(si, op, n, seed):
        h = grids[si]
        N, M, V = sizes[si]
        ax = axes[seed]
        if op == "forward":
            check(L.gg_forward_project(h, ax.ctypes.data, n, fp_out[si].ctypes.data, None), h)
        else:
            check(L.gg_back_project(h, ax.ctypes.data, n, img_in[si].ctypes.data, None, 0), h)
            check(L.gg_get_cas_volume(h, bp_out[si].ctypes.data), h)

    for _, si, op, n, seed in closed[:16]:
        plain(si, op, min(n, 64), seed)

    def sequential_once():
        t0 = time.perf_counter()
        for _, si, op, n, seed in closed:
            plain(si, op, n, seed)
        return len(closed) / (time.perf_counter() - t0)

    # alternate the two arms so that drifts of the shared GPU hit both alike
    served_runs, seq_runs = [], []
    if "closed" in legs:
        for _ in range(max(1, args.serve_repeats)):
            served_runs.append(served_once())
            seq_runs.append(sequential_once())
    for h in grids:
        L.gg_destroy(h)

    res_offered = res_70 = None
    cap = args.serve_capacity
    if "offered" in legs:
        # ten times what one GPU serves: the backlog bound sheds what cannot be
        # served within about that many seconds, as an overloaded server does
        res_offered = open_loop(offered, backlog=args.serve_backlog)
        cap = res_offered["throughput_rps"]
    if "load70" in legs and cap > 0:
        rate70 = 0.7 * min(cap, args.serve_rate)
        res_70 = open_loop(offered[:max(1, int(rate70 * args.serve_seconds))], scale=args.serve_rate / rate70)
    srv.close()
    closed_res = None
    if served_runs:
        closed_res = {"requests": len(closed), "repeats": len(served_runs),
                      "served_rps": statistics.median(served_runs),
                      "sequential_plain_rps": statistics.median(seq_runs),
                      "speedup": statistics.median(a / b for a, b in zip(served_runs, seq_runs)),
                      "served_rps_runs": served_runs, "sequential_plain_rps_runs": seq_runs}
    return {"workload": "Poisson arrivals at %g req/s for %g s: forwardProject/backProject 50/50 on resident FP32 "
                        "volumes 64^3/128^3/192^3/256^3 (weights .4/.3/.2/.1, interpFactor 2), directions "
                        "log-uniform 16-4096 (random quaternions); back requests return the CAS volume"
                        % (args.serve_rate, args.serve_seconds),
            "lanes": args.serve_lanes, "quantum_ms": args.serve_quantum_ms, "offered": res_offered,
            "at_70pct_capacity": res_70, "capacity_rps": cap, "closed_loop": closed_res}


# ---- storage precision at 256^3 ------------------------------------------------
PREC_SUBSET = 64  # directions of the 5,000 compared against the FP64 oracle


PREC_WORKLOADS = {
    "256": "256^3 volume (400 blobs), interpFactor 2 (CAS volume 518^3), 5,000 random-quaternion directions",
    "128": "128^3 volume (100 blobs), interpFactor 2 (CAS volume 262^3), the 10,000 directions of the 100x100 grid",
}


def precision_workload(kind="256"):
    """(N, directions, volume, axes, subset, batch, timed steps) of a precision
    workload: "256" the 256^3 storage-precision configuration, "128" the
    benchmark's own 128^3 step."""
    from multigpugridder_gb300 import synthetic

    if kind == "128":
        N, n = 128, 10000
        vol = synthetic.blob_volume(N, 100, seed=2)
        axes = synthetic.grid_axes(100, 100).astype(np.float32)
        batch, reps = 2000, 3
    else:
        N, n = 256, 5000
        vol = synthetic.blob_volume(N, 400, seed=3)
        axes = synthetic.quaternion_axes(n, seed=3).astype(np.float32)
        batch, reps = 1000, 1
    sub = np.linspace(0, n - 1, PREC_SUBSET).round().astype(int)
    return N, n, vol, axes, sub, batch, reps


def run_precision(args, kind="256"):
    """setVolume + forwardProject + reconstructVol of a precision workload
    (precision_workload) with FP32, BF16 and FP16 storage (FP32 accumulation).
    Reports pairs/s per storage type and the relative L2 of the images and the
    reconstruction against the FP32 path.  It also keeps, per storage type,
    the images of a fixed subset of 64 directions and a reconstructVol of the
    FP32 path's images of those directions, for the FP64 comparison that the
    CPU leg makes (check_precision_vs_f64)."""
    import torch

    import multigpugridder_gb300 as gg
    from multigpugridder_gb300._lib import check, lib

    L = lib()
    N, n, vol, axes, sub, batch, reps = precision_workload(kind)
    dev = torch.device("cuda", torch.cuda.current_device())
    d_vol = torch.from_numpy(np.ascontiguousarray(vol)).to(dev)
    d_axes = torch.from_numpy(np.ascontiguousarray(axes)).to(dev)
    d_sub = torch.from_numpy(sub).to(dev)
    d_sub_axes = d_axes[d_sub].contiguous()
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    out, ref, keep = {}, {}, {}
    sub_imgs_f32 = None

    def vp(t):
        return ctypes.c_void_p(t.data_ptr())

    # "bf16_vol": BF16 volume, FP32 CAS images for the back projection
    for prec in ("f32", "bf16", "f16", "bf16_vol"):
        g = gg.MultiGPUGridder(N, n, 2.0, MaxAxesToAllocate=batch, precision="bf16" if prec == "bf16_vol" else prec)
        if prec == "bf16_vol":
            g.set_image_precision("f32")
        h = g.handle
        imgs = torch.empty((n, N, N), dtype=torch.float32, device=dev)
        rec = torch.empty((N, N, N), dtype=torch.float32, device=dev)

        def step():
            check(L.gg_set_volume_dev(h, vp(d_vol), sp), h)
            check(L.gg_forward_project_dev(h, vp(d_axes), n, vp(imgs), None, sp), h)
            check(L.gg_reconstruct_volume_dev(h, vp(d_axes), n, vp(imgs), vp(rec), sp), h)

        with torch.cuda.stream(stream):
            step()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                step()
            b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        res = {"pairs_per_s": n / (ms / 1e3), "ms_per_step": ms}
        if prec == "f32":
            ref = {"images": imgs.clone(), "rec": rec.clone()}
            sub_imgs_f32 = imgs[d_sub].contiguous()
        else:
            for k, t in (("images", imgs), ("rec", rec)):
                res["rel_l2_%s_vs_f32" % k] = float(torch.linalg.vector_norm((t - ref[k]).double())
                                                    / torch.linalg.vector_norm(ref[k].double()))
        # reconstructVol of the subset's FP32 images (the same input for every storage type)
        rec_sub = torch.empty((N, N, N), dtype=torch.float32, device=dev)
        with torch.cuda.stream(stream):
            check(L.gg_reconstruct_volume_dev(h, vp(d_sub_axes), len(sub), vp(sub_imgs_f32), vp(rec_sub), sp), h)
        torch.cuda.synchronize()
        keep[prec] = {"images": imgs[d_sub].cpu().numpy(), "rec": rec_sub.cpu().numpy()}
        out[prec] = res
        g.close()
        del imgs, rec, rec_sub
    keep["input_images"] = sub_imgs_f32.cpu().numpy()
    return {"workload": PREC_WORKLOADS[kind] + ": setVolume + forwardProject + reconstructVol, storage f32/bf16/f16 "
                        "(volume and CAS images) and bf16_vol (BF16 volume, FP32 CAS images), FP32 accumulation",
            "results": out}, keep


def check_precision_vs_f64(keep, kind="256"):
    """FP64 oracle references for the precision leg (part of the CPU leg):
    forwardProject of the 64-direction subset and reconstructVol of the FP32
    path's images of those directions, both in FP64 on the host; returns
    rel-L2 of each storage type's images and reconstruction against them."""
    from oracle import oracle as O

    N, n, vol, axes, sub, _, _ = precision_workload(kind)
    p = O.Params(N)
    t0 = time.perf_counter()
    ref_imgs, _ = O.forward_project(vol, axes[sub], p, precision="f64")
    ref_rec, _, _ = O.reconstruct_vol(keep["input_images"].astype(np.float64), axes[sub], p, precision="f64")
    res = {"subset": "%d of the %d directions (evenly spaced); images: forwardProject; rec: reconstructVol of the "
                     "FP32 path's images of those directions" % (len(sub), n),
           "oracle_seconds": time.perf_counter() - t0}
    for prec, k in keep.items():
        if prec == "input_images":
            continue
        res[prec] = {"rel_l2_images_vs_f64": O.rel_l2(k["images"], ref_imgs),
                     "rel_l2_rec_vs_f64": O.rel_l2(k["rec"], ref_rec)}
    return res


# ---- differentiation -----------------------------------------------------------
def run_autograd(args):
    """torch FP32 volume 128^3 (requires_grad, Gaussian-blob init), interpFactor
    2, batches of 4,096 random directions, loss ||P(V) - Y||^2 with
    Y = P(V_true) + Gaussian noise at SNR 0.1, backward through the exact
    adjoint; 20 gradient-descent iterations timed, cycling over 4 batches.

    Step size 1 / L with L = 2 * 1.1 * lambda_max(P^T P), lambda_max from 15
    power iterations on the first batch (untimed): for a quadratic loss a
    step of 1 / L never increases it.  The noise floor is sum ||noise_k||^2
    over the 4 batches; `excess_removed` is the fraction of the loss above
    that floor that the 20 iterations remove (last cycle against first)."""
    import torch

    from multigpugridder_gb300 import synthetic
    from multigpugridder_gb300.autograd import ForwardProjector

    N, B, iters, nb = 128, 4096, 20, 4
    dev = torch.device("cuda", torch.cuda.current_device())
    proj = ForwardProjector(N, 2.0, max_batch=B)
    v_true = torch.from_numpy(synthetic.blob_volume(N, 100, seed=4)).to(dev)
    batches = []
    floor = 0.0
    for k in range(nb):
        ax = torch.from_numpy(synthetic.quaternion_axes(B, seed=40 + k).astype(np.float32)).to(dev)
        with torch.no_grad():
            clean = proj.project(v_true, ax)
            sigma = float(torch.sqrt(clean.var() / 0.1))
            gen = torch.Generator(device=dev).manual_seed(400 + k)
            noise = sigma * torch.randn(clean.shape, device=dev, generator=gen)
            floor += float(torch.sum(noise.double() ** 2))
            y = clean + noise
        batches.append((ax, y))
        del clean, noise
    # largest eigenvalue of P^T P by power iteration
    with torch.no_grad():
        x = torch.randn((N,) * 3, device=dev, generator=torch.Generator(device=dev).manual_seed(7))
        lam = 0.0
        for _ in range(15):
            x = x / torch.linalg.vector_norm(x)
            x = proj.adjoint(proj.project(x, batches[0][0]), batches[0][0])
            lam = float(torch.linalg.vector_norm(x))
    lr = 1.0 / (2.0 * 1.1 * lam)
    vol = torch.from_numpy(synthetic.blob_volume(N, 100, seed=41)).to(dev).requires_grad_(True)
    vol0 = vol.detach().clone()

    def it(k):
        ax, y = batches[k % nb]
        loss = torch.sum((proj.project(vol, ax) - y) ** 2)
        loss.backward()
        with torch.no_grad():
            vol.sub_(lr * vol.grad)
            vol.grad = None
        return loss.detach()

    # warm-up on the same iterations, then restart from the initial volume
    for k in range(2):
        it(k)
    with torch.no_grad():
        vol.copy_(vol0)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    losses = []
    a.record()
    for k in range(iters):
        losses.append(it(k))
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / iters
    with torch.no_grad():
        err0 = float(torch.linalg.vector_norm(vol0 - v_true) / torch.linalg.vector_norm(v_true))
        err1 = float(torch.linalg.vector_norm(vol.detach() - v_true) / torch.linalg.vector_norm(v_true))
    proj.close()
    first = sum(float(x) for x in losses[:nb])
    last = sum(float(x) for x in losses[-nb:])
    return {"workload": "128^3 FP32 volume, interpFactor 2, batches of 4,096 random directions (4 batches "
                        "cycled), loss ||P(V) - Y||^2 (Y = P(V_true) + noise at SNR 0.1), 20 gradient-descent "
                        "iterations, step 1/L from power iteration",
            "ms_per_iteration": ms, "directions_per_s": B / (ms / 1e3), "step_size": lr,
            "lambda_max": lam, "loss_first_cycle": first, "loss_last_cycle": last, "noise_floor": floor,
            "excess_removed": (first - last) / (first - floor) if first > floor else None,
            "losses": [float(x) for x in losses],
            "rel_error_to_v_true": {"start": err0, "end": err1}}


# ---- CTF application before back projection ------------------------------------
def run_ctf(args, vol, axes):
    """reconstructVol of the step's images with and without the CTF applied
    before the back projection (device pointers, FP32): defoci uniform in
    8,000-25,000 Å, 300 kV, Cs 2.7 mm, amplitude contrast 0.1, 1 Å pixels."""
    import torch

    from multigpugridder_gb300 import MultiGPUGridder
    from multigpugridder_gb300._lib import check, lib

    L = lib()
    N, n = args.size, len(axes)
    dev = torch.device("cuda", torch.cuda.current_device())
    g = MultiGPUGridder(N, n, 2.0, MaxAxesToAllocate=args.batch)
    h = g.handle
    s = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(s.cuda_stream)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    d_vol = torch.from_numpy(np.ascontiguousarray(vol)).to(dev)
    d_ax = torch.from_numpy(np.ascontiguousarray(axes)).to(dev)
    d_img = torch.empty((n, N, N), device=dev)
    d_out = torch.empty((N, N, N), device=dev)
    df = torch.from_numpy(np.random.default_rng(9).uniform(8000.0, 25000.0, n).astype(np.float32)).to(dev)
    check(L.gg_set_volume_dev(h, vp(d_vol), sp), h)
    check(L.gg_forward_project_dev(h, vp(d_ax), n, vp(d_img), None, sp), h)
    calls = {"plain": lambda: check(L.gg_reconstruct_volume_dev(h, vp(d_ax), n, vp(d_img), vp(d_out), sp), h),
             "ctf": lambda: check(L.gg_reconstruct_volume_ctf_dev(h, vp(d_ax), n, vp(d_img), vp(df), None, None, 300.0,
                                                                  2.7, 0.1, 1.0, vp(d_out), sp), h)}
    res = {}
    for name, call in calls.items():
        for _ in range(max(3, args.warmup)):
            call()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(s)
        for _ in range(args.steps):
            call()
        b.record(s)
        torch.cuda.synchronize()
        res[name + "_ms"] = a.elapsed_time(b) / args.steps
    res["finite"] = bool(torch.isfinite(d_out).all())
    g.close()
    res["ctf_over_plain"] = res["ctf_ms"] / res["plain_ms"]
    res["workload"] = ("reconstructVol of %d images %d^2 (interpFactor 2), FP32, device pointers; CTF: defoci "
                       "8,000-25,000 Å, 300 kV, Cs 2.7 mm, A 0.1, 1 Å pixels" % (n, N))
    return res


def run_e2e(args, g, vol, axes, world, dev):
    """The same step through the host-pointer ABI with pinned host buffers:
    volume and axes in, this rank's images out and back in, volume out.  With
    W > 1 ranks the images go back in as the sums call's device input (one
    pinned copy) and the step ends with the all-reduce, the division and getVol
    as in the timed step; time is the max over ranks."""
    import torch
    import torch.distributed as dist

    from multigpugridder_gb300._lib import check, lib
    from multigpugridder_gb300.sharding import max_over_ranks

    L = lib()
    h = g.handle
    n, N, V = len(axes), args.size, g.V
    h_vol = torch.from_numpy(np.ascontiguousarray(vol)).pin_memory()
    h_axes = torch.from_numpy(np.ascontiguousarray(axes)).pin_memory()
    h_imgs = torch.empty((n, N, N), dtype=torch.float32).pin_memory()
    h_out = torch.empty((N, N, N), dtype=torch.float32).pin_memory()
    dims = (ctypes.c_int * 3)(N, N, N)
    if world > 1:
        stream = torch.cuda.Stream(device=dev)
        sp = ctypes.c_void_p(stream.cuda_stream)
        d_axes = torch.empty((n, 9), dtype=torch.float32, device=dev)
        d_imgs = torch.empty((n, N, N), dtype=torch.float32, device=dev)
        d_sums = torch.empty((2, V, V, V), dtype=torch.float32, device=dev)
        d_out = torch.empty((N, N, N), dtype=torch.float32, device=dev)

    def vp(t):
        return ctypes.c_void_p(t.data_ptr())

    def step():
        check(L.gg_set_volume(h, vp(h_vol), dims), h)
        check(L.gg_forward_project(h, vp(h_axes), n, vp(h_imgs), None), h)
        if world == 1:
            check(L.gg_reconstruct_volume(h, vp(h_axes), n, vp(h_imgs), vp(h_out)), h)
            return
        with torch.cuda.stream(stream):
            d_axes.copy_(h_axes, non_blocking=True)
            d_imgs.copy_(h_imgs, non_blocking=True)
            check(L.gg_back_project_sums_dev(h, vp(d_axes), n, vp(d_imgs), vp(d_sums), sp), h)
            dist.all_reduce(d_sums)
            check(L.gg_volume_from_sums_dev(h, vp(d_sums), vp(d_out), sp), h)
            h_out.copy_(d_out, non_blocking=True)
        stream.synchronize()

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = max_over_ranks((time.perf_counter() - t0) / args.steps, device=dev)
    ok = bool(np.isfinite(h_out.numpy()).all())
    h2d = vol.nbytes + 2 * axes.nbytes + n * N * N * 4
    d2h = n * N * N * 4 + vol.nbytes
    return {"value": world * n / dt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": dt * 1e3, "finite": ok}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
