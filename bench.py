"""Benchmark of the generalised geodesic distance engine on one GB300 per rank.

Default workload (one "step"): the plain 3D transform of a 1x1x128x256x256
float32 volume -- Gaussian-smoothed (sigma 2) uniform[0,1] noise, spacing
(2.0, 0.5, 0.5), soft mask all 1.0 except one 6^3 seed cube, v = 1e10,
iterations 4 -- run once for each lamb in {0.0, 0.5, 1.0} through the drop-in
API.  Inputs are synthetic, seeded, generated on the host.

Metric: Gvoxel-passes/s, where one voxel-pass is one cell updated in one
directional sweep (a 3D transform is voxels x 6 x iterations voxel-passes).

Printed as one JSON line by rank 0, with the kernel roofline, the CPU
baseline (the oracle restatement of the reference's OpenMP CPU path, timed on
this host), the end-to-end figure with host buffers, and the SM clocks seen.

`--impl reference` times the reference's CPU path instead (its own build from
the reference sources where present, else the oracle restatement) on all host
cores, on the same workload, metric and unit.

Several GPUs (torchrun): the path does not shard a single volume, so every
rank runs an independent replica of the workload (weak scaling); the time is
the maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 1024 * 1024
FLUSH_BYTES = 512 * 1024 * 1024


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def smooth_noise(rng, shape, sigma, lo, hi):
    from scipy.ndimage import gaussian_filter

    x = rng.uniform(lo, hi, size=shape).astype(np.float32)
    return gaussian_filter(x, sigma=sigma, truncate=4.0).astype(np.float32)


def workload(name: str, seed: int = 1):
    if name in ("t1", "t2"):
        # Toivanen's raster scan on the c1 / c2 data (two passes per iteration)
        w = workload("c1" if name == "t1" else "c2", seed)
        w.update(name=name, method="toivanen",
                 desc=w["desc"].replace("generalised_geodesic", "generalised_geodesic_toivanen", 1)
                      .replace("geodesic_toivanen2d", "geodesic2d_toivanen")
                      .replace("geodesic_toivanen3d", "geodesic3d_toivanen"))
        return w
    if name == "b256":
        # a batch of 8 independent 256^3 volumes, one transform each
        vols = [workload("vol256", seed + k) for k in range(8)]
        lambs = [[0.0, 0.5, 1.0][k % 3] for k in range(8)]
        w = dict(vols[0], name=name, lambs=lambs, images=[(v["image"], v["mask"]) for v in vols])
        w["desc"] = ("generalised_geodesic3d batch of 8 volumes 1x1x256x256x256 fp32, each smoothed (sigma 2) "
                     "uniform[0,1] noise with its own 6^3 seed cube, spacing (1.0, 1.0, 1.0), v=1e10, "
                     "iterations 4, lamb cycling 0.0 / 0.5 / 1.0; one transform per volume")
        return w
    rng = np.random.default_rng(seed)
    if name in ("c2", "vol256", "slab"):
        # slab: 64 slices of 1024 x 1024, a cross-section larger than the
        # resident tiles hold (the sweep along the slices runs chunked)
        shape = {"c2": (128, 256, 256), "vol256": (256, 256, 256), "slab": (64, 1024, 1024)}[name]
        vol = smooth_noise(rng, shape, 2.0, 0.0, 1.0)
        mask = np.ones(shape, np.float32)
        c = [int(rng.integers(0, n - 6)) for n in shape]
        mask[c[0]:c[0] + 6, c[1]:c[1] + 6, c[2]:c[2] + 6] = 0.0
        sp = [2.0, 0.5, 0.5] if name == "c2" else [1.0, 1.0, 1.0]
        return dict(name=name, dims=3, image=vol[None, None], mask=mask[None, None], spacing=sp,
                    v=1e10, lambs=[0.0, 0.5, 1.0], iters=4, C=1,
                    desc=f"generalised_geodesic3d 1x1x{shape[0]}x{shape[1]}x{shape[2]} fp32, smoothed "
                         f"(sigma 2) uniform[0,1] noise, spacing {tuple(sp)}, one 6^3 seed cube, v=1e10, "
                         "iterations 4, one transform per lamb in {0.0, 0.5, 1.0}")
    if name == "c1":
        shape = (512, 512)
        img = smooth_noise(rng, shape, 3.0, 0.0, 255.0)
        mask = np.ones(shape, np.float32)
        yy, xx = np.mgrid[:512, :512]
        for _ in range(5):
            cy, cx = rng.integers(0, 512, 2)
            mask[(yy - cy) ** 2 + (xx - cx) ** 2 <= 16] = 0.0
        return dict(name=name, dims=2, image=img[None, None], mask=mask[None, None], spacing=None,
                    v=1e10, lambs=[1.0], iters=2, C=1,
                    desc="generalised_geodesic2d 1x1x512x512 fp32, smoothed (sigma 3) uniform[0,255] "
                         "noise, 5 seed disks r=4, v=1e10, lamb 1.0, iterations 2")
    raise SystemExit(f"unknown workload {name}")


def batch_workload(seed: int = 3, n: int = 64):
    """64 uneven 2D images: H, W ~ U[128, 2048] (multiples of 4), C in {1, 3},
    Gaussian-smoothed (sigma 3) uniform[0, 255] noise, 1-10 seed disks (r=4)
    per soft mask, lamb ~ U[0, 1], iterations 2; plain and signed transforms.
    Smoothing runs on the GPU (separable kernel truncated at 4 sigma)."""
    import torch

    rng = np.random.default_rng(seed)
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device="cpu").manual_seed(seed)
    sig = 3.0
    r = int(4 * sig + 0.5)
    x = torch.arange(-r, r + 1, dtype=torch.float32)
    k = torch.exp(-0.5 * (x / sig) ** 2)
    k = (k / k.sum()).to(dev)
    items = []
    for _ in range(n):
        H = int(rng.integers(32, 513)) * 4
        W = int(rng.integers(32, 513)) * 4
        C = int(rng.choice([1, 3]))
        im = (torch.rand((C, 1, H, W), generator=g) * 255.0).to(dev)
        im = torch.nn.functional.conv2d(torch.nn.functional.pad(im, (r, r, 0, 0), mode="reflect"), k.view(1, 1, 1, -1))
        im = torch.nn.functional.conv2d(torch.nn.functional.pad(im, (0, 0, r, r), mode="reflect"), k.view(1, 1, -1, 1))
        im = im.view(1, C, H, W).contiguous()
        m = torch.ones((1, 1, H, W), device=dev)
        yy = torch.arange(H, device=dev).view(H, 1)
        xx = torch.arange(W, device=dev).view(1, W)
        for _ in range(int(rng.integers(1, 11))):
            cy, cx = int(rng.integers(0, H)), int(rng.integers(0, W))
            m[0, 0][(yy - cy) ** 2 + (xx - cx) ** 2 <= 16] = 0.0
        items.append((im, m, float(rng.random())))
    return items


def batch_cpu_sample(images, masks, lambs, budget_s=15.0, kind_pref="port", build=False):
    """CPU baseline of the uneven batch: plain and signed transform of images
    taken in a fixed spread over the batch (each once before any twice), until
    about `budget_s` seconds.  kind_pref "reference": the reference's own
    installed package (its public API, OpenMP CPU path; its signed transform
    runs the second map in a std::async thread) where it is built here, else
    the C restatement of its CPU path (the `port`).  images[i]: [C, H, W],
    masks[i]: [1, H, W] (numpy).  Returns (Gvoxel-passes/s, kind, cores, sample
    description)."""
    from math import gcd

    from oracle import oracle

    FG = reference_install(build=build) if kind_pref == "reference" else None
    if FG is not None:
        import torch

        cores = host_threads()

        def plain(i):
            FG.generalised_geodesic2d(torch.from_numpy(images[i])[None], torch.from_numpy(masks[i])[None], 1e10,
                                      lambs[i], 2)

        def signed(i):
            FG.signed_generalised_geodesic2d(torch.from_numpy(images[i])[None], torch.from_numpy(masks[i])[None],
                                             1e10, lambs[i], 2)

        kind = "reference"
    else:
        cores = oracle.max_threads()

        def plain(i):
            oracle.geodesic2d(images[i], masks[i], 1e10, lambs[i], 2)

        def signed(i):
            oracle.signed2d(images[i], masks[i], 1e10, lambs[i], 2)

        kind = "port"
    n = len(images)
    stride = 37 if gcd(37, n) == 1 else 1
    t_total, vp, done = 0.0, 0.0, 0
    for k in range(4 * n):
        i = (k * stride) % n
        t0 = time.perf_counter()
        plain(i)
        signed(i)
        t_total += time.perf_counter() - t0
        H, W = images[i].shape[1:]
        vp += float(H) * W * 4 * 2 * 3  # 4 passes x 2 iterations; plain + signed (two maps)
        done += 1
        if t_total >= budget_s:
            break
    sample = f"{done} images of the batch, plain + signed transform each (iterations 2), {t_total:.1f} s"
    return vp / t_total / 1e9, kind, cores, sample


def run_batch_reference_arm(args, rank, world=1):
    """The uneven batch on the reference's CPU path (its installed package where
    it builds here, else its C restatement; all host threads): a bounded sample
    of the batch's plain + signed transforms."""
    import torch

    if rank != 0:
        return
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    items = batch_workload()  # generated (smoothed) on the device, then copied to the host
    images = [im[0].cpu().numpy() for im, _, _ in items]
    masks = [m[0].cpu().numpy() for _, m, _ in items]
    t0 = time.perf_counter()
    value, kind, cores, sample = batch_cpu_sample(images, masks, [l for _, _, l in items], budget_s=args.cpu_budget,
                                                  kind_pref="reference", build=True)
    wall = time.perf_counter() - t0
    line = {
        "impl": "reference", "metric": "generalised_geodesic2d uneven batch throughput", "value": round(value, 4),
        "unit": "Gvoxel-passes/s", "n_gpus": world, "steps": 1, "warmup": 0,
        "ms_per_step": round(1e3 * wall, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "64 images H,W ~ U[128,2048] step 4, C in {1,3}, smoothed noise [0,255], "
                               "1-10 seed disks, lamb ~ U[0,1], iterations 2; plain and signed per step",
                   "step": "one bounded sample of the batch"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gvoxel-passes/s", "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Gvoxel-passes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batch_arm(args, rank, world):
    """Uneven 2D batch: the batched persistent launch (CUDA graph) against the
    plain per-call drop-in path, both on device-resident inputs."""
    import torch

    import fastgeodis_gb300 as fg

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    items = batch_workload()
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im, _, _ in items]
    n = len(items)
    # every image twice, plain and signed, in one persistent launch
    plan = fg.GeodesicBatch2d(shapes + shapes, signed=[False] * n + [True] * n, iterations=2, use_graph=True,
                              inputs=([im for im, _, _ in items] * 2, [m for _, m, _ in items] * 2))
    plan.v, plan.lambs = 1e10, [l for _, _, l in items] * 2
    vp = float(sum(s[1] * s[2] for s in shapes)) * 4 * 2 * 3  # plain + signed (2 transforms)
    flush = torch.empty(FLUSH_BYTES // 4, device="cuda")

    def batched():
        plan.run()

    def per_call():
        for im, m, l in items:
            fg.generalised_geodesic2d(im, m, 1e10, l, 2)
            fg.signed_generalised_geodesic2d(im, m, 1e10, l, 2)

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        tot = 0.0
        for k in range(steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / steps

    clocks = ClockSampler(local).start()
    ms_b = timed(batched, args.steps)
    clk = clocks.stop()
    ms_p = timed(per_call, max(1, min(args.steps, 3)))
    fg.check_status()
    # end to end: host images in pinned memory, copied in, batch run, results read back
    h_imgs = [im.cpu().pin_memory() for im, _, _ in items]
    h_msks = [m.cpu().pin_memory() for _, m, _ in items]
    h_outs = [torch.empty(o.shape, pin_memory=True) for o in plan.outputs]

    def e2e_step():
        for i in range(n):  # the plain and signed entries share their input tensors
            plan.images[i].copy_(h_imgs[i], non_blocking=True)
            plan.masks[i].copy_(h_msks[i], non_blocking=True)
        batched()
        for i, o in enumerate(plan.outputs):
            h_outs[i].copy_(o, non_blocking=True)
        torch.cuda.synchronize()

    for _ in range(max(1, args.warmup)):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    h2d = sum(t.numel() * 4 for t in h_imgs + h_msks)
    d2h = sum(o.numel() * 4 for o in plan.outputs)
    if rank != 0:
        return
    i0 = min(range(len(items)), key=lambda i: shapes[i][1] * shapes[i][2])  # the smallest image of the batch
    batched()
    torch.cuda.synchronize()
    plan.check()
    f64 = fp64_check(plan.outputs[i0][0].cpu().numpy(), items[i0][0][0].cpu().numpy(),
                     items[i0][1][0].cpu().numpy(), 1e10, items[i0][2], 2)
    f64["image"] = "the smallest of the batch, plain transform"
    cpu_val, cpu_kind, cpu_cores, cpu_sample = batch_cpu_sample(
        [im[0].cpu().numpy() for im, _, _ in items], [m[0].cpu().numpy() for _, m, _ in items],
        [l for _, _, l in items], budget_s=args.cpu_budget, kind_pref="reference")
    line = {
        "metric": "generalised_geodesic2d uneven batch throughput", "value": round(vp / ms_b / 1e6, 4),
        "unit": "Gvoxel-passes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_b, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "64 images H,W ~ U[128,2048] step 4, C in {1,3}, smoothed noise [0,255], "
                               "1-10 seed disks, lamb ~ U[0,1], iterations 2; plain and signed per step",
                   "path": "GeodesicBatch2d: plain and signed transforms in one persistent launch, the largest "
                           "images tiled over several CTAs in a cooperative launch beside it (one CUDA graph)",
                   "jobs": len(plan.jobs), "split_signed_images": sum(1 for _, part in plan.jobs if part == 1),
                   "tiled_images": {f"{shapes[i % n][0]}x{shapes[i % n][1]}x{shapes[i % n][2]}"
                                    f"{' signed' if i >= n else ''}": k for i, k in sorted(plan.tiled.items())},
                   "per_call_value": round(vp / ms_p / 1e6, 4), "per_call_ms_per_step": round(ms_p, 3),
                   "speedup_vs_per_call": round(ms_p / ms_b, 2),
                   "l2": f"flushed between steps ({FLUSH_BYTES >> 20} MiB write outside the timed events)",
                   "fp64_check": f64},
        "e2e": {"value": round(vp / e2e_s / 1e9, 4), "unit": "Gvoxel-passes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "cpu_baseline": {"value": round(cpu_val, 4), "unit": "Gvoxel-passes/s", "cores": cpu_cores,
                         "kind": cpu_kind, "sample": cpu_sample},
        "clocks": clk, "gpu_launches": 1 + len(plan._tiled_groups),
    }
    print(json.dumps(line), flush=True)


def run_grad_arm(args, rank, world):
    """Differentiable geodesic2d: batch 16x1x512x512 smoothed noise, soft
    mask sigmoid(smoothed Gaussian noise), lamb 0.75, iterations 2, v 10,
    loss = sum(w * D) with w ~ U[0,1]; forward + backward timed, gradients
    checked against float64 central finite differences (eps 1e-3) of the
    oracle scan at 64 random voxels of the first image."""
    import torch

    import fastgeodis_gb300 as fg
    from oracle import oracle

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rng = np.random.default_rng(4)
    B, H, W = 16, 512, 512
    v, lamb, it = 10.0, 0.75, 2
    img = np.stack([smooth_noise(rng, (H, W), 3.0, 0.0, 255.0) for _ in range(B)])[:, None]
    msk = np.stack([1.0 / (1.0 + np.exp(-smooth_noise(rng, (H, W), 3.0, -6.0, 6.0) * 4.0)) for _ in range(B)])
    msk = msk[:, None].astype(np.float32)
    wts = rng.random((B, 1, H, W)).astype(np.float32)
    ti = torch.from_numpy(img).cuda().requires_grad_(True)
    tm = torch.from_numpy(msk).cuda().requires_grad_(True)
    tw = torch.from_numpy(wts).cuda()
    flush = torch.empty(FLUSH_BYTES // 4, device="cuda")

    def step():
        ti.grad = None
        tm.grad = None
        d = fg.generalised_geodesic2d_differentiable(ti, tm, v, lamb, it)
        (d * tw).sum().backward()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local).start()
    tot = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    clk = clocks.stop()
    ms = tot / args.steps
    gi = ti.grad[0, 0].cpu().numpy().astype(np.float64)
    gm = tm.grad[0, 0].cpu().numpy().astype(np.float64)
    if rank != 0:
        return
    # float64 finite differences of the same scan (oracle), first image
    eps = 1e-3
    w0 = wts[0, 0].astype(np.float64)
    im0, m0 = img[0].astype(np.float64), msk[0].astype(np.float64)

    def loss(im, m):
        return float((oracle.geodesic2d_f64(im, m, v, lamb, it)[0] * w0).sum())

    pts = [(int(rng.integers(0, H)), int(rng.integers(0, W))) for _ in range(64)]
    agree_i = agree_m = 0
    max_rel = 0.0
    t0 = time.perf_counter()
    for (y, x) in pts:
        p, q = im0.copy(), im0.copy()
        p[0, y, x] += eps
        q[0, y, x] -= eps
        fd_i = (loss(p, m0) - loss(q, m0)) / (2 * eps)
        p, q = m0.copy(), m0.copy()
        p[0, y, x] += eps
        q[0, y, x] -= eps
        fd_m = (loss(im0, p) - loss(im0, q)) / (2 * eps)
        for fd, g, tag in ((fd_i, gi[y, x], "i"), (fd_m, gm[y, x], "m")):
            rel = abs(fd - g) / max(1.0, abs(fd))
            ok = rel <= 1e-2
            if tag == "i":
                agree_i += ok
            else:
                agree_m += ok
            if ok:
                max_rel = max(max_rel, rel)
    fd_s = time.perf_counter() - t0
    vp = float(B * H * W * 4 * it)  # forward voxel-passes; the adjoint walks the same passes once more
    line = {
        "metric": "differentiable generalised_geodesic2d forward+backward throughput",
        "value": round(2 * vp / ms / 1e6, 4), "unit": "Gvoxel-passes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "16x1x512x512 smoothed noise [0,255], softmask sigmoid(smoothed noise), lamb 0.75, "
                               "v 10, iterations 2, loss sum(w*D), w ~ U[0,1]; forward + backward per step",
                   "grad_check": {"voxels": 64, "eps": 1e-3, "reference": "float64 central differences of the scan",
                                  "image_agree": int(agree_i), "mask_agree": int(agree_m),
                                  "tolerance": "1e-2 relative (1e-2 absolute below 1)",
                                  "max_rel_err_agreeing": max_rel, "seconds": round(fd_s, 1)},
                   "l2": f"flushed between steps ({FLUSH_BYTES >> 20} MiB write outside the timed events)"},
        "clocks": clk, "gpu_launches": 2,  # the forward and the adjoint kernel
    }
    print(json.dumps(line), flush=True)


def run_serve_arm(args, rank, world):
    """Served interactive stream: Poisson arrivals at 200 req/s; 70% 2D
    (256^2-2048^2, 1-3 channels), 30% 3D (64^3-256^3, spacing U[0.5, 3] per
    axis); 1-5 click seeds each; 10% of requests GSF (theta 0.5); v 1e10,
    lamb 1.0, iterations 2.  Images live on the device (a pool of 12 2D and
    6 3D images, registered once), masks are rasterised from the clicks on the
    device.  The continuous-batching server (8 in flight, 4 streams, 16 GB
    budget) is compared with the same arrivals served one at a time on one
    stream (the plain per-call path)."""
    import torch

    from fastgeodis_gb300.serving import GeodesicServer, Request

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rng = np.random.default_rng(11)
    g = torch.Generator(device="cpu").manual_seed(11)
    pool2d, pool3d = [], []
    for _ in range(12):
        H, W, C = int(rng.integers(256, 2049)), int(rng.integers(256, 2049)), int(rng.integers(1, 4))
        pool2d.append(torch.rand((1, C, H, W), generator=g) * 255)
    for _ in range(6):
        n = [int(rng.integers(64, 257)) for _ in range(3)]
        pool3d.append(torch.rand((1, 1) + tuple(n), generator=g))
    n_req = args.requests
    rate = 200.0
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    specs = []
    for i in range(n_req):
        is3d = rng.random() < 0.3
        key = ("v", int(rng.integers(0, len(pool3d)))) if is3d else ("i", int(rng.integers(0, len(pool2d))))
        img = pool3d[key[1]] if is3d else pool2d[key[1]]
        shape = img.shape[2:]
        clicks = [[int(rng.integers(0, s)) for s in shape] for _ in range(int(rng.integers(1, 6)))]
        sp = [float(x) for x in rng.uniform(0.5, 3.0, 3)] if is3d else None
        op = "gsf" if rng.random() < 0.1 else "plain"
        cells = float(np.prod(shape))
        vp = cells * (6 if is3d else 4) * 2 * (6 if op == "gsf" else 1)
        specs.append((key, clicks, sp, op, vp))

    def serve(max_inflight, streams):
        srv = GeodesicServer(budget_bytes=16 << 30, max_inflight=max_inflight, streams=streams)
        for i, t in enumerate(pool2d):
            srv.register_image(("i", i), t)
        for i, t in enumerate(pool3d):
            srv.register_image(("v", i), t)
        # warm-up: one request of every image (kernel variants, workspaces)
        for key in [("i", i) for i in range(len(pool2d))] + [("v", i) for i in range(len(pool3d))]:
            img = srv.executor.images[key]
            srv.submit(Request(image_id=key, clicks=[[0] * (img.dim() - 2)], v=1e10, lamb=1.0,
                               spacing=[1.0, 1.0, 1.0] if img.dim() == 5 else None))
        srv.drain()
        srv.scheduler.completed.clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reqs = []
        for (key, clicks, sp, op, vp), ta in zip(specs, arrivals):
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            reqs.append(srv.submit(Request(image_id=key, clicks=clicks, op=op, v=1e10, lamb=1.0, iterations=2,
                                           spacing=sp, theta=0.5, radius=3)))
        srv.drain(timeout=600)
        wall = time.perf_counter() - t0
        errs = [r.error for r in reqs if r.error is not None]
        if errs:
            raise errs[0]
        pct = srv.scheduler.latency_percentiles((50, 99))
        peak = srv.scheduler.peak_inflight
        srv.close()
        return pct, wall, peak

    clocks = ClockSampler(local).start()
    pct_b, wall_b, peak_b = serve(16, 8)
    clk = clocks.stop()
    pct_s, wall_s, _ = serve(1, 1)
    vp_total = sum(s[4] for s in specs)
    if rank != 0:
        return
    line = {
        "metric": "served geodesic requests: throughput (p50/p99 latency in config)",
        "value": round(n_req / wall_b, 2), "unit": "requests/s", "n_gpus": world, "steps": n_req,
        "warmup": 18, "ms_per_step": round(wall_b / n_req * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n_req} requests, Poisson arrivals at 200/s, 70% 2D 256^2-2048^2 C 1-3, "
                               "30% 3D 64^3-256^3 spacing U[0.5,3], 1-5 clicks (r=3), 10% GSF (theta 0.5), "
                               "v 1e10, lamb 1, iterations 2",
                   "server": "continuous batching, 16 in flight, 8 streams, 16 GB HBM budget",
                   "p50_ms": round(pct_b["p50"], 3), "p99_ms": round(pct_b["p99"], 3),
                   "peak_inflight": peak_b, "gvoxel_passes_per_s": round(vp_total / wall_b / 1e9, 3),
                   "per_call_path": {"p50_ms": round(pct_s["p50"], 3), "p99_ms": round(pct_s["p99"], 3),
                                     "requests_per_s": round(n_req / wall_s, 2)}},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def voxel_passes(w) -> float:
    n = float(np.prod(w["image"].shape[2:]))
    per = 2 if w.get("method") == "toivanen" else (6 if w["dims"] == 3 else 4)
    return n * per * w["iters"] * len(w["lambs"])


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def fp64_check(got, image, mask, v, lamb, iters, spacing=None):
    """Error of one float32 transform against the oracle's float64 scan of
    the same inputs (the same raster scan in double precision)."""
    from oracle import oracle

    t0 = time.perf_counter()
    if spacing is None:
        ref = oracle.geodesic2d_f64(image, mask, v, lamb, iters)
    else:
        ref = oracle.geodesic3d_f64(image, mask, spacing, v, lamb, iters)
    got = np.asarray(got, np.float64)
    err = np.abs(got - ref)
    rel = err / np.maximum(np.abs(ref), 1e-30)
    # a distance is a sum of up to about (sum of the extents) rounded float32
    # additions, each off by at most 2^-24 of the running value
    path = int(sum(got.shape[-3:] if spacing is not None else got.shape[-2:]))
    bound = path * 2.0 ** -23
    return {"lamb": lamb, "max_abs_err": float(err.max()), "max_rel_err": float(rel.max()),
            "rel_bound": bound, "within_bound": bool(np.all(err <= 1e-4 + bound * np.abs(ref))),
            "bound_note": "1e-4 + (sum of extents) * 2^-23 relative: float32 rounding along a path",
            "reference": "oracle float64 scan of the same inputs", "seconds": round(time.perf_counter() - t0, 2)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_traffic(workload_name):
    """Per-launch DRAM bytes of the dominant kernel from a committed ncu
    summary (profiles/traffic.json), or None if not captured."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(workload_name)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------
# CPU side: oracle / reference timing
# ---------------------------------------------------------------------------

def reference_install(build: bool = True):
    """The reference as its users install it: its own ``FastGeodis`` package
    over its ``FastGeodisCpp`` extension (OpenMP CPU path, CUDA path for
    sm_103a), assembled in baseline/_ref by oracle/build_oracle.py from the
    reference's source files staged there.  Compiled on first use on this
    machine when `build`; None when the sources are not present."""
    from oracle import build_oracle

    try:
        FG = build_oracle.load_reference_install()
        if FG is None and build and build_oracle.build_reference_install() is not None:
            FG = build_oracle.load_reference_install()
        return FG
    except Exception as exc:  # a failed build leaves the port as the CPU baseline
        print(f"reference install unavailable: {exc}", file=sys.stderr)
        return None


def host_threads() -> int:
    """Every host core: the OpenMP threads of the reference's CPU path."""
    import torch

    n = os.cpu_count() or 1
    torch.set_num_threads(n)
    return torch.get_num_threads()


def reference_call(FG, w):
    """f(image, mask, lamb) through the reference's public API
    (FastGeodis/__init__.py:37-98, :165-238) for the workload's method."""
    tv = w.get("method") == "toivanen"
    if w["dims"] == 3:
        fn = FG.generalised_geodesic3d_toivanen if tv else FG.generalised_geodesic3d
        return lambda im, m, lamb: fn(im, m, w["spacing"], w["v"], lamb, w["iters"])
    fn = FG.generalised_geodesic2d_toivanen if tv else FG.generalised_geodesic2d
    return lambda im, m, lamb: fn(im, m, w["v"], lamb, w["iters"])


def cpu_transform_fn(kind_pref="reference", build=False):
    """Returns (callable(w, lamb, k), kind, cores).  kind 'reference' = the
    reference's own build (its installed package in baseline/_ref, else its
    CPU sources compiled into oracle/_ref), 'port' = the C restatement in
    oracle/.  k selects the workload's k-th (image, mask) pair."""
    from oracle import build_oracle, oracle

    def pair(w, k):
        return (w.get("images") or [(w["image"], w["mask"])])[k % len(w.get("images") or [0])]

    if kind_pref == "reference":
        FG = reference_install(build=build)
        if FG is not None:
            import torch

            cores = host_threads()

            def f(w, lamb, k=0):
                im, m = pair(w, k)
                return reference_call(FG, w)(torch.from_numpy(im), torch.from_numpy(m), lamb)

            return f, "reference", cores
        ref = build_oracle.load_reference()
        if ref is not None:
            import torch

            cores = host_threads()

            def f(w, lamb, k=0):
                im, m = pair(w, k)
                img, msk = torch.from_numpy(im), torch.from_numpy(m)
                if w.get("method") == "toivanen":  # geodis_toivanen.cpp: one thread
                    if w["dims"] == 3:
                        return ref.generalised_geodesic3d_toivanen(img, msk, w["spacing"], w["v"], lamb, 1 - lamb,
                                                                   w["iters"])
                    return ref.generalised_geodesic2d_toivanen(img, msk, w["v"], lamb, 1 - lamb, w["iters"])
                if w["dims"] == 3:
                    return ref.generalised_geodesic3d(img, msk, w["spacing"], w["v"], lamb, 1 - lamb, w["iters"])
                return ref.generalised_geodesic2d(img, msk, w["v"], lamb, 1 - lamb, w["iters"])

            return f, "reference", cores
    cores = oracle.max_threads()

    def f(w, lamb, k=0):
        im, m = pair(w, k)
        if w.get("method") == "toivanen":
            if w["dims"] == 3:
                return oracle.toivanen3d(im[0], m[0], w["spacing"], w["v"], lamb, w["iters"])
            return oracle.toivanen2d(im[0], m[0], w["v"], lamb, w["iters"])
        if w["dims"] == 3:
            return oracle.geodesic3d(im[0], m[0], w["spacing"], w["v"], lamb, w["iters"])
        return oracle.geodesic2d(im[0], m[0], w["v"], lamb, w["iters"])

    return f, "port", cores


def time_cpu_sample(w, kind_pref="reference", max_runs=None, budget_s=20.0):
    """Times single transforms (cycling through the workload's transforms)
    until about `budget_s` seconds of CPU work; returns Gvp/s and a description."""
    f, kind, cores = cpu_transform_fn(kind_pref)
    if w.get("method") == "toivanen":
        cores = 1  # Toivanen's scan is sequential in the reference (and the port)
    vp_one = voxel_passes(w) / len(w["lambs"])
    f(w, w["lambs"][0], 0)  # warm-up (page-in, thread pool)
    t_total, runs = 0.0, 0
    while True:
        lamb = w["lambs"][runs % len(w["lambs"])]
        t0 = time.perf_counter()
        f(w, lamb, runs)
        t_total += time.perf_counter() - t0
        runs += 1
        if (max_runs and runs >= max_runs) or (not max_runs and t_total >= budget_s) or runs >= 30:
            break
    value = vp_one * runs / t_total / 1e9
    sample = f"{runs} single transforms of the workload (lamb cycling {w['lambs']}), {t_total:.2f} s total"
    return value, kind, cores, sample


def reference_cuda_record(FG, w, steps):
    """The reference's own CUDA kernels (fastgeodis_cuda.cu:131-318, :407-656,
    built for sm_103a) on the workload's step, timed with CUDA events on the
    stream they launch on (the legacy default stream, which is torch's
    default stream), and their difference from the oracle (the reference's
    CPU semantics): the reference's thread blocks read neighbour cells at
    their seams without ordering, so cells there may differ."""
    import torch

    from oracle import oracle

    if w.get("method") == "toivanen" or not torch.cuda.is_available():
        return None
    dev = torch.device("cuda", torch.cuda.current_device())
    pairs = w.get("images") or [(w["image"], w["mask"])] * len(w["lambs"])
    d_in = [(torch.from_numpy(im).to(dev), torch.from_numpy(m).to(dev)) for im, m in pairs]
    call = reference_call(FG, w)

    def step():
        return [call(im, m, lamb) for (im, m), lamb in zip(d_in, w["lambs"])]

    try:
        step()
        torch.cuda.synchronize()
    except Exception as exc:  # built without its CUDA path
        return {"unavailable": f"{type(exc).__name__}: {str(exc).splitlines()[0][:200]}"}
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    tot = 0.0
    for k in range(steps):
        flush.fill_(float(k))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        outs = step()
        e1.record(stream)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    ms = tot / steps
    worst = {"max_abs_diff": 0.0, "max_rel_diff": 0.0, "cells_differing": 0, "cells_compared": 0}
    for (im, m), lamb, o in list(zip(pairs, w["lambs"], outs))[:3]:
        want = (oracle.geodesic3d(im[0], m[0], w["spacing"], w["v"], lamb, w["iters"]) if w["dims"] == 3
                else oracle.geodesic2d(im[0], m[0], w["v"], lamb, w["iters"]))
        got = o[0].cpu().numpy()
        d = np.abs(got.astype(np.float64) - want.astype(np.float64))
        worst["max_abs_diff"] = max(worst["max_abs_diff"], float(d.max()))
        worst["max_rel_diff"] = max(worst["max_rel_diff"],
                                    float((d / np.maximum(np.abs(want.astype(np.float64)), 1e-30)).max()))
        worst["cells_differing"] += int(np.count_nonzero(got.view(np.uint32) != want.view(np.uint32)))
        worst["cells_compared"] += int(got.size)
    return {"value": round(voxel_passes(w) / (ms * 1e-3) / 1e9, 4), "unit": "Gvoxel-passes/s",
            "ms_per_step": round(ms, 3), "steps": steps,
            "timing": "CUDA events on the legacy default stream, inputs resident, L2 flushed between steps",
            "vs_oracle": worst, "build": "the reference's fastgeodis_cuda.cu for sm_103a, nvcc defaults (FMA on)"}


def signed_gsf_record(FG, repeats=3):
    """The reference's signed and GSF transforms on the host cores, as it
    calls them (fastgeodis.cpp:241-258, :319-343: the second transform of a
    signed pair in a std::async thread) and as sequential plain calls (2 per
    signed, 6 per GSF), on the 512^2 image of the 2D workload."""
    import torch

    w = workload("c1")
    img, m = torch.from_numpy(w["image"]), torch.from_numpy(w["mask"])
    lamb, it, v = 1.0, 2, 1e10

    def med(fn):
        fn()
        ts = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts))

    def plain_pairs(n):
        def fn():
            for k in range(n):
                FG.generalised_geodesic2d(img, m if k % 2 == 0 else 1 - m, v, lamb, it)
        return fn

    t_signed = med(lambda: FG.signed_generalised_geodesic2d(img, m, v, lamb, it))
    t_2 = med(plain_pairs(2))
    t_gsf = med(lambda: FG.GSF2d(img, m, 0.5, v, lamb, it))
    t_6 = med(plain_pairs(6))
    return {"image": "1x1x512x512 (the 2D workload), lamb 1.0, iterations 2", "repeats": repeats,
            "signed2d_s": round(t_signed, 4), "two_sequential_plain_s": round(t_2, 4),
            "GSF2d_s": round(t_gsf, 4), "six_sequential_plain_s": round(t_6, 4),
            "note": "median seconds; the reference's signed/GSF run each pair's second transform in a std::async "
                    "thread beside the first, two OpenMP teams on the same cores"}


def signed_gsf_gpu_record(fg, repeats=5):
    """This engine's plain, signed and GSF transforms of the 2D workload's
    512^2 image on the device (CUDA events, median of `repeats` after
    warm-up): the counterpart of the reference arm's signed_gsf_cpu record.
    A signed transform sweeps both maps in each pass; GSF is a signed
    transform, thresholds and a second signed transform."""
    import torch

    w = workload("c1")
    img, m = (torch.from_numpy(a).cuda() for a in (w["image"], w["mask"]))
    lamb, it, v = 1.0, 2, 1e10

    def med(fn):
        fn()
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    t_plain = med(lambda: fg.generalised_geodesic2d(img, m, v, lamb, it))
    t_signed = med(lambda: fg.signed_generalised_geodesic2d(img, m, v, lamb, it))
    t_gsf = med(lambda: fg.GSF2d(img, m, 0.5, v, lamb, it))
    return {"image": "1x1x512x512 (the 2D workload), lamb 1.0, iterations 2, theta 0.5 for GSF", "repeats": repeats,
            "plain2d_ms": round(t_plain, 4), "signed2d_ms": round(t_signed, 4), "GSF2d_ms": round(t_gsf, 4),
            "note": "median device milliseconds through the public API, inputs resident"}


def run_reference_arm(args, w, rank, world):
    """The reference's own implementation on the workload, on all host cores:
    its installed package (OpenMP CPU path) where it could be built here,
    else its CPU sources (oracle/_ref), else the C restatement."""
    if rank != 0:
        return
    f, kind, cores = cpu_transform_fn("reference", build=True)
    if w.get("method") == "toivanen":
        cores = 1  # Toivanen's scan is sequential in the reference (and the port)
    units = [(k, lamb) for k, lamb in enumerate(w["lambs"])]
    vp_unit = voxel_passes(w) / len(units)
    t0 = time.perf_counter()
    f(w, units[0][1], units[0][0])  # page-in, thread pool
    t_unit = time.perf_counter() - t0
    # a step is the GPU arm's step (every transform of the workload) when it
    # fits in about 4 s of CPU time, else one transform, cycling
    whole = t_unit * len(units) <= 4.0
    per_step = units if whole else None

    def step(i):
        todo = per_step if per_step else [units[i % len(units)]]
        for k, lamb in todo:
            f(w, lamb, k)
        return len(todo)

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    done = sum(step(i) for i in range(args.steps))
    dt = time.perf_counter() - t0
    value = vp_unit * done / dt / 1e9
    line = {
        "impl": "reference",
        "metric": metric_name(w), "value": round(value, 4), "unit": "Gvoxel-passes/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["desc"],
                   "step": ("every transform of the workload per step, as the GPU arm's step" if whole else
                            "one transform per step, cycling through the workload's transforms"),
                   "implementation": {"reference": "the reference's FastGeodis package and its FastGeodisCpp "
                                                   "OpenMP CPU path, built on this host",
                                      "port": "the oracle's C restatement of the reference's CPU path"}[kind]},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gvoxel-passes/s", "cores": cores, "kind": kind,
                         "sample": f"{args.steps} steps ({done} transforms) after {args.warmup} warm-up steps"},
        "e2e": {"value": round(value, 4), "unit": "Gvoxel-passes/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    FG = reference_install(build=False) if kind == "reference" else None
    if FG is not None:
        try:
            rc = reference_cuda_record(FG, w, max(1, min(args.steps, 5)))
            if rc:
                line["reference_cuda"] = rc
        except Exception as exc:
            line["reference_cuda"] = {"unavailable": f"{type(exc).__name__}: {str(exc)[:200]}"}
        if w["name"] in ("c1", "c2") and not args.no_signed_gsf:
            line["signed_gsf_cpu"] = signed_gsf_record(FG)
    print(json.dumps(line), flush=True)


def _one_launch(w):
    """Whether the workload's transforms each run in one launch (a 2D image
    the per-call path hands to the one-CTA kernel)."""
    from fastgeodis_gb300 import _lib

    return w["dims"] == 2 and _lib.runs_in_one_launch(w["image"].shape[2:])


def sweep_kernel_name(w, tuned):
    """The kernel of the workload's sweep passes: the pinned plans' kind."""
    if w.get("method") == "toivanen":
        return "fg_toivanen_kernel"
    if _one_launch(w):
        return "fg_row2d_kernel"
    from fastgeodis_gb300 import _lib, tune

    plans = (tuned or {}).get("plans", {})
    sms = torch_sms()
    flags = []
    for key in tune.pass_keys(w["image"].shape[2:]):
        v = plans.get(",".join(map(str, key)))
        # a pinned plan's flags, else the planner's plan for the pass
        flags.append(int(v[3]) if v and int(v[0]) > 0 else
                     _lib.plan_describe(*key, C=int(w["image"].shape[1]), sms=sms)["lean"])
    flags += [int(v[3]) for k, v in plans.items() if k.count(",") == 3 and int(v[0]) > 0]  # per-mode plans
    names = []
    for f in flags:
        name = ("fg_row_tile_kernel" if f & _lib.FG_PLAN_ROWS else
                "fg_sweep_cluster_kernel" if f & _lib.FG_PLAN_RUNS2 else
                "fg_pass_cluster_kernel" if f & _lib.FG_PLAN_CLUSTER else "fg_pass_kernel")
        if name not in names:
            names.append(name)
    return " + ".join(names)  # the sweep kernels of the transform's passes


def torch_sms():
    """SMs of the current device (152 without one: the planner's default)."""
    import torch

    if not torch.cuda.is_available():
        return 152
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def metric_name(w):
    name = "generalised_geodesic3d" if w["dims"] == 3 else "generalised_geodesic2d"
    return name + ("_toivanen" if w.get("method") == "toivanen" else "") + " throughput"


def transform_fns(fg, w):
    """The public functions of the workload's method: (3D, 2D)."""
    if w.get("method") == "toivanen":
        return fg.generalised_geodesic3d_toivanen, fg.generalised_geodesic2d_toivanen
    return fg.generalised_geodesic3d, fg.generalised_geodesic2d


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def smooth_noise_gpu(gen, shape, sigma, lo, hi, dev):
    """uniform[lo, hi] noise from `gen`, Gaussian-smoothed on the device
    (separable kernel truncated at 4 sigma, reflected borders), float32."""
    import torch
    import torch.nn.functional as F

    x = (torch.rand(shape, generator=gen, device=dev) * (hi - lo) + lo)[None, None]
    r = int(4 * sigma + 0.5)
    t = torch.arange(-r, r + 1, dtype=torch.float32, device=dev)
    k = torch.exp(-0.5 * (t / sigma) ** 2)
    k = k / k.sum()
    nd = len(shape)
    conv = F.conv3d if nd == 3 else F.conv2d
    for ax in range(nd):
        if shape[ax] <= r:
            continue
        pad = [0, 0] * nd
        pad[2 * (nd - 1 - ax)] = pad[2 * (nd - 1 - ax) + 1] = r
        view = [1, 1] + [1] * nd
        view[2 + ax] = 2 * r + 1
        x = conv(F.pad(x, pad, mode="reflect"), k.view(view))
    return x[0, 0].contiguous()


def _max_over_ranks(x, dist, dev):
    if not dist:
        return x
    import torch

    t = torch.tensor([float(x)], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def b256_record(args, dev, rank, world, dist, n=8, steps=5):
    """The batched-volume target (>= 60% of the HBM roofline on 256^3): a batch of
    8 volumes 256^3 (smoothed noise generated on the device, one 6^3 seed cube
    each, spacing 1, iterations 4, lamb cycling 0 / 0.5 / 1), one transform per
    volume, through GeodesicBatch3d (cluster plans pinned by the batch,
    replayed from one CUDA graph).  Volumes are split across ranks."""
    import torch

    import fastgeodis_gb300 as fg
    from fastgeodis_gb300.replicas import partition

    shape = (256, 256, 256)
    mine = partition([1.0] * n, world)[rank]
    gen = torch.Generator(device=dev).manual_seed(256)
    rng = np.random.default_rng(256)
    imgs, msks, lambs = [], [], []
    for k in range(n):
        vol = smooth_noise_gpu(gen, shape, 2.0, 0.0, 1.0, dev)
        c = [int(rng.integers(0, s - 6)) for s in shape]
        if k not in mine:
            continue
        m = torch.ones(shape, device=dev)
        m[c[0]:c[0] + 6, c[1]:c[1] + 6, c[2]:c[2] + 6] = 0.0
        imgs.append(vol[None, None])
        msks.append(m[None, None])
        lambs.append([0.0, 0.5, 1.0][k % 3])
    b = fg.GeodesicBatch3d([(1,) + shape] * len(imgs), iterations=4, use_graph=False, streams=max(1, len(imgs)),
                           inputs=(imgs, msks), device=dev)
    b.v, b.lambs, b.spacings = 1e10, lambs, [(1.0, 1.0, 1.0)] * len(imgs)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def timed_batch(run):
        for _ in range(2):
            run()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        tot = 0.0
        for k in range(steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run()
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        return _max_over_ranks(tot / steps, dist, dev)

    # launched from the host each step (the block scheduler honours the
    # streams' priorities), then replayed from one captured CUDA graph
    ms = timed_batch(b.run)
    b.use_graph = True
    ms_graph = timed_batch(b.run)
    b.check()
    plans = sorted({str(fg_plan) for fg_plan in b._pinned})
    b.release_plans()
    streamed = [o.clone() for o in b.outputs]
    del b
    # the same batch in one persistent launch (a job queue over co-resident clusters)
    pb = fg.PersistentBatch3d([(1,) + shape] * len(imgs), iterations=4, use_graph=True, inputs=(imgs, msks),
                              device=dev)
    pb.v, pb.lambs, pb.spacings = 1e10, lambs, [(1.0, 1.0, 1.0)] * len(imgs)
    for _ in range(2):
        pb.run()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    tot1 = 0.0
    for k in range(steps):
        flush.fill_(float(k))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pb.run()
        e1.record(stream)
        e1.synchronize()
        tot1 += e0.elapsed_time(e1)
    pb.check()
    same = all(torch.equal(a.view(torch.int32), o.view(torch.int32)) for a, o in zip(streamed, pb.outputs))
    ms1 = _max_over_ranks(tot1 / steps, dist, dev)
    pinfo = dict(pb.info)
    del pb, imgs, msks, streamed
    torch.cuda.empty_cache()
    vp = float(n) * float(np.prod(shape)) * 6 * 4
    value = vp / (ms * 1e-3) / 1e9
    value1 = vp / (ms1 * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    return {"workload": "8 volumes 1x1x256x256x256, smoothed (sigma 2) uniform[0,1] noise generated on the device, "
                        "one 6^3 seed cube each, spacing 1, v 1e10, iterations 4, lamb cycling 0/0.5/1",
            "api": "GeodesicBatch3d, 8 priority streams launched from the host each step, cluster plans pinned "
                   "by the batch",
            "plans_pinned_for": plans, "steps": steps, "ms_per_step": round(ms, 3),
            "value": round(value, 2), "unit": "Gvoxel-passes/s",
            "graph_replay": {"ms_per_step": round(ms_graph, 3),
                             "value": round(vp / (ms_graph * 1e-3) / 1e9, 2),
                             "note": "the same batch replayed from one captured CUDA graph"},
            "hbm_achieved_gbs": round(value * 12, 1), "hbm_frac": round(value * 12 / peak, 4),
            "peak_gbs": peak, "peak_source": peak_kind, "target_frac": 0.6,
            "bytes_per_voxel_pass": 12, "l2": "flushed between steps",
            "one_launch": {"api": "PersistentBatch3d: every volume's prologue and passes in one job queue, one "
                                  "persistent launch of co-resident clusters, one CUDA graph per step",
                           "ms_per_step": round(ms1, 3), "value": round(value1, 2),
                           "hbm_frac": round(value1 * 12 / peak, 4), "launch": pinfo,
                           "bits_equal_to_streamed": bool(same)}}


def c3_record(args, dev, rank, world, dist, steps=5):
    """The uneven-batch target (>= 5x the plain per-call drop-in on the uneven 2D
    batch): the 64-image batch, plain and signed of every image, through
    GeodesicBatch2d (one CUDA graph) against the same transforms called one
    by one through the drop-in API.  Images are split across ranks."""
    import torch

    import fastgeodis_gb300 as fg
    from fastgeodis_gb300.replicas import partition, transform_cost

    items = batch_workload()
    mine = partition([transform_cost(tuple(im.shape[2:]), 2) for im, _, _ in items], world)[rank]
    items = [items[i] for i in mine]
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im, _, _ in items]
    n = len(items)
    plan = fg.GeodesicBatch2d(shapes + shapes, signed=[False] * n + [True] * n, iterations=2, use_graph=True,
                              inputs=([im for im, _, _ in items] * 2, [m for _, m, _ in items] * 2))
    plan.v, plan.lambs = 1e10, [l for _, _, l in items] * 2
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def per_call():
        for im, m, l in items:
            fg.generalised_geodesic2d(im, m, 1e10, l, 2)
            fg.signed_generalised_geodesic2d(im, m, 1e10, l, 2)

    def timed(fn, k_steps):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        tot = 0.0
        for k in range(k_steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        return _max_over_ranks(tot / k_steps, dist, dev)

    ms_b = timed(plan.run, steps)
    plan.check()
    ms_p = timed(per_call, 2)
    fg.check_status()
    tiled = len(plan.tiled)
    del plan
    torch.cuda.empty_cache()
    vp_all = _sum_over_ranks(float(sum(s[1] * s[2] for s in shapes)) * 4 * 2 * 3, dist, dev)
    return {"workload": "64 images H,W ~ U[128,2048] step 4, C in {1,3}, smoothed noise [0,255], 1-10 seed disks, "
                        "lamb ~ U[0,1], iterations 2; plain and signed of every image",
            "api": "GeodesicBatch2d (one persistent launch + tiled launch, one CUDA graph) vs the per-call drop-in",
            "tiled_images": tiled, "steps": steps,
            "batched_ms_per_step": round(ms_b, 3), "batched_value": round(vp_all / (ms_b * 1e-3) / 1e9, 2),
            "per_call_ms_per_step": round(ms_p, 3), "per_call_value": round(vp_all / (ms_p * 1e-3) / 1e9, 2),
            "speedup_vs_per_call": round(ms_p / ms_b, 2), "target_speedup": 5.0, "unit": "Gvoxel-passes/s",
            "l2": "flushed between steps"}


def _sum_over_ranks(x, dist, dev):
    if not dist:
        return x
    import torch

    t = torch.tensor([float(x)], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_gpu_arm(args, w, rank, world):
    import torch

    import fastgeodis_gb300 as fg
    from fastgeodis_gb300 import _lib

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    # a batch of independent volumes is split across ranks (no collective on
    # the data path); a single-image workload is replicated on every rank
    vp_all = voxel_passes(w) * (1 if w.get("images") else world)
    if w.get("images") and world > 1:
        from fastgeodis_gb300.replicas import partition

        mine = partition([float(np.prod(im.shape)) for im, _ in w["images"]], world)[rank]
        w = dict(w, images=[w["images"][i] for i in mine], lambs=[w["lambs"][i] for i in mine])
    # inputs of the step's transforms: one (image, mask) per transform, or the
    # workload's one image for all (several lambs of one image)
    pairs = w.get("images") or [(w["image"], w["mask"])] * len(w["lambs"])
    d_in, cache = [], {}
    for im_np, mk_np in pairs:
        if id(im_np) not in cache:
            cache[id(im_np)] = (torch.from_numpy(im_np).to(dev), torch.from_numpy(mk_np).to(dev))
        d_in.append(cache[id(im_np)])
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    tuned = None
    if args.plans and w.get("method") != "toivanen":
        # plans tuned by an earlier run (--save-plans): a profiler serialises
        # the kernels, so plans tuned under it would be tuned for no concurrency
        from fastgeodis_gb300 import tune

        res = tune.load(args.plans)
        tuned = {"plans": {",".join(map(str, k)): [int(x) for x in v[:4]] for k, v in res.items()},
                 "note": f"loaded from {os.path.basename(args.plans)} (--plans)"}
    elif (args.tune and w.get("method") != "toivanen"
          and not _one_launch(w)):
        # untimed: plans of the step's transforms run together (small images
        # run in one launch and have no pass plans to tune)
        from fastgeodis_gb300 import tune

        shape = tuple(w["image"].shape[2:])
        t_tune = time.perf_counter()
        res = tune.autotune(shape, channels=int(w["image"].shape[1]), lambs=w["lambs"],
                            spacing=w.get("spacing", (1.0, 1.0, 1.0)), iterations=1)
        if args.save_plans and rank == 0:
            tune.save(res, args.save_plans)
        tuned = {"plans": {",".join(map(str, k)): [v[0], v[1], v[2], v[3]] for k, v in res.items()},
                 "note": "(cross, N1, N2): (S, T1, T2, flags: 1 = 64-register kernel, 2 = cluster plan); "
                         "S = 0 keeps the cost model's plan",
                 "seconds": round(time.perf_counter() - t_tune, 2)}

    # the step's transforms are independent: one CUDA stream each, so their
    # passes share the SMs (each call runs on the current stream); the
    # costliest arithmetic goes first, on the highest-priority stream, since
    # the step ends with its slowest transform
    from fastgeodis_gb300.batch3d import priority_streams, transform_cost

    main = torch.cuda.current_stream()
    n_tr = len(w["lambs"])
    vol = tuple(int(x) for x in d_in[0][0].shape[1:])
    vol = vol if len(vol) == 4 else (vol[0], 1) + vol[1:]
    order = sorted(range(n_tr), key=lambda i: -transform_cost(vol, w["lambs"][i]))
    by_rank = priority_streams(n_tr)
    streams = [None] * n_tr
    for r, i in enumerate(order):
        streams[i] = by_rank[r]

    f3, f2 = transform_fns(fg, w)

    def step(inputs):
        outs = [None] * n_tr
        for s in streams:
            s.wait_stream(main)
        for i in order:
            lamb, s, (im, mk) = w["lambs"][i], streams[i], inputs[i]
            with torch.cuda.stream(s):
                if w["dims"] == 3:
                    outs[i] = f3(im, mk, w["spacing"], w["v"], lamb, w["iters"])
                else:
                    outs[i] = f2(im, mk, w["v"], lamb, w["iters"])
        for s in streams:
            main.wait_stream(s)
        return outs

    # clocks sampled across all of this arm's GPU work (warm-up, timed steps,
    # end-to-end leg and the records below): the timed steps alone are too
    # short for nvidia-smi's sampling period
    clocks = ClockSampler(local).start()
    nvtx = torch.cuda.nvtx  # ranges let a profiler select the timed launches (ncu --nvtx-include timed/)
    nvtx.range_push("warmup")
    for _ in range(args.warmup):
        step(d_in)
    torch.cuda.synchronize()
    nvtx.range_pop()
    fg.check_status()

    stream = torch.cuda.current_stream()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    _lib.profile_begin()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))  # evict the inputs from L2 between steps (outside the timed events)
        nvtx.range_push("timed")
        starts[k].record(stream)
        step(d_in)
        ends[k].record(stream)
        nvtx.range_pop()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    pass_ms, pass_launches, pass_vp = _lib.profile_end()
    aux_launches = _lib.profile_aux_launches()
    if dist:
        dist.barrier()
    fg.check_status()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = float(np.sum(step_ms) / args.steps)
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    vp_step = voxel_passes(w)
    value = vp_all / (ms * 1e-3) / 1e9

    if args.kernels_only:
        clocks.stop()
        if rank == 0:
            print(json.dumps({"kernels_only": True, "ms_per_step": round(ms, 4), "pass_launches": pass_launches}))
        return
    graph_batch = None
    if w.get("images") and w["dims"] == 3 and w.get("method") != "toivanen":
        # the same batch through the batched API, replayed from one CUDA graph
        # (the plans pinned above stay in force)
        b = fg.GeodesicBatch3d([tuple(int(x) for x in im.shape[1:]) for im, _ in d_in], iterations=w["iters"],
                               use_graph=True, streams=len(d_in), inputs=([im for im, _ in d_in], [mk for _, mk in d_in]),
                               plans=None, device=dev)
        b.v, b.lambs, b.spacings = w["v"], list(w["lambs"]), [tuple(w["spacing"])] * len(d_in)
        for _ in range(args.warmup):
            b.run()
        torch.cuda.synchronize()
        g_ms = []
        for k in range(args.steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.run()
            e1.record(stream)
            e1.synchronize()
            g_ms.append(e0.elapsed_time(e1))
        b.check()
        gm = float(np.mean(g_ms))
        graph_batch = {"api": f"GeodesicBatch3d, {len(d_in)} streams, one CUDA graph per step",
                       "ms_per_step": round(gm, 4), "value": round(vp_all / (gm * 1e-3) / 1e9, 4)}
    # end to end through the public API with host buffers (pinned): every call
    # copies its inputs to the device and returns its result in host memory.
    # The step's calls are independent, so each is issued from its own host
    # thread on its own stream, as a server handling them would.
    h_in, cache = [], {}
    for im_np, mk_np in pairs:
        if id(im_np) not in cache:
            cache[id(im_np)] = (torch.from_numpy(im_np).pin_memory(), torch.from_numpy(mk_np).pin_memory())
        h_in.append(cache[id(im_np)])

    def host_call(k):
        h_img, h_msk = h_in[k]
        with torch.cuda.device(dev), torch.cuda.stream(streams[k]):
            lamb = w["lambs"][k]
            if w["dims"] == 3:
                return f3(h_img, h_msk, w["spacing"], w["v"], lamb, w["iters"])
            return f2(h_img, h_msk, w["v"], lamb, w["iters"])

    from concurrent.futures import ThreadPoolExecutor

    pool = ThreadPoolExecutor(max_workers=len(w["lambs"]))

    def host_step():
        return list(pool.map(host_call, range(len(w["lambs"]))))

    for _ in range(max(1, args.warmup)):
        host_step()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e_steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(e_steps):
        host_step()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e_steps
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    pool.shutdown()

    # the dominant kernel timed alone: one transform of the step (the middle
    # lamb) on one stream, every pass launch bracketed by CUDA events, so the
    # roofline below divides by the kernel's own duration (in the step above
    # three transforms share the SMs)
    alone = None
    if w.get("method") != "toivanen" and not _one_launch(w):
        ka = len(w["lambs"]) // 2
        im_a, mk_a = d_in[ka]
        n_alone = max(3, min(args.steps, 10))
        for _ in range(2):
            f3(im_a, mk_a, w["spacing"], w["v"], w["lambs"][ka], w["iters"]) if w["dims"] == 3 else \
                f2(im_a, mk_a, w["v"], w["lambs"][ka], w["iters"])
        torch.cuda.synchronize()
        _lib.profile_begin()
        for k in range(n_alone):
            flush.fill_(float(k))
            if w["dims"] == 3:
                f3(im_a, mk_a, w["spacing"], w["v"], w["lambs"][ka], w["iters"])
            else:
                f2(im_a, mk_a, w["v"], w["lambs"][ka], w["iters"])
        torch.cuda.synchronize()
        a_ms, a_launches, a_vp = _lib.profile_end()
        alone = {"lamb": w["lambs"][ka], "transforms": n_alone, "pass_ms": a_ms, "launches": a_launches, "vp": a_vp}
    extra = {}
    sg = signed_gsf_gpu_record(fg) if w["name"] in ("c1", "c2") and not args.kernels_only else None
    if w["name"] == "c2" and not args.no_extras:
        # the batch targets, measured in the same run (outside the timed steps)
        extra["b256"] = b256_record(args, dev, rank, world, dist)
        extra["c3"] = c3_record(args, dev, rank, world, dist)
    clk = clocks.stop()
    n_calls = len(w["lambs"])
    h2d = sum((im.numel() + mk.numel()) * 4 for im, mk in h_in)
    d2h = sum(mk.numel() * 4 for _, mk in h_in)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # roofline of the dominant kernel (the sweep pass): algorithmic bytes per
    # launch = cells x (4*C image bytes + 4 read + 4 write of the distance)
    bytes_per_vp = 4 * w["C"] + 8
    avg_launch_ms = pass_ms / max(pass_launches, 1)
    alg_bytes_launch = pass_vp / max(pass_launches, 1) * bytes_per_vp
    achieved_step = alg_bytes_launch / (avg_launch_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic = committed_traffic(w["name"])
    if alone:
        avg_alone = alone["pass_ms"] / max(alone["launches"], 1)
        bytes_alone = alone["vp"] / max(alone["launches"], 1) * bytes_per_vp
        achieved = bytes_alone / (avg_alone * 1e-3) / 1e9
    else:
        avg_alone, bytes_alone, achieved = avg_launch_ms, alg_bytes_launch, achieved_step
    # per transform besides the passes: the v*mask initialisation and the
    # image transpose (Toivanen's scan: initialisation only; a 2D image in one
    # launch: none, its one kernel is the pass launch)
    per_call = (0 if sweep_kernel_name(w, tuned) == "fg_row2d_kernel" else
                1 if w.get("method") == "toivanen" else 2)
    init_launches = n_calls * args.steps * per_call
    cpu_val, cpu_kind, cpu_cores, cpu_sample = time_cpu_sample(w, "reference", budget_s=args.cpu_budget)
    f64 = None
    if w.get("method") != "toivanen":
        # the transform of the step with the middle lamb, against the float64 scan
        k = len(w["lambs"]) // 2
        im, mk = d_in[k]
        lamb = w["lambs"][k]
        out = (f3(im, mk, w["spacing"], w["v"], lamb, w["iters"]) if w["dims"] == 3
               else f2(im, mk, w["v"], lamb, w["iters"]))
        f64 = fp64_check(out[0].cpu().numpy(), im[0].cpu().numpy(), mk[0].cpu().numpy(), w["v"], lamb, w["iters"],
                         spacing=w["spacing"] if w["dims"] == 3 else None)
    line = {
        "metric": metric_name(w), "value": round(value, 4), "unit": "Gvoxel-passes/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": w["desc"], "parallelism": f"replicas x{world}",
                   "streams": f"{len(w['lambs'])} transforms per step on {len(w['lambs'])} CUDA streams",
                   "plans": ({"autotuned": tuned} if tuned else
                             "wavefront, no plan" if w.get("method") == "toivanen" else
                             "the whole transform in one launch, no pass plans"
                             if sweep_kernel_name(w, None) == "fg_row2d_kernel" else "cost model"),
                   "l2": f"flushed between steps ({FLUSH_BYTES >> 20} MiB write outside the timed events)",
                   "wall_s_timed_region": round(wall, 4),
                   **({"graph_batch": graph_batch} if graph_batch else {}),
                   **({"fp64_check": f64} if f64 else {})},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "traffic_source": ("dram__bytes_read.sum + dram__bytes_write.sum per launch from an ncu "
                                        "capture committed in profiles/traffic.json, not measured in this run"
                                        if traffic else None),
                     "kernel": sweep_kernel_name(w, tuned),
                     "avg_launch_ms": round(avg_alone, 5),
                     "alg_bytes_per_launch": int(bytes_alone), "peak_source": peak_kind,
                     "measured": ("one transform of the step (lamb %s) alone on one stream, %d launches, CUDA events "
                                  "around each launch" % (alone["lamb"], alone["launches"]) if alone else
                                  "the timed steps' launches"),
                     "in_step": {"avg_launch_ms": round(avg_launch_ms, 5), "achieved": round(achieved_step, 1),
                                 "frac": round(achieved_step / peak, 4),
                                 "note": "launches of the timed steps, where the step's transforms share the SMs"},
                     "pass_time_share": round(pass_ms / (ms * args.steps), 4),
                     "achieved_aggregate": round(pass_vp * bytes_per_vp / (ms * args.steps * 1e-3) / 1e9, 1),
                     "frac_aggregate": round(pass_vp * bytes_per_vp / (ms * args.steps * 1e-3) / 1e9 / peak, 4)},
        "cpu_baseline": {"value": round(cpu_val, 4), "unit": "Gvoxel-passes/s", "cores": cpu_cores,
                         "kind": cpu_kind, "sample": cpu_sample},
        "e2e": {"value": round(vp_all / e2e_s / 1e9, 4), "unit": "Gvoxel-passes/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "path": f"public API with pinned host tensors, {n_calls} calls per step from {n_calls} host threads"},
        "clocks": clk,
        "gpu_launches": int((pass_launches + aux_launches + init_launches) / args.steps),
        **({"batch_targets": extra} if extra else {}),
        **({"signed_gsf_gpu": sg} if sg else {}),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def spawn_ranks(n: int, argv) -> int:
    """Re-launch this script as n ranks on this node (torch.distributed.run,
    one process per GPU, rendezvous on 127.0.0.1); returns its exit code.
    NCCL's own log stays on (NCCL_DEBUG=INFO unless set), so the ranks of
    every communicator are visible on stderr."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *argv]
    env = dict(os.environ)
    env.setdefault("NCCL_DEBUG", "INFO")
    return subprocess.call(cmd, env=env)


def run_dry(args, rank, world):
    """The multi-rank plumbing without the workload: process group (NCCL on
    GPUs, gloo without), barrier, the max-over-ranks reduction of a per-rank
    time, and rank 0's line with the world size."""
    import torch
    import torch.distributed as dist

    t = float(rank + 1)
    if world > 1:
        gpu = torch.cuda.is_available() and torch.cuda.device_count() >= world and args.impl == "ours"
        if gpu:
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl" if gpu else "gloo")
        dist.barrier()
        x = torch.tensor([t], device="cuda" if gpu else "cpu")
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
        dist.destroy_process_group()
    if rank == 0:
        line = {"dry_run": True, "n_gpus": world, "max_over_ranks": t}
        if args.impl == "reference":
            line["impl"] = "reference"
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "vol256", "slab", "b256", "c3", "c4", "c5", "t1", "t2"])
    ap.add_argument("--requests", type=int, default=300, help="requests of the served stream (c5)")
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU baseline sampling")
    ap.add_argument("--no-tune", dest="tune", action="store_false",
                    help="use the cost model's plans instead of autotuning the workload's shape before warm-up")
    ap.add_argument("--save-plans", default=None, help="write the autotuned plans to this JSON file")
    ap.add_argument("--plans", default=None, help="pin plans from this JSON file (from --save-plans) instead of tuning")
    ap.add_argument("--kernels-only", action="store_true",
                    help="run warm-up and timed GPU steps only (no end-to-end or CPU legs): for profiler captures")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batch-target records (batch of 256^3 volumes, uneven 2D batch) of the default run")
    ap.add_argument("--no-signed-gsf", action="store_true",
                    help="reference arm: skip the signed / GSF timings of the reference's CPU path")
    ap.add_argument("--dry-run", action="store_true",
                    help="only the multi-rank plumbing (spawn, rendezvous, max over ranks): no workload")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: launched here when the caller did not use torchrun
        sys.exit(spawn_ranks(args.gpus, sys.argv[1:]))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.dry_run:
        run_dry(args, rank, world)
        return
    if args.workload == "c5":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no server"}))
            return
        run_serve_arm(args, rank, world)
        return
    if args.workload == "c4":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no gradient"}))
            return
        run_grad_arm(args, rank, world)
        return
    if args.workload == "c3":
        if args.impl == "reference":
            run_batch_reference_arm(args, rank, world)
            return
        run_batch_arm(args, rank, world)
        return
    w = workload(args.workload)
    if args.impl == "reference":
        run_reference_arm(args, w, rank, world)
        return
    run_gpu_arm(args, w, rank, world)


if __name__ == "__main__":
    main()
