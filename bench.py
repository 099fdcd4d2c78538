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
    rng = np.random.default_rng(seed)
    if name in ("c2", "vol256"):
        shape = (128, 256, 256) if name == "c2" else (256, 256, 256)
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


def run_batch_arm(args, rank, world):
    """Uneven 2D batch: the batched persistent launch (CUDA graph) against the
    plain per-call drop-in path, both on device-resident inputs."""
    import torch

    import fastgeodis_gb300 as fg

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    items = batch_workload()
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im, _, _ in items]
    plans = []
    for signed in (False, True):
        p = fg.GeodesicBatch2d(shapes, signed=signed, iterations=2, use_graph=True,
                               inputs=([im for im, _, _ in items], [m for _, m, _ in items]))
        p.v, p.lambs = 1e10, [l for _, _, l in items]
        plans.append(p)
    vp = float(sum(s[1] * s[2] for s in shapes)) * 4 * 2 * 3  # plain + signed (2 transforms)
    flush = torch.empty(FLUSH_BYTES // 4, device="cuda")

    def batched():
        for p in plans:
            p.run()

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
    h_outs = [torch.empty(o.shape, pin_memory=True) for o in plans[0].outputs]

    def e2e_step():
        for i in range(len(items)):
            plans[0].images[i].copy_(h_imgs[i], non_blocking=True)
            plans[0].masks[i].copy_(h_msks[i], non_blocking=True)
        batched()
        for p in plans:
            for i, o in enumerate(p.outputs):
                h_outs[i].copy_(o, non_blocking=True)
        torch.cuda.synchronize()

    for _ in range(max(1, args.warmup)):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    h2d = sum(t.numel() * 4 for t in h_imgs + h_msks)
    d2h = 2 * sum(o.numel() * 4 for o in plans[0].outputs)
    if rank != 0:
        return
    line = {
        "metric": "generalised_geodesic2d uneven batch throughput", "value": round(vp / ms_b / 1e6, 4),
        "unit": "Gvoxel-passes/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_b, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "64 images H,W ~ U[128,2048] step 4, C in {1,3}, smoothed noise [0,255], "
                               "1-10 seed disks, lamb ~ U[0,1], iterations 2; plain and signed per step",
                   "path": "GeodesicBatch2d (one persistent launch per variant, CUDA graph)",
                   "per_call_value": round(vp / ms_p / 1e6, 4), "per_call_ms_per_step": round(ms_p, 3),
                   "speedup_vs_per_call": round(ms_p / ms_b, 2),
                   "l2": f"flushed between steps ({FLUSH_BYTES >> 20} MiB write outside the timed events)"},
        "e2e": {"value": round(vp / e2e_s / 1e9, 4), "unit": "Gvoxel-passes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "clocks": clk, "gpu_launches": 2,
    }
    print(json.dumps(line), flush=True)


def voxel_passes(w) -> float:
    n = float(np.prod(w["image"].shape[2:]))
    per = 6 if w["dims"] == 3 else 4
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

def cpu_transform_fn(kind_pref="reference"):
    """Returns (callable(w, lamb), kind, cores).  kind 'reference' = the
    reference's own CPU build (where its sources were available to compile),
    'port' = the C restatement in oracle/."""
    from oracle import build_oracle, oracle

    ref = build_oracle.load_reference() if kind_pref == "reference" else None
    if ref is not None:
        import torch

        cores = torch.get_num_threads()

        def f(w, lamb):
            img = torch.from_numpy(w["image"])
            m = torch.from_numpy(w["mask"])
            if w["dims"] == 3:
                return ref.generalised_geodesic3d(img, m, w["spacing"], w["v"], lamb, 1 - lamb, w["iters"])
            return ref.generalised_geodesic2d(img, m, w["v"], lamb, 1 - lamb, w["iters"])

        return f, "reference", cores
    cores = oracle.max_threads()

    def f(w, lamb):
        if w["dims"] == 3:
            return oracle.geodesic3d(w["image"][0], w["mask"][0], w["spacing"], w["v"], lamb, w["iters"])
        return oracle.geodesic2d(w["image"][0], w["mask"][0], w["v"], lamb, w["iters"])

    return f, "port", cores


def time_cpu_sample(w, kind_pref="reference", max_runs=None, budget_s=20.0):
    """Times single transforms (cycling through the workload's lambs) until
    about `budget_s` seconds of CPU work; returns Gvp/s and a description."""
    f, kind, cores = cpu_transform_fn(kind_pref)
    vp_one = voxel_passes(w) / len(w["lambs"])
    f(w, w["lambs"][0])  # warm-up (page-in, thread pool)
    t_total, runs = 0.0, 0
    while True:
        lamb = w["lambs"][runs % len(w["lambs"])]
        t0 = time.perf_counter()
        f(w, lamb)
        t_total += time.perf_counter() - t0
        runs += 1
        if (max_runs and runs >= max_runs) or (not max_runs and t_total >= budget_s) or runs >= 30:
            break
    value = vp_one * runs / t_total / 1e9
    sample = f"{runs} single transforms of the workload (lamb cycling {w['lambs']}), {t_total:.2f} s total"
    return value, kind, cores, sample


def run_reference_arm(args, w, rank):
    if rank != 0:
        return
    f, kind, cores = cpu_transform_fn("reference")
    vp_one = voxel_passes(w) / len(w["lambs"])
    for i in range(args.warmup):
        f(w, w["lambs"][i % len(w["lambs"])])
    t0 = time.perf_counter()
    for i in range(args.steps):
        f(w, w["lambs"][i % len(w["lambs"])])
    dt = time.perf_counter() - t0
    value = vp_one * args.steps / dt / 1e9
    line = {
        "impl": "reference",
        "metric": metric_name(w), "value": round(value, 4), "unit": "Gvoxel-passes/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["desc"], "step": "one transform per step, lamb cycling through the set"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gvoxel-passes/s", "cores": cores, "kind": kind,
                         "sample": f"{args.steps} single transforms after {args.warmup} warm-up transforms"},
        "e2e": {"value": round(value, 4), "unit": "Gvoxel-passes/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def metric_name(w):
    return ("generalised_geodesic3d throughput" if w["dims"] == 3 else "generalised_geodesic2d throughput")


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

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
    img = torch.from_numpy(w["image"]).to(dev)
    msk = torch.from_numpy(w["mask"]).to(dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step(im, mk):
        outs = []
        for lamb in w["lambs"]:
            if w["dims"] == 3:
                outs.append(fg.generalised_geodesic3d(im, mk, w["spacing"], w["v"], lamb, w["iters"]))
            else:
                outs.append(fg.generalised_geodesic2d(im, mk, w["v"], lamb, w["iters"]))
        return outs

    for _ in range(args.warmup):
        step(img, msk)
    torch.cuda.synchronize()
    fg.check_status()

    stream = torch.cuda.current_stream()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local).start()
    _lib.profile_begin()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))  # evict the inputs from L2 between steps (outside the timed events)
        starts[k].record(stream)
        step(img, msk)
        ends[k].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    pass_ms, pass_launches, pass_vp = _lib.profile_end()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    fg.check_status()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = float(np.sum(step_ms) / args.steps)
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    vp_step = voxel_passes(w)
    value = world * vp_step / (ms * 1e-3) / 1e9

    if args.kernels_only:
        if rank == 0:
            print(json.dumps({"kernels_only": True, "ms_per_step": round(ms, 4), "pass_launches": pass_launches}))
        return
    # end to end through the public API with host buffers (pinned), result read back each call
    h_img = torch.from_numpy(w["image"]).pin_memory()
    h_msk = torch.from_numpy(w["mask"]).pin_memory()
    for _ in range(max(1, args.warmup)):
        step(h_img, h_msk)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e_steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(e_steps):
        step(h_img, h_msk)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e_steps
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    n_calls = len(w["lambs"])
    h2d = n_calls * (h_img.numel() + h_msk.numel()) * 4
    d2h = n_calls * h_msk.numel() * 4

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # roofline of the dominant kernel (the sweep pass): algorithmic bytes per
    # launch = cells x (4*C image bytes + 4 read + 4 write of the distance)
    bytes_per_vp = 4 * w["C"] + 8
    avg_launch_ms = pass_ms / max(pass_launches, 1)
    alg_bytes_launch = pass_vp / max(pass_launches, 1) * bytes_per_vp
    achieved = alg_bytes_launch / (avg_launch_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic = committed_traffic(w["name"])
    init_launches = n_calls * args.steps  # v*mask initialisation, one per transform
    cpu_val, cpu_kind, cpu_cores, cpu_sample = time_cpu_sample(w, "port", budget_s=args.cpu_budget)
    line = {
        "metric": metric_name(w), "value": round(value, 4), "unit": "Gvoxel-passes/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": w["desc"], "parallelism": f"replicas x{world}",
                   "l2": f"flushed between steps ({FLUSH_BYTES >> 20} MiB write outside the timed events)",
                   "wall_s_timed_region": round(wall, 4)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": "fg_pass_kernel", "avg_launch_ms": round(avg_launch_ms, 5),
                     "alg_bytes_per_launch": int(alg_bytes_launch), "peak_source": peak_kind,
                     "pass_time_share": round(pass_ms / (ms * args.steps), 4)},
        "cpu_baseline": {"value": round(cpu_val, 4), "unit": "Gvoxel-passes/s", "cores": cpu_cores,
                         "kind": cpu_kind, "sample": cpu_sample},
        "e2e": {"value": round(world * vp_step / e2e_s / 1e9, 4), "unit": "Gvoxel-passes/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "clocks": clk,
        "gpu_launches": int((pass_launches + init_launches) / args.steps),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "vol256", "c3"])
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU baseline sampling")
    ap.add_argument("--kernels-only", action="store_true",
                    help="run warm-up and timed GPU steps only (no end-to-end or CPU legs): for profiler captures")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.workload == "c3":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the uneven batch has no reference CPU arm here"}))
            return
        run_batch_arm(args, rank, world)
        return
    w = workload(args.workload)
    if args.impl == "reference":
        run_reference_arm(args, w, rank)
        return
    run_gpu_arm(args, w, rank, world)


if __name__ == "__main__":
    main()
