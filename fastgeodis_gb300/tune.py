"""Autotuner: picks each pass's tiling by measurement instead of by the model.

The engine plans every pass (tile extents T1 x T2 of the cross-section, halo
hand-off every S steps) from a cost model of one step.  `autotune` replaces the
model's choice by timing: for each distinct pass cross-section of a transform
it tries candidate plans, runs the workload on seeded synthetic data of that
shape with each candidate, and pins the fastest plan with
``fg_plan_override``.  Cross-sections are tuned one after another with the
others held fixed, so differences in the total are the tuned pass's own.

A workload of several transforms of one shape that run at the same time
(one per stream: several lambdas of one image, or concurrent requests) is
tuned as such: the timed unit is all of them, launched on their own streams,
and the candidates include plans with fewer, larger tiles (a fraction of the
SMs per transform), which waste less work on halos while the transforms
share the GPU.  Volume passes also try cluster plans: one thread-block
cluster of up to 16 CTAs owns the whole cross-section (no halo, no hand-off
through global memory), so concurrent transforms each take a few SMs.

Every plan computes the same bits; only the time changes.  Pinned plans hold
for the process (all calls with that cross-section) until `clear`.
"""
from __future__ import annotations

import json
import math
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib

# Limits of one CTA, as the engine checks them (fg_common.cuh): one thread per
# run of 4 cells, 512 threads (1024 for volume sweeps with one image channel
# and one map), regions of at most 4 cells per thread.
THREADS = 512
THREADS_LEAN = 1024

Key = Tuple[int, int, int]        # (cross, N1, N2)
Choice = Tuple[int, int, int]     # (S, T1, T2)
# A pinned plan: (S, T1, T2, flags); flags FG_PLAN_LEAN asks for the
# 64-register kernel, FG_PLAN_CLUSTER for a cluster plan (fg_plan_override).


def _ceil(a: int, b: int) -> int:
    return -(-a // b)


def candidates(cross: int, N1: int, N2: int, sms: int, steps=(4, 8), max_per_step: int = 24,
               lean: bool = False, tile_fracs: Sequence[float] = (1.0,)) -> List[Choice]:
    """Valid plans for a cross-section: for each tile count along N2 the
    smallest tile height T1 that keeps the tiles within `frac * sms` (all
    co-resident), for every fraction in `tile_fracs`."""
    max_threads = THREADS_LEAN if (lean and cross == 2) else THREADS
    max_region = 4 * max_threads
    out: List[Choice] = []
    for S in steps:
        for frac in tile_fracs:
            cap = max(1, int(sms * frac))
            seen_T2 = set()
            n = 0
            for t2 in range(1, N2 + 1):
                T2 = _ceil(N2, t2)
                if t2 > 1:
                    T2 = (T2 + 3) // 4 * 4  # runs of 4 cells must not straddle tiles
                if T2 in seen_T2 or _ceil(N2, T2) > cap:
                    continue
                seen_T2.add(T2)
                tt2 = _ceil(N2, T2)
                K2 = S if tt2 > 1 else 0
                if tt2 > 1 and T2 < K2:
                    break
                if cross == 1:
                    T1, K1 = 1, 0
                else:
                    T1 = next((c for c in range(1, N1 + 1) if _ceil(N1, c) * tt2 <= cap), None)
                    if T1 is None:
                        continue
                    K1 = S if _ceil(N1, T1) > 1 else 0
                    if K1 and T1 < K1:
                        T1 = min(K1, N1)
                        K1 = S if _ceil(N1, T1) > 1 else 0
                R1 = T1 + 2 * K1 if cross == 2 else 1
                R2 = T2 + 2 * K2
                if R1 * R2 > max_region or R1 * _ceil(R2, 4) > max_threads:
                    continue
                if (S, T1, T2) not in out:
                    out.append((S, T1, T2))
                    n += 1
                if n >= max_per_step:
                    break
    return out


def cluster_candidates(cross: int, N1: int, N2: int, lean_capable: bool = True, one_channel: bool = True,
                       sizes: Sequence[int] = (16, 12, 8, 6, 4)) -> List[Tuple[int, int, int, int]]:
    """Cluster plans of a volume cross-section: (S, T1, N2, flags) for about
    `sizes` strips of T1 whole rows, one CTA each (2 to 16 per cluster).  On
    the pass kernel a thread owns one run of 4 cells (at most 1024 threads
    with the 64-register kernel, 512 without); on the cluster sweep kernel
    (passes that read at most one image channel) 2 vertically adjacent runs,
    T1 even, at most 512 threads."""
    if cross != 2:
        return []
    out = []
    rpr = _ceil(N2, 4)
    for rpt, flag in ((1, 0), (2, _lib.FG_PLAN_RUNS2)):
        if rpt > 1 and not one_channel:
            continue
        max_threads = (THREADS_LEAN if lean_capable else THREADS) if rpt == 1 else THREADS
        for G in sizes:
            T1 = _ceil(_ceil(N1, G), rpt) * rpt
            g = _ceil(N1, T1)
            threads = (T1 // rpt) * rpr
            if g < 2 or g > 16 or threads > max_threads:
                continue
            lean = _lib.FG_PLAN_LEAN if rpt == 1 and threads > THREADS else 0
            c = (8, T1, N2, _lib.FG_PLAN_CLUSTER | lean | flag)
            if c not in out:
                out.append(c)
    return out


def pass_keys(shape: Sequence[int]) -> List[Key]:
    """Distinct (cross, N1, N2) cross-sections of a transform's passes."""
    if len(shape) == 2:
        H, W = (int(s) for s in shape)
        keys = [(1, 1, W), (1, 1, H)]       # along H over [H][W], along W over [W][H]
    elif len(shape) == 3:
        D, H, W = (int(s) for s in shape)
        keys = [(2, H, W), (2, D, W), (2, D, H)]  # along D, H, W
    else:
        raise ValueError("shape must be (H, W) or (D, H, W)")
    return list(dict.fromkeys(keys))


def pin(choices: Dict[Key, Tuple[int, int, int, int]]) -> None:
    """Pin plans {(cross, N1, N2): (S, T1, T2, lean)}."""
    L = _lib.load()
    for (cross, N1, N2), (S, T1, T2, lean) in choices.items():
        _lib.check(L.fg_plan_override(cross, N1, N2, S, T1, T2, lean))


def clear(shape: Sequence[int]) -> None:
    """Unpin the plans of a shape's cross-sections (the cost model decides again)."""
    L = _lib.load()
    for cross, N1, N2 in pass_keys(shape):
        _lib.check(L.fg_plan_override(cross, N1, N2, 0, 0, 0, 0))


def autotune(shape: Sequence[int], channels: int = 1, lamb: float = 0.5, spacing=(1.0, 1.0, 1.0),
             iterations: int = 1, repeats: int = 3, device=None, max_per_step: int = 24,
             lambs: Optional[Sequence[float]] = None, verbose: bool = False) -> Dict[Key, Tuple[int, int, int, int, float]]:
    """Measure candidate plans for a 2D (H, W) or 3D (D, H, W) transform of
    `channels` image channels and pin the fastest for each cross-section.

    `lambs`: the workload's transforms that run at the same time, one per
    stream (default: one transform with `lamb`).  With several, the 64-register
    kernel is tried too (two CTAs of different transforms per SM).  Returns
    {(cross, N1, N2): (S, T1, T2, lean, best ms of the workload)}; the model's
    own plan competes as the unpinned entry (S = 0)."""
    import fastgeodis_gb300 as fg

    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    shape = tuple(int(s) for s in shape)
    lambs = [float(lamb)] if lambs is None else [float(x) for x in lambs]
    L = _lib.load()
    g = torch.Generator(device="cpu").manual_seed(0)
    result = {}
    with torch.cuda.device(dev):
        img = torch.rand((1, channels) + shape, generator=g).to(dev)
        msk = torch.ones((1, 1) + shape, device=dev)
        msk.view(-1)[msk.numel() // 2] = 0.0
        main = torch.cuda.current_stream(dev)
        streams = [torch.cuda.Stream(dev) for _ in lambs]

        def run():
            for s in streams:
                s.wait_stream(main)
            for lm, s in zip(lambs, streams):
                with torch.cuda.stream(s):
                    if len(shape) == 2:
                        fg.generalised_geodesic2d(img, msk, 1e10, lm, iterations)
                    else:
                        fg.generalised_geodesic3d(img, msk, list(spacing), 1e10, lm, iterations)
            for s in streams:
                main.wait_stream(s)

        def measure() -> float:
            run()  # first launch of a plan sets up its kernel attributes
            torch.cuda.synchronize(dev)
            best = math.inf
            for _ in range(repeats):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(main)
                run()
                e1.record(main)
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            return best

        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fracs = (1.0,) if len(lambs) == 1 else (1.0, 0.75, 0.5, 0.34)
        lean = channels <= 1
        for key in pass_keys(shape):
            cross, N1, N2 = key
            _lib.check(L.fg_plan_override(cross, N1, N2, 0, 0, 0, 0))
            best_c, best_t = (0, 0, 0, 0), measure()
            if verbose:
                print(f"[tune] {key} model plan: {best_t:.3f} ms")
            trials = []
            for c in candidates(cross, N1, N2, sms, max_per_step=max_per_step, lean=lean, tile_fracs=fracs):
                trials.append(c + (0,))
                small = (c[1] + 2 * c[0]) * _ceil(c[2] + 2 * c[0], 4) <= THREADS
                if lean and cross == 2 and len(lambs) > 1 and small:
                    trials.append(c + (1,))  # 64-register kernel: two CTAs per SM
            # cluster plans (one thread-block cluster per transform): they pay
            # off when several transforms share the GPU
            trials += cluster_candidates(cross, N1, N2, lean_capable=lean, one_channel=channels <= 1)
            for c in trials:
                _lib.check(L.fg_plan_override(cross, N1, N2, *c))
                try:
                    t = measure()
                except _lib.EngineError:
                    # a cluster plan the device cannot co-schedule: the launch is
                    # refused before anything runs
                    if not c[3] & _lib.FG_PLAN_CLUSTER:
                        raise
                    torch.cuda.synchronize(dev)
                    continue
                if verbose:
                    print(f"[tune] {key} S={c[0]} T={c[1]}x{c[2]} lean={c[3]}: {t:.3f} ms")
                if t < best_t:
                    best_c, best_t = c, t
            _lib.check(L.fg_plan_override(cross, N1, N2, *best_c))
            result[key] = best_c + (best_t,)
        fg.check_status(dev)
    return result


def save(result: Dict[Key, Tuple], path: str) -> None:
    """Write tuned plans as JSON ({"cross,N1,N2": [S, T1, T2, lean, ms]})."""
    with open(path, "w") as f:
        json.dump({",".join(map(str, k)): list(v) for k, v in result.items()}, f, indent=1)


def load(path: str, apply: bool = True) -> Dict[Key, Tuple]:
    """Read plans written by `save` and (by default) pin them."""
    with open(path) as f:
        raw = json.load(f)
    result = {tuple(int(x) for x in k.split(",")): tuple(v) for k, v in raw.items()}
    if apply:
        pin({k: tuple(int(x) for x in v[:4]) for k, v in result.items() if int(v[0]) > 0})
    return result
