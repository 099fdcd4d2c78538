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

Transforms of one shape that differ in arithmetic mode (l_grad = 0, l_eucl =
0 with l_grad = 1, or the general expression -- e.g. the lambdas 0, 1 and 0.5
of one image) cost different amounts per step, and the slowest sets the
time of the group.  After one plan per cross-section is tuned for all of
them, each mode may take its own plan (``FG_PLAN_MODE``), the costliest mode
first, where that makes the group measurably faster.

Every plan computes the same bits; only the time changes.  Pinned plans hold
for the process (all calls with that cross-section) until `clear`.
"""
from __future__ import annotations

import json
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib

# Limits of one CTA, as the engine checks them (fg_common.cuh): one thread per
# run of 4 cells, 512 threads (1024 for volume sweeps with one image channel
# and one map), regions of at most 4 cells per thread.
THREADS = 512
THREADS_LEAN = 1024

Key = Tuple[int, ...]             # (cross, N1, N2), or (cross, N1, N2, mode) for a per-mode plan
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


def row_tile_candidates(cross: int, N2: int, sms: int, channels: int = 1,
                        periods: Sequence[int] = (16, 32), widths: Sequence[int] = (32, 64, 128)
                        ) -> List[Tuple[int, int, int, int]]:
    """Row-tile plans of a 2D pass: (S, 1, T2, FG_PLAN_ROWS) for tiles of
    `widths` cells narrower than the row, halos of S cells, at most 512
    threads (T2 + 2 S) and every tile resident; images of 1 to 4 channels.
    Where the tiles can form one thread-block cluster (2 to 16 tiles, S <=
    T2) the clustered form (| FG_PLAN_CLUSTER) follows each."""
    if cross != 1 or channels > 4:
        return []
    out = []
    for S in periods:
        for T2 in widths:
            if T2 < N2 and T2 + 2 * S <= 512 and _ceil(N2, T2) <= sms:
                out.append((S, 1, T2, _lib.FG_PLAN_ROWS))
                if _ceil(N2, T2) <= 16 and S <= T2:
                    out.append((S, 1, T2, _lib.FG_PLAN_ROWS | _lib.FG_PLAN_CLUSTER))
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


MODE_GENERAL, MODE_EUCLID, MODE_GEO = 0, 1, 2


def mode_of(lamb: float) -> int:
    """The engine's arithmetic mode of a transform with this lamb: the
    weights as the drop-in narrows them (l_grad = lamb, l_eucl = 1 - lamb)."""
    import numpy as np

    lg, le = np.float32(lamb), np.float32(1.0 - float(lamb))
    if lg == 0.0:
        return MODE_EUCLID
    if le == 0.0 and lg == 1.0:
        return MODE_GEO
    return MODE_GENERAL


def _mode_flag(key: Key) -> int:
    return _lib.FG_PLAN_MODE(key[3]) if len(key) == 4 else 0


def pin(choices: Dict[Key, Tuple[int, int, int, int]]) -> None:
    """Pin plans {(cross, N1, N2[, mode]): (S, T1, T2, flags)}."""
    L = _lib.load()
    for key, (S, T1, T2, lean) in choices.items():
        _lib.check(L.fg_plan_override(*key[:3], S, T1, T2, lean | _mode_flag(key)))


def clear(shape: Sequence[int]) -> None:
    """Unpin the plans of a shape's cross-sections, for every mode (the cost
    model decides again)."""
    L = _lib.load()
    for cross, N1, N2 in pass_keys(shape):
        _lib.check(L.fg_plan_override(cross, N1, N2, 0, 0, 0, 0))
        for m in (MODE_GENERAL, MODE_EUCLID, MODE_GEO):
            _lib.check(L.fg_plan_override(cross, N1, N2, 0, 0, 0, _lib.FG_PLAN_MODE(m)))


def autotune(shape: Sequence[int], channels: int = 1, lamb: float = 0.5, spacing=(1.0, 1.0, 1.0),
             iterations: int = 1, repeats: int = 3, device=None, max_per_step: int = 24,
             lambs: Optional[Sequence[float]] = None, verbose: bool = False,
             per_mode: bool = False, final_top: int = 4, final_iterations: int = 4,
             final_repeats: int = 5) -> Dict[Key, Tuple[int, int, int, int, float]]:
    """Measure candidate plans for a 2D (H, W) or 3D (D, H, W) transform of
    `channels` image channels and pin the fastest for each cross-section.

    `lambs`: the workload's transforms that run at the same time, one per
    stream (default: one transform with `lamb`).  With several, the 64-register
    kernel is tried too (two CTAs of different transforms per SM), and when
    they differ in arithmetic mode (`per_mode`) each mode then tries its own
    plan in place of the shared one (the costliest mode -- general, then
    l_eucl = 0, then l_grad = 0 -- first), kept only when the workload runs at
    least 2% faster.  Returns {(cross, N1, N2[, mode]): (S, T1, T2, flags, best
    ms of the workload)}; S = 0: the model's plan (shared keys), the shared
    plan (per-mode keys).

    Each cross-section is searched with `iterations` per transform (short
    runs, best of `repeats`); the `final_top` fastest plans are then timed
    again on `final_iterations` iterations, averaged over `final_repeats`
    runs, and the fastest of those is pinned: short runs rank plans well but
    their noise, and the start and end of transforms that overlap, had picked
    plans up to 10% slower on the full workload."""
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

        def run(iters):
            for s in streams:
                s.wait_stream(main)
            for lm, s in zip(lambs, streams):
                with torch.cuda.stream(s):
                    if len(shape) == 2:
                        fg.generalised_geodesic2d(img, msk, 1e10, lm, iters)
                    else:
                        fg.generalised_geodesic3d(img, msk, list(spacing), 1e10, lm, iters)
            for s in streams:
                main.wait_stream(s)

        def measure(iters=iterations, reps=repeats, mean=False) -> float:
            run(iters)  # first launch of a plan sets up its kernel attributes
            torch.cuda.synchronize(dev)
            ts = []
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(main)
                run(iters)
                e1.record(main)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            return sum(ts) / len(ts) if mean else min(ts)

        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fracs = (1.0,) if len(lambs) == 1 else (1.0, 0.75, 0.5, 0.34)
        lean = channels <= 1
        present = {mode_of(x) for x in lambs}
        modes = [m for m in (MODE_GENERAL, MODE_GEO, MODE_EUCLID) if m in present]
        clear(shape)
        # one plan per cross-section first; then, for transforms of several
        # modes, each mode may replace it with its own plan where that is
        # measurably faster (by 2%: a refinement never loses to noise)
        tuned = pass_keys(shape)
        if per_mode and len(modes) > 1:
            tuned = tuned + [k + (m,) for k in pass_keys(shape) for m in modes]
        leaders = {}
        for key in tuned:
            cross, N1, N2 = key[:3]
            mflag = _mode_flag(key)
            margin = 0.98 if mflag else 1.0
            # S = 0: the model's plan (a shared plan), or the shared plan (a per-mode key)
            best_c, best_t = (0, 0, 0, 0), measure()
            scores = [(best_t, best_c)]
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
            # 2D rows: one thread per cell on row tiles
            trials += row_tile_candidates(cross, N2, sms, channels)
            for c in trials:
                _lib.check(L.fg_plan_override(cross, N1, N2, *c[:3], c[3] | mflag))
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
                scores.append((t, c))
                if t < best_t * (margin if best_c[0] == 0 else 1.0):
                    best_c, best_t = c, t
            _lib.check(L.fg_plan_override(cross, N1, N2, *best_c[:3], best_c[3] | mflag))
            result[key] = best_c + (best_t,)
            leaders[key] = [best_c] + [c for _, c in sorted(scores, key=lambda x: x[0]) if c != best_c]
        if final_top > 1:
            # the leading plans of each cross-section again, on the full
            # workload, with every other cross-section on its chosen plan
            for key in tuned:
                cross, N1, N2 = key[:3]
                mflag = _mode_flag(key)
                margin = 0.98 if mflag else 1.0
                finals = []
                for c in leaders[key][:final_top]:
                    _lib.check(L.fg_plan_override(cross, N1, N2, *c[:3], c[3] | mflag))
                    finals.append((measure(final_iterations, final_repeats, mean=True), c))
                    if verbose:
                        print(f"[tune] {key} final S={c[0]} T={c[1]}x{c[2]} flags={c[3]}: {finals[-1][0]:.3f} ms")
                base = [t for t, c in finals if c == (0, 0, 0, 0)]
                best_t, best_c = min(finals, key=lambda x: x[0])
                if mflag and base and best_c != (0, 0, 0, 0) and best_t > base[0] * margin:
                    best_t, best_c = base[0], (0, 0, 0, 0)  # a per-mode plan must beat the shared one clearly
                _lib.check(L.fg_plan_override(cross, N1, N2, *best_c[:3], best_c[3] | mflag))
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
