"""Accuracy harness: the raster scans against fast marching (test
infrastructure; only tests/ and the accuracy report use it).

The reference reports its accuracy by comparing its raster-scan distances
with fast-marching arrival times on the same image (FastGeodis README,
"Accuracy", joint histograms).  Its own fast-marching entry points
(FastGeodis/geodis_fastmarch.cpp:163-236, 323-391) cannot run under the
installed torch: their gradient helper builds a CPU tensor with device index 1
(geodis_fastmarch.cpp:63, :254), which torch rejects.  So this module
restates that entry's speed field and hands it to the same vendored solver
(dependency/fmm: HighAccuracyVaryingSpeedEikonalSolver + SignedArrivalTime,
seeds where the soft mask is 0 at time 0), compiled by
oracle/build_oracle.py:build_fastmarch from oracle/fg_fastmarch.cpp.

Speed field (geodis_fastmarch.cpp:58-104, 189-209; 3D :251-321, 357-379):
per channel the forward differences along each in-plane axis with a zero
beyond the last cell, |dx| and |dy| averaged (x 0.5 in 2D), summed over
channels; the solver's speed is 1 / (l_grad * grad + l_eucl + sqrt(eps_f32)).
In 3D the reference's z-difference kernel is never filled (its taps are
written through the y kernel's accessor), so its gradient is
(|dx| + |dy|) / 3 with no z term; restated as it runs.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

_LIB = None
FEPS = np.float32(np.sqrt(np.finfo(np.float32).eps))  # std::sqrt(std::numeric_limits<float>::epsilon())


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build_fastmarch()
        if path is None:
            raise RuntimeError("the fast-marching solver header (the reference's dependency/fmm) is not available")
        L = ctypes.CDLL(path)
        p = ctypes.c_void_p
        L.fgo_fastmarch.argtypes = [ctypes.c_int, p, p, p, p, p]
        L.fgo_fastmarch.restype = ctypes.c_int
        L.fgo_fastmarch_error.restype = ctypes.c_char_p
        _LIB = L
    return _LIB


def available() -> bool:
    return build_oracle.fmm_include_dir() is not None


def _fwd_diff_abs(img: np.ndarray, axis: int) -> np.ndarray:
    """|I[i+1] - I[i]| along `axis`, with I = 0 beyond the last cell."""
    nxt = np.zeros_like(img)
    sl_dst = [slice(None)] * img.ndim
    sl_src = [slice(None)] * img.ndim
    sl_dst[axis] = slice(0, -1)
    sl_src[axis] = slice(1, None)
    nxt[tuple(sl_dst)] = img[tuple(sl_src)]
    return np.abs(nxt - img)


def speed_field(image: np.ndarray, l_grad: float, l_eucl: float) -> np.ndarray:
    """The solver's speed per cell for an image [C, H, W] or [C, D, H, W]."""
    img = np.asarray(image, np.float32)
    if img.ndim == 3:  # [C, H, W]: x along W, y along H
        g = np.float32(0.5) * (_fwd_diff_abs(img, 2) + _fwd_diff_abs(img, 1))
    elif img.ndim == 4:  # [C, D, H, W]: x along W, y along H, no z term
        g = np.float32(1.0 / 3.0) * (_fwd_diff_abs(img, 3) + _fwd_diff_abs(img, 2))
    else:
        raise ValueError("image must be [C, H, W] or [C, D, H, W]")
    grad = g.sum(axis=0, dtype=np.float32)
    c = np.float32(l_grad) * grad + np.float32(l_eucl) + FEPS
    return (np.float32(1.0) / c).astype(np.float32)


def fastmarch(image: np.ndarray, mask: np.ndarray, lamb: float, spacing=None) -> np.ndarray:
    """Arrival times from the cells where mask == 0 (image [C, ...], mask
    [1, ...] or [...]); l_grad = lamb, l_eucl = 1 - lamb as the reference's
    Python layer passes them (FastGeodis/__init__.py:441-443, :468-470)."""
    m = np.asarray(mask, np.float32)
    m = m[0] if m.ndim == np.asarray(image).ndim else m
    sp = speed_field(image, float(np.float32(lamb)), float(np.float32(1.0 - lamb)))
    nd = sp.ndim
    spacing = [1.0] * nd if spacing is None else [float(s) for s in spacing]
    seed = np.ascontiguousarray(m == 0, dtype=np.uint8)
    if not seed.any():
        raise ValueError("fast marching needs at least one seed (a mask value of 0)")
    out = np.empty(sp.shape, np.float32)
    dims = (ctypes.c_int * nd)(*sp.shape)
    spc = np.asarray(spacing, np.float32)
    sp = np.ascontiguousarray(sp)
    rc = lib().fgo_fastmarch(nd, dims, sp.ctypes.data, seed.ctypes.data, spc.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise RuntimeError("fast marching failed: " + lib().fgo_fastmarch_error().decode())
    return out


def compare(dist: np.ndarray, arrival: np.ndarray, mask: np.ndarray) -> dict:
    """Agreement of a raster-scan distance map with fast-marching arrival
    times over the non-seed cells: absolute and relative differences and the
    Pearson correlation (the reference's joint histograms, in numbers)."""
    d = np.asarray(dist, np.float64).reshape(-1)
    t = np.asarray(arrival, np.float64).reshape(-1)
    m = np.asarray(mask).reshape(-1) != 0
    sel = m & np.isfinite(d) & np.isfinite(t) & (t > 0)
    d, t = d[sel], t[sel]
    err = d - t
    rel = np.abs(err) / t
    return {"cells": int(sel.sum()), "mean_arrival": float(t.mean()), "mean_abs_diff": float(np.abs(err).mean()),
            "max_abs_diff": float(np.abs(err).max()), "mean_signed_diff": float(err.mean()),
            "mean_rel_diff": float(rel.mean()), "p95_rel_diff": float(np.percentile(rel, 95)),
            "pearson": float(np.corrcoef(d, t)[0, 1])}
