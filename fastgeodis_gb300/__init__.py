"""fastgeodis_gb300 -- generalised geodesic distance transforms on one GB300.

Drop-in for the raster-scan functions of FastGeodis (masadcv/FastGeodis
1.0.5, ``FastGeodis/__init__.py``): same names, argument order, defaults,
argument meaning and exception types.  Use it as::

    import fastgeodis_gb300 as FastGeodis
    d = FastGeodis.generalised_geodesic2d(image, softmask, v, lamb, iter)

Differences a caller may notice:

* the computation always runs on the GPU.  CUDA tensors are processed on
  their device and stream; CPU tensors are copied to the current CUDA device
  and the result is copied back (a CPU tensor is returned), so code written
  for the reference's CPU path keeps working and gets the GPU.
* results are bit-identical to the reference's CPU path (float32, same
  operation order); the reference's CUDA path can differ from that at its
  thread-block seams, this one does not.
"""
from __future__ import annotations

import os
import threading
from typing import List

import torch

from . import _lib

__version__ = "1.0.5"  # API level of the FastGeodis release this mirrors

__all__ = [
    "generalised_geodesic2d_differentiable",
    "GeodesicBatch2d",
    "generalised_geodesic2d_batch",
    "signed_generalised_geodesic2d_batch",
    "GeodesicBatch3d",
    "PersistentBatch3d",
    "generalised_geodesic3d_batch",
    "signed_generalised_geodesic3d_batch",
    "generalised_geodesic2d",
    "generalised_geodesic3d",
    "signed_generalised_geodesic2d",
    "signed_generalised_geodesic3d",
    "GSF2d",
    "GSF3d",
    "generalised_geodesic2d_toivanen",
    "generalised_geodesic3d_toivanen",
    "signed_generalised_geodesic2d_toivanen",
    "signed_generalised_geodesic3d_toivanen",
    "GSF2d_toivanen",
    "GSF3d_toivanen",
    "check_status",
]

_ws_lock = threading.Lock()
_workspaces = {}  # (device index, stream handle) -> uint8 tensor
_CHECK_EVERY_CALL = os.environ.get("FASTGEODIS_GB300_CHECK", "0") == "1"


# ---------------------------------------------------------------------------
# input validation, mirroring FastGeodis/common.h:53-120 and
# FastGeodis/fastgeodis.cpp:44-146
# ---------------------------------------------------------------------------

def _check_data_dim(t: torch.Tensor, dims: int) -> None:
    # common.h:97-106 (the reference's message says "2D" for both ranks)
    if t.dim() != dims:
        raise ValueError(f"function only supports 2D spatial inputs, received {t.dim() - 2}")


def _check_single_batch(t: torch.Tensor) -> None:
    # common.h:89-95
    if t.size(0) != 1:
        raise ValueError("FastGeodis currently only supports single batch input.")


def _check_input_dimensions(image: torch.Tensor, mask: torch.Tensor, dims: int) -> None:
    # common.h:108-120
    _check_data_dim(image, dims)
    _check_data_dim(mask, dims)
    _check_single_batch(image)
    _check_single_batch(mask)
    if image.dim() != mask.dim():
        raise ValueError(
            f"dimensions of input tensors do not match {image.dim() - 2} vs {mask.dim() - 2}")
    for i in range(dims - 2):
        if image.size(2 + i) != mask.size(2 + i):
            raise ValueError("shapes of input tensors do not match")


def _check_spacing(spacing) -> List[float]:
    # fastgeodis.cpp:116-120
    sp = [float(s) for s in spacing]
    if len(sp) != 3:
        raise ValueError(f"function only supports 3D spacing inputs, received {len(sp)}")
    return sp


def _check_devices(image: torch.Tensor, mask: torch.Tensor) -> None:
    # fastgeodis.cpp:69-88 and common.h:73-87; additionally the CUDA device
    # index must match (the reference launches on the image's device only)
    if image.is_cuda:
        if not mask.is_cuda:
            raise ValueError("input is not on CUDA device, try using data.to('cuda') on input")
        if mask.device != image.device:
            raise ValueError(
                f"inputs are on different CUDA devices ({image.device} and {mask.device})")
    else:
        if mask.is_cuda:
            raise ValueError("input is not on CPU device, try using data.to('cpu') on input")
    for t in (image, mask):
        if t.dtype != torch.float32:
            # the reference reads data_ptr<float>(), a c10 error (RuntimeError)
            raise RuntimeError(f"expected scalar type Float but found {t.dtype}")


# ---------------------------------------------------------------------------
# execution
# ---------------------------------------------------------------------------

def _workspace(device: torch.device, nbytes: int, stream) -> torch.Tensor:
    key = (device.index, stream.cuda_stream)
    with _ws_lock:
        ws = _workspaces.get(key)
        if ws is None or ws.numel() < nbytes:
            ws = torch.zeros(max(nbytes, 1 << 16), dtype=torch.uint8, device=device)
            _workspaces[key] = ws
        return ws


def _run(kind: str, image, mask, v, lamb, iterations, spacing=None, theta=None, toivanen=False):
    is3d = kind.endswith("3d")
    dims = 5 if is3d else 4
    _check_input_dimensions(image, mask, dims)
    if is3d:
        spacing = _check_spacing(spacing)
    _check_devices(image, mask)
    L = _lib.load()
    host = not image.is_cuda
    if host:
        if not torch.cuda.is_available():
            raise RuntimeError("fastgeodis_gb300 needs a CUDA device; torch.cuda.is_available() is False")
        device = torch.device("cuda", torch.cuda.current_device())
    else:
        device = image.device
    with torch.cuda.device(device):
        stream = torch.cuda.current_stream(device)
        img = image.to(device, non_blocking=True).contiguous()
        msk = mask.to(device, non_blocking=True).contiguous()
        C, Cm = int(img.size(1)), int(msk.size(1))
        sizes = [int(s) for s in img.shape[2:]]
        D, H, W = (sizes if is3d else [1] + sizes)
        out = torch.empty(msk.shape, dtype=torch.float32, device=device)
        op = {"plain": _lib.FG_OP_PLAIN, "signed": _lib.FG_OP_SIGNED, "gsf": _lib.FG_OP_GSF}[kind[:-2]]
        nbytes = int(L.fg_workspace_bytes(op, C, D, H, W))
        ws = _workspace(device, nbytes, stream)
        sh = ctypes_stream(stream)
        vf = float(v)
        it = int(iterations)
        if kind.startswith("gsf"):
            lam = float(lamb)  # the reference narrows lambda to float and forms 1 - lambda in C++
        else:
            lg = float(lamb)
            le = 1.0 - float(lamb)  # FastGeodis/__init__.py:63-65: 1 - lamb in Python floats
        ptr = lambda t: t.data_ptr()  # noqa: E731
        if is3d:
            sp = (_ctypes_float3(spacing))
        # the C entry of this kind; Toivanen's scan has the same arguments under a suffixed name
        fn = lambda name: getattr(L, name + ("_toivanen" if toivanen else ""))  # noqa: E731
        if kind == "plain2d":
            rc = fn("fg_generalised_geodesic2d")(ptr(img), C, H, W, ptr(msk), Cm, ptr(out), vf, lg, le, it,
                                             ptr(ws), ws.numel(), sh)
        elif kind == "signed2d":
            rc = fn("fg_signed_generalised_geodesic2d")(ptr(img), C, H, W, ptr(msk), Cm, ptr(out), vf, lg, le,
                                                    it, ptr(ws), ws.numel(), sh)
        elif kind == "plain3d":
            rc = fn("fg_generalised_geodesic3d")(ptr(img), C, D, H, W, ptr(msk), Cm, sp, ptr(out), vf, lg, le,
                                             it, ptr(ws), ws.numel(), sh)
        elif kind == "signed3d":
            rc = fn("fg_signed_generalised_geodesic3d")(ptr(img), C, D, H, W, ptr(msk), Cm, sp, ptr(out), vf,
                                                    lg, le, it, ptr(ws), ws.numel(), sh)
        elif kind == "gsf2d":
            rc = fn("fg_GSF2d")(ptr(img), C, H, W, ptr(msk), Cm, float(theta), vf, lam, it, ptr(out), ptr(ws),
                            ws.numel(), sh)
        elif kind == "gsf3d":
            rc = fn("fg_GSF3d")(ptr(img), C, D, H, W, ptr(msk), Cm, float(theta), sp, vf, lam, it, ptr(out),
                            ptr(ws), ws.numel(), sh)
        else:  # pragma: no cover
            raise AssertionError(kind)
        _lib.check(rc)
        if host:
            # result into page-locked host memory on the call's stream; the
            # status read below synchronises that stream, so it is complete
            # when the call returns
            res = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
            res.copy_(out, non_blocking=True)
        if host or _CHECK_EVERY_CALL:
            _lib.check(L.fg_workspace_status(ptr(ws), sh))
        if host:
            return res
        return out


def ctypes_stream(stream) -> int:
    return int(stream.cuda_stream)


def _ctypes_float3(vals):
    import ctypes

    return (ctypes.c_float * 3)(*vals)


def check_status(device=None) -> None:
    """Synchronise and raise if a kernel on `device` (all devices used so
    far if None) gave up a bounded wait.  Results of such a call are invalid."""
    L = _lib.load()
    with _ws_lock:
        items = list(_workspaces.items())
    for (dev, sh), ws in items:
        if device is not None and torch.device(device).index != dev:
            continue
        with torch.cuda.device(dev):
            _lib.check(L.fg_workspace_status(ws.data_ptr(), sh))


# ---------------------------------------------------------------------------
# public API (FastGeodis/__init__.py:37-162, 526-585)
# ---------------------------------------------------------------------------

def generalised_geodesic2d(image: torch.Tensor, softmask: torch.Tensor, v: float, lamb: float, iter: int = 2):
    r"""Generalised geodesic distance of a 2D image by raster scanning.

    Args:
        image: ``[1, C, H, W]`` float32 image (grayscale or multi-channel).
        softmask: ``[1, Cm, H, W]`` float32 soft mask in [0, 1], 0 at the seeds.
        v: weight of the unary term; the initial distance is ``v * softmask``.
        lamb: 0.0 gives the Euclidean distance, 1.0 the pure geodesic one.
        iter: number of passes of the iterative raster scan.

    Returns:
        ``[1, Cm, H, W]`` float32 distance map on the input's device.
    """
    return _run("plain2d", image, softmask, v, lamb, iter)


def generalised_geodesic3d(image: torch.Tensor, softmask: torch.Tensor, spacing: List, v: float, lamb: float,
                           iter: int = 4):
    r"""Generalised geodesic distance of a 3D volume by raster scanning.

    Args:
        image: ``[1, C, D, H, W]`` float32 volume.
        softmask: ``[1, Cm, D, H, W]`` float32 soft mask in [0, 1].
        spacing: voxel spacing along (D, H, W), three numbers.
        v, lamb, iter: as in :func:`generalised_geodesic2d`.
    """
    return _run("plain3d", image, softmask, v, lamb, iter, spacing=spacing)


def signed_generalised_geodesic2d(image: torch.Tensor, softmask: torch.Tensor, v: float, lamb: float,
                                  iter: int = 2):
    r"""Signed distance ``D(softmask) - D(1 - softmask)`` of a 2D image."""
    return _run("signed2d", image, softmask, v, lamb, iter)


def signed_generalised_geodesic3d(image: torch.Tensor, softmask: torch.Tensor, spacing: List, v: float,
                                  lamb: float, iter: int = 4):
    r"""Signed distance ``D(softmask) - D(1 - softmask)`` of a 3D volume."""
    return _run("signed3d", image, softmask, v, lamb, iter, spacing=spacing)


def GSF2d(image: torch.Tensor, softmask: torch.Tensor, theta: float, v: float, lamb: float, iter: int):
    r"""Geodesic symmetric filtering of a 2D soft mask (Criminisi et al., GeoS):
    ``-signed(1 - [Ds > theta]) + signed([Ds > -theta])`` with ``Ds = signed(softmask)``."""
    return _run("gsf2d", image, softmask, v, lamb, iter, theta=theta)


def GSF3d(image: torch.Tensor, softmask: torch.Tensor, theta: float, spacing: List, v: float, lamb: float,
          iter: int):
    r"""Geodesic symmetric filtering of a 3D soft mask."""
    return _run("gsf3d", image, softmask, v, lamb, iter, spacing=spacing, theta=theta)


# ---------------------------------------------------------------------------
# Toivanen's raster scan (FastGeodis/__init__.py:165-308, 587-656).  The
# reference runs it on the CPU only and rejects CUDA tensors; here CPU tensors
# give the reference's CPU bits (computed on the GPU by a wavefront of the same
# sequential scan) and CUDA tensors are accepted as well.
# ---------------------------------------------------------------------------

def generalised_geodesic2d_toivanen(image: torch.Tensor, softmask: torch.Tensor, v: float, lamb: float,
                                    iter: int = 2):
    r"""Generalised geodesic distance of a 2D image by Toivanen's raster scan
    (Toivanen, Pattern Recognition Letters 17.5, 1996): one forward and one
    backward pass over the whole image per iteration, each cell taking the
    minimum over its four causal neighbours.  Arguments as in
    :func:`generalised_geodesic2d`."""
    return _run("plain2d", image, softmask, v, lamb, iter, toivanen=True)


def generalised_geodesic3d_toivanen(image: torch.Tensor, softmask: torch.Tensor, spacing: List, v: float,
                                    lamb: float, iter: int = 4):
    r"""Generalised geodesic distance of a 3D volume by Toivanen's raster scan
    (13 neighbours per pass).  Arguments as in :func:`generalised_geodesic3d`."""
    return _run("plain3d", image, softmask, v, lamb, iter, spacing=spacing, toivanen=True)


def signed_generalised_geodesic2d_toivanen(image: torch.Tensor, softmask: torch.Tensor, v: float, lamb: float,
                                           iter: int = 2):
    r"""Signed distance ``D(softmask) - D(1 - softmask)`` by Toivanen's scan, 2D."""
    return _run("signed2d", image, softmask, v, lamb, iter, toivanen=True)


def signed_generalised_geodesic3d_toivanen(image: torch.Tensor, softmask: torch.Tensor, spacing: List, v: float,
                                           lamb: float, iter: int = 4):
    r"""Signed distance ``D(softmask) - D(1 - softmask)`` by Toivanen's scan, 3D."""
    return _run("signed3d", image, softmask, v, lamb, iter, spacing=spacing, toivanen=True)


def GSF2d_toivanen(image: torch.Tensor, softmask: torch.Tensor, theta: float, v: float, lamb: float, iter: int):
    r"""Geodesic symmetric filtering (as :func:`GSF2d`) by Toivanen's scan."""
    return _run("gsf2d", image, softmask, v, lamb, iter, theta=theta, toivanen=True)


def GSF3d_toivanen(image: torch.Tensor, softmask: torch.Tensor, theta: float, spacing: List, v: float, lamb: float,
                   iter: int):
    r"""Geodesic symmetric filtering (as :func:`GSF3d`) by Toivanen's scan."""
    return _run("gsf3d", image, softmask, v, lamb, iter, spacing=spacing, theta=theta, toivanen=True)


from .batch import GeodesicBatch2d, generalised_geodesic2d_batch, signed_generalised_geodesic2d_batch  # noqa: E402
from .batch3d import (GeodesicBatch3d, PersistentBatch3d, generalised_geodesic3d_batch,  # noqa: E402
                      signed_generalised_geodesic3d_batch)
from .autograd import generalised_geodesic2d_differentiable  # noqa: E402
