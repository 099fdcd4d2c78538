"""ctypes wrapper around the C oracle (``oracle/fg_oracle.c``).

TEST INFRASTRUCTURE ONLY: used by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` to check and time against.  The product
package never imports this module.

All functions take and return numpy arrays in the reference's layout:
image ``[C, (D,) H, W]``, mask ``[Cm, (D,) H, W]`` (the batch dimension of the
reference's tensors, which must be 1, is dropped).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build_port()
        L = ctypes.CDLL(path)
        f32p = ctypes.POINTER(ctypes.c_float)
        f64p = ctypes.POINTER(ctypes.c_double)
        i, f, d = ctypes.c_int, ctypes.c_float, ctypes.c_double
        L.fgo_geodesic2d.argtypes = [f32p, i, i, i, f32p, i, f32p, f, f, f, i, i]
        L.fgo_geodesic3d.argtypes = [f32p, i, i, i, i, f32p, i, f32p, f32p, f, f, f, i, i]
        L.fgo_signed2d.argtypes = L.fgo_geodesic2d.argtypes
        L.fgo_signed3d.argtypes = L.fgo_geodesic3d.argtypes
        L.fgo_gsf2d.argtypes = [f32p, i, i, i, f32p, i, f, f32p, f, f, i, i]
        L.fgo_gsf3d.argtypes = [f32p, i, i, i, i, f32p, i, f, f32p, f32p, f, f, i, i]
        L.fgo_geodesic2d_f64.argtypes = [f64p, i, i, i, f64p, i, f64p, d, d, d, i, i]
        L.fgo_geodesic3d_f64.argtypes = [f64p, i, i, i, i, f64p, i, f64p, f64p, d, d, d, i, i]
        L.fgo_toivanen2d.argtypes = [f32p, i, i, i, f32p, i, f32p, f, f, f, i]
        L.fgo_toivanen3d.argtypes = [f32p, i, i, i, i, f32p, i, f32p, f32p, f, f, f, i]
        L.fgo_signed_toivanen2d.argtypes = L.fgo_toivanen2d.argtypes
        L.fgo_signed_toivanen3d.argtypes = L.fgo_toivanen3d.argtypes
        L.fgo_gsf_toivanen2d.argtypes = [f32p, i, i, i, f32p, i, f, f32p, f, f, i]
        L.fgo_gsf_toivanen3d.argtypes = [f32p, i, i, i, i, f32p, i, f, f32p, f32p, f, f, i]
        L.fgo_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _p32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _p64(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def max_threads() -> int:
    return int(lib().fgo_max_threads())


def _threads(nthreads):
    return max_threads() if nthreads is None else int(nthreads)


def _l_eucl_from_python(lamb: float) -> float:
    # FastGeodis/__init__.py:63-65: 1 - lamb evaluated on Python floats, the
    # pybind layer then narrows both weights to float.
    return float(np.float32(1.0 - float(lamb)))


def geodesic2d(image, mask, v, lamb, iterations=2, nthreads=None):
    image, mask = _f32(image), _f32(mask)
    C, H, W = image.shape
    out = np.empty(mask.shape, np.float32)
    lib().fgo_geodesic2d(_p32(image), C, H, W, _p32(mask), mask.shape[0], _p32(out),
                         float(np.float32(v)), float(np.float32(lamb)),
                         _l_eucl_from_python(lamb), int(iterations), _threads(nthreads))
    return out


def geodesic3d(image, mask, spacing, v, lamb, iterations=4, nthreads=None):
    image, mask = _f32(image), _f32(mask)
    C, D, H, W = image.shape
    sp = np.asarray(spacing, np.float32)
    out = np.empty(mask.shape, np.float32)
    lib().fgo_geodesic3d(_p32(image), C, D, H, W, _p32(mask), mask.shape[0], _p32(sp),
                         _p32(out), float(np.float32(v)), float(np.float32(lamb)),
                         _l_eucl_from_python(lamb), int(iterations), _threads(nthreads))
    return out


def signed2d(image, mask, v, lamb, iterations=2, nthreads=None):
    image, mask = _f32(image), _f32(mask)
    C, H, W = image.shape
    out = np.empty(mask.shape, np.float32)
    lib().fgo_signed2d(_p32(image), C, H, W, _p32(mask), mask.shape[0], _p32(out),
                       float(np.float32(v)), float(np.float32(lamb)),
                       _l_eucl_from_python(lamb), int(iterations), _threads(nthreads))
    return out


def signed3d(image, mask, spacing, v, lamb, iterations=4, nthreads=None):
    image, mask = _f32(image), _f32(mask)
    C, D, H, W = image.shape
    sp = np.asarray(spacing, np.float32)
    out = np.empty(mask.shape, np.float32)
    lib().fgo_signed3d(_p32(image), C, D, H, W, _p32(mask), mask.shape[0], _p32(sp),
                       _p32(out), float(np.float32(v)), float(np.float32(lamb)),
                       _l_eucl_from_python(lamb), int(iterations), _threads(nthreads))
    return out


def gsf2d(image, mask, theta, v, lamb, iterations, nthreads=None):
    image, mask = _f32(image), _f32(mask)
    C, H, W = image.shape
    out = np.empty(mask.shape, np.float32)
    lib().fgo_gsf2d(_p32(image), C, H, W, _p32(mask), mask.shape[0], float(np.float32(theta)),
                    _p32(out), float(np.float32(v)), float(np.float32(lamb)),
                    int(iterations), _threads(nthreads))
    return out


def gsf3d(image, mask, theta, spacing, v, lamb, iterations, nthreads=None):
    image, mask = _f32(image), _f32(mask)
    C, D, H, W = image.shape
    sp = np.asarray(spacing, np.float32)
    out = np.empty(mask.shape, np.float32)
    lib().fgo_gsf3d(_p32(image), C, D, H, W, _p32(mask), mask.shape[0], float(np.float32(theta)),
                    _p32(sp), _p32(out), float(np.float32(v)), float(np.float32(lamb)),
                    int(iterations), _threads(nthreads))
    return out


# Toivanen's sequential raster scan (FastGeodis/geodis_toivanen.cpp), one thread.

def toivanen2d(image, mask, v, lamb, iterations=2, signed=False):
    image, mask = _f32(image), _f32(mask)
    C, H, W = image.shape
    out = np.empty(mask.shape, np.float32)
    fn = lib().fgo_signed_toivanen2d if signed else lib().fgo_toivanen2d
    fn(_p32(image), C, H, W, _p32(mask), mask.shape[0], _p32(out), float(np.float32(v)),
       float(np.float32(lamb)), _l_eucl_from_python(lamb), int(iterations))
    return out


def toivanen3d(image, mask, spacing, v, lamb, iterations=4, signed=False):
    image, mask = _f32(image), _f32(mask)
    C, D, H, W = image.shape
    sp = np.asarray(spacing, np.float32)
    out = np.empty(mask.shape, np.float32)
    fn = lib().fgo_signed_toivanen3d if signed else lib().fgo_toivanen3d
    fn(_p32(image), C, D, H, W, _p32(mask), mask.shape[0], _p32(sp), _p32(out), float(np.float32(v)),
       float(np.float32(lamb)), _l_eucl_from_python(lamb), int(iterations))
    return out


def gsf_toivanen2d(image, mask, theta, v, lamb, iterations):
    image, mask = _f32(image), _f32(mask)
    C, H, W = image.shape
    out = np.empty(mask.shape, np.float32)
    lib().fgo_gsf_toivanen2d(_p32(image), C, H, W, _p32(mask), mask.shape[0], float(np.float32(theta)),
                             _p32(out), float(np.float32(v)), float(np.float32(lamb)), int(iterations))
    return out


def gsf_toivanen3d(image, mask, theta, spacing, v, lamb, iterations):
    image, mask = _f32(image), _f32(mask)
    C, D, H, W = image.shape
    sp = np.asarray(spacing, np.float32)
    out = np.empty(mask.shape, np.float32)
    lib().fgo_gsf_toivanen3d(_p32(image), C, D, H, W, _p32(mask), mask.shape[0], float(np.float32(theta)),
                             _p32(sp), _p32(out), float(np.float32(v)), float(np.float32(lamb)),
                             int(iterations))
    return out


def geodesic2d_f64(image, mask, v, lamb, iterations=2, nthreads=None):
    image = np.ascontiguousarray(image, np.float64)
    mask = np.ascontiguousarray(mask, np.float64)
    C, H, W = image.shape
    out = np.empty(mask.shape, np.float64)
    lib().fgo_geodesic2d_f64(_p64(image), C, H, W, _p64(mask), mask.shape[0], _p64(out),
                             float(v), float(lamb), 1.0 - float(lamb), int(iterations),
                             _threads(nthreads))
    return out


def geodesic3d_f64(image, mask, spacing, v, lamb, iterations=4, nthreads=None):
    image = np.ascontiguousarray(image, np.float64)
    mask = np.ascontiguousarray(mask, np.float64)
    C, D, H, W = image.shape
    sp = np.asarray(spacing, np.float64)
    out = np.empty(mask.shape, np.float64)
    lib().fgo_geodesic3d_f64(_p64(image), C, D, H, W, _p64(mask), mask.shape[0], _p64(sp),
                             _p64(out), float(v), float(lamb), 1.0 - float(lamb),
                             int(iterations), _threads(nthreads))
    return out
