"""Reading the reference's sample data formats: PNG images and NIfTI-1 volumes.

The reference's demos load their inputs with PIL (``np.asarray(Image.open(p),
np.float32)``) and SimpleITK (``sitk.GetArrayFromImage(sitk.ReadImage(p))``,
spacing reversed to (z, y, x)) -- FastGeodis ``samples/simpledemo2d.py:11``,
``samples/simpledemo3d.py:14-24``.  Neither library is a dependency here, so
this module reads both formats directly (zlib / gzip from the standard
library) and returns arrays laid out as those calls return them:

* :func:`read_png` -> ``[H, W]`` for grey, ``[H, W, 2]`` grey+alpha,
  ``[H, W, 3]`` RGB, ``[H, W, 4]`` RGBA; palette images give their palette
  indices ``[H, W]`` (PIL's mode ``P``).  8- and 16-bit samples, all five
  scanline filters; interlaced files are refused.
* :func:`read_nifti` -> ``(array [z, y, x], spacing (z, y, x))`` for
  ``.nii`` / ``.nii.gz`` single-file NIfTI-1 volumes of the common voxel
  types, in stored order, with the header's scaling applied when it is not
  the identity.

:func:`as_image_tensor` turns such an array into the ``[1, C, ...]`` float32
tensor the transforms take.
"""
from __future__ import annotations

import gzip
import struct
import zlib
from typing import Tuple

import numpy as np

_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_PNG_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}  # colour type -> samples per pixel


def _unfilter(raw: bytes, rows: int, stride: int, bpp: int) -> np.ndarray:
    """Undo the PNG scanline filters (none, sub, up, average, Paeth)."""
    data = np.frombuffer(raw, dtype=np.uint8)
    if data.size != rows * (stride + 1):
        raise ValueError("PNG: image data has the wrong length")
    data = data.reshape(rows, stride + 1)
    out = np.zeros((rows, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for r in range(rows):
        ftype = int(data[r, 0])
        line = data[r, 1:].astype(np.int32)
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        elif ftype == 1:
            # running sum per byte lane of a pixel
            pad = (-stride) % bpp
            v = np.concatenate([line, np.zeros(pad, np.int32)]).reshape(-1, bpp)
            cur = (np.cumsum(v, axis=0) & 0xFF).reshape(-1)[:stride]
        elif ftype in (3, 4):
            cur = np.zeros(stride, dtype=np.int32)
            ln, pv = line.tolist(), prev.tolist()
            c = [0] * stride
            for i in range(stride):
                a = c[i - bpp] if i >= bpp else 0
                b = pv[i]
                if ftype == 3:
                    c[i] = (ln[i] + ((a + b) >> 1)) & 0xFF
                else:
                    cc = pv[i - bpp] if i >= bpp else 0
                    p = a + b - cc
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - cc)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else cc)
                    c[i] = (ln[i] + pred) & 0xFF
            cur = np.asarray(c, dtype=np.int32)
        else:
            raise ValueError(f"PNG: unknown filter type {ftype}")
        out[r] = cur
        prev = cur
    return out


def read_png(path: str) -> np.ndarray:
    """Decode a PNG file into a numpy array (uint8, or uint16 for 16-bit
    samples), shaped as ``np.asarray(PIL.Image.open(path))``."""
    with open(path, "rb") as f:
        blob = f.read()
    if blob[:8] != _PNG_SIG:
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos + 8 <= len(blob):
        (n,) = struct.unpack(">I", blob[pos:pos + 4])
        kind = blob[pos + 4:pos + 8]
        body = blob[pos + 8:pos + 8 + n]
        if len(body) != n:
            raise ValueError(f"{path}: truncated {kind!r} chunk")
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + n
    if hdr is None or not idat:
        raise ValueError(f"{path}: missing IHDR or IDAT")
    W, H, depth, ctype, comp, filt, interlace = hdr
    if comp != 0 or filt != 0:
        raise ValueError(f"{path}: unknown compression or filter method")
    if interlace != 0:
        raise ValueError(f"{path}: interlaced PNG is not supported")
    if ctype not in _PNG_CHANNELS or depth not in (8, 16) or (ctype == 3 and depth != 8):
        raise ValueError(f"{path}: colour type {ctype} at bit depth {depth} is not supported")
    ch = _PNG_CHANNELS[ctype]
    bps = depth // 8
    stride = W * ch * bps
    rows = _unfilter(zlib.decompress(b"".join(idat)), H, stride, max(1, ch * bps))
    if depth == 16:
        px = rows.reshape(H, W * ch, 2).astype(np.uint16)
        arr = (px[..., 0] << 8) | px[..., 1]
    else:
        arr = rows
    arr = arr.reshape(H, W, ch)
    return arr[..., 0] if ch == 1 else arr


_NIFTI_TYPES = {2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64, 256: np.int8,
                512: np.uint16, 768: np.uint32, 1024: np.int64, 1280: np.uint64}


def read_nifti(path: str) -> Tuple[np.ndarray, Tuple[float, ...]]:
    """Read a single-file NIfTI-1 volume (``.nii`` or ``.nii.gz``).

    Returns the voxel array in the order SimpleITK's GetArrayFromImage gives
    it (slowest axis first: ``[z, y, x]`` for a 3D volume) and the spacing in
    the same order (the reference demo's ``spacing_raw`` reversed)."""
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rb") as f:
        blob = f.read()
    if len(blob) < 348:
        raise ValueError(f"{path}: too short for a NIfTI-1 header")
    for end in ("<", ">"):
        if struct.unpack(end + "i", blob[:4])[0] == 348:
            break
    else:
        raise ValueError(f"{path}: not a NIfTI-1 file (sizeof_hdr != 348)")
    if blob[344:347] != b"n+1":
        raise ValueError(f"{path}: only single-file NIfTI-1 ('n+1') is supported")
    dim = struct.unpack(end + "8h", blob[40:56])
    datatype = struct.unpack(end + "h", blob[70:72])[0]
    pixdim = struct.unpack(end + "8f", blob[76:108])
    vox_offset, slope, inter = struct.unpack(end + "3f", blob[108:120])
    nd = int(dim[0])
    if not 1 <= nd <= 7:
        raise ValueError(f"{path}: bad dimension count {nd}")
    if datatype not in _NIFTI_TYPES:
        raise ValueError(f"{path}: voxel datatype {datatype} is not supported")
    shape_xyz = [int(d) for d in dim[1:1 + nd]]
    dt = np.dtype(_NIFTI_TYPES[datatype]).newbyteorder(end)
    count = int(np.prod(shape_xyz))
    off = int(vox_offset)
    data = np.frombuffer(blob, dtype=dt, count=count, offset=off)
    arr = data.reshape(shape_xyz[::-1]).astype(dt.newbyteorder("="))  # x fastest in the file
    while arr.ndim > 3 and arr.shape[0] == 1:  # trailing unit dimensions (t, ...)
        arr = arr[0]
    if slope != 0.0 and not (slope == 1.0 and inter == 0.0):
        arr = arr.astype(np.float32) * np.float32(slope) + np.float32(inter)
    spacing = tuple(float(p) for p in pixdim[1:1 + min(nd, 3)])[::-1]
    return arr, spacing


def as_image_tensor(arr: np.ndarray, channels_last: bool = True):
    """``[1, C, ...]`` float32 tensor of an image array: a 2D or 3D array
    gives one channel; with `channels_last`, a trailing axis of 2-4 samples
    (RGB, RGBA, grey+alpha) becomes the channel axis."""
    import torch

    a = np.asarray(arr, dtype=np.float32)
    if channels_last and a.ndim == 3 and a.shape[-1] in (2, 3, 4):
        a = np.moveaxis(a, -1, 0)
    else:
        a = a[None]
    return torch.from_numpy(np.ascontiguousarray(a))[None]
