"""Readers of the reference's sample data formats (fastgeodis_gb300.io) and
the golden vectors made from its demo data.

PNG decoding is checked against an encoder written here (every scanline
filter, grey / grey+alpha / RGB / RGBA / palette, 8 and 16 bits); NIfTI-1
against volumes written here (both byte orders, gzip or not, with and
without scaling).  The demo fixtures (tests/golden/demo/) hold the
reference's outputs on its own sample data; the oracle must reproduce their
digests bit for bit."""
import gzip
import hashlib
import json
import os
import struct
import zlib

import numpy as np
import pytest

from fastgeodis_gb300 import io as fgio
from oracle import build_oracle, oracle

HERE = os.path.dirname(os.path.abspath(__file__))
DEMO = os.path.join(HERE, "golden", "demo")
REF_DATA = os.path.join(build_oracle.DEFAULT_REF_ROOT, "data")


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def encode_png(arr, ctype, depth, filters, palette=None):
    """A minimal PNG encoder: rows filtered with the given filter types (cycled)."""
    H, W = arr.shape[:2]
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    a = arr.reshape(H, W * ch)
    if depth == 16:
        raw = np.stack([(a >> 8) & 0xFF, a & 0xFF], axis=-1).reshape(H, -1).astype(np.int64)
    else:
        raw = a.astype(np.int64)
    bpp = max(1, ch * depth // 8)
    out = bytearray()
    prev = np.zeros(raw.shape[1], np.int64)
    for r in range(H):
        f = filters[r % len(filters)]
        line = raw[r]
        enc = np.zeros_like(line)
        for i in range(line.size):
            left = line[i - bpp] if i >= bpp else 0
            up = prev[i]
            ul = prev[i - bpp] if i >= bpp else 0
            pred = [0, left, up, (left + up) >> 1, _paeth(left, up, ul)][f]
            enc[i] = (line[i] - pred) & 0xFF
        out.append(f)
        out += bytes(enc.astype(np.uint8))
        prev = line

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, 0))
    if palette is not None:
        png += chunk(b"PLTE", bytes(palette))
    data = zlib.compress(bytes(out))
    return png + chunk(b"IDAT", data[: len(data) // 2]) + chunk(b"IDAT", data[len(data) // 2:]) + chunk(b"IEND", b"")


@pytest.mark.parametrize("ctype,depth", [(0, 8), (0, 16), (2, 8), (2, 16), (3, 8), (4, 8), (6, 8), (6, 16)])
def test_png_round_trip_every_filter(tmp_path, ctype, depth):
    rng = np.random.default_rng(ctype * 100 + depth)
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    H, W = 13, 11
    hi = 256 if depth == 8 else 65536
    arr = rng.integers(0, hi, size=(H, W, ch)).astype(np.uint16 if depth == 16 else np.uint8)
    if ctype == 3:
        arr = arr % 7
    p = tmp_path / "x.png"
    p.write_bytes(encode_png(arr, ctype, depth, [0, 1, 2, 3, 4], palette=[0] * 21 if ctype == 3 else None))
    got = fgio.read_png(str(p))
    want = arr[..., 0] if ch == 1 else arr
    assert got.shape == want.shape and got.dtype == want.dtype
    assert np.array_equal(got, want)


def test_png_refuses_interlaced_and_garbage(tmp_path):
    p = tmp_path / "bad.png"
    p.write_bytes(b"not a png")
    with pytest.raises(ValueError):
        fgio.read_png(str(p))
    good = encode_png(np.zeros((2, 2, 1), np.uint8), 0, 8, [0])
    ihdr = struct.pack(">IIBBBBB", 2, 2, 8, 0, 0, 0, 1)  # interlace method 1
    bad = good[:16] + ihdr + struct.pack(">I", zlib.crc32(b"IHDR" + ihdr) & 0xFFFFFFFF) + good[33:]
    p.write_bytes(bad)
    with pytest.raises(ValueError, match="interlaced"):
        fgio.read_png(str(p))


def write_nifti(path, arr, spacing_xyz, end="<", slope=0.0, inter=0.0, dtype_code=4):
    hdr = bytearray(352)
    struct.pack_into(end + "i", hdr, 0, 348)
    dims = [arr.ndim] + list(arr.shape[::-1]) + [1] * (7 - arr.ndim)
    struct.pack_into(end + "8h", hdr, 40, *dims)
    struct.pack_into(end + "hh", hdr, 70, dtype_code, arr.dtype.itemsize * 8)
    struct.pack_into(end + "8f", hdr, 76, 1.0, *spacing_xyz, *([0.0] * (7 - len(spacing_xyz))))
    struct.pack_into(end + "3f", hdr, 108, 352.0, slope, inter)
    hdr[344:348] = b"n+1\x00"
    body = bytes(hdr) + arr.astype(arr.dtype.newbyteorder(end)).tobytes()
    if str(path).endswith(".gz"):
        body = gzip.compress(body)
    with open(path, "wb") as f:
        f.write(body)


@pytest.mark.parametrize("end", ["<", ">"])
@pytest.mark.parametrize("name", ["v.nii", "v.nii.gz"])
def test_nifti_round_trip(tmp_path, end, name):
    rng = np.random.default_rng(3)
    arr = rng.integers(-500, 1500, size=(5, 7, 9)).astype(np.int16)  # [z, y, x]
    p = tmp_path / name
    write_nifti(p, arr, (0.5, 0.75, 2.5), end=end)
    got, sp = fgio.read_nifti(str(p))
    assert got.dtype == np.int16 and np.array_equal(got, arr)
    assert sp == pytest.approx((2.5, 0.75, 0.5))
    write_nifti(p, arr, (1.0, 1.0, 1.0), end=end, slope=2.0, inter=-3.0)
    got, _ = fgio.read_nifti(str(p))
    assert got.dtype == np.float32 and np.array_equal(got, arr.astype(np.float32) * 2 - 3)


def demo_fixture(name):
    with np.load(os.path.join(DEMO, name + ".npz")) as z:
        return z["image"], z["mask"], json.loads(str(z["params"]))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


@pytest.mark.skipif(not os.path.isdir(REF_DATA), reason="the reference's sample data is not mounted")
def test_readers_on_the_reference_sample_data():
    img, _, _ = demo_fixture("demo2d")
    assert np.array_equal(fgio.read_png(os.path.join(REF_DATA, "img2d.png")), img)
    vol, _, p = demo_fixture("demo3d")
    full, sp = fgio.read_nifti(os.path.join(REF_DATA, "img3d.nii.gz"))
    assert full.shape == (45, 229, 300) and np.array_equal(full[18:38, 63:183, 93:233], vol)
    assert list(sp) == p["spacing"]
    t = fgio.as_image_tensor(fgio.read_png(os.path.join(REF_DATA, "brain.png")))
    assert tuple(t.shape) == (1, 3, 313, 323)


@pytest.mark.parametrize("name", ["demo2d", "demo3d"])
def test_oracle_reproduces_the_reference_on_its_demo_data(name):
    img, msk, p = demo_fixture(name)
    im = np.asarray(img, np.float32)[None]
    m = msk[None]
    for lamb in p["lambs"]:
        if p["spacing"] is None:
            got = oracle.geodesic2d(im, m, p["v"], lamb, p["iter"])[0]
            tv = oracle.toivanen2d(im, m, p["v"], lamb, p["iter"])[0]
        else:
            got = oracle.geodesic3d(im, m, p["spacing"], p["v"], lamb, p["iter"])[0]
            tv = oracle.toivanen3d(im, m, p["spacing"], p["v"], lamb, p["iter"])[0]
        assert digest(got) == p["digests"][f"raster_l{lamb}"], (name, lamb)
        assert digest(tv) == p["digests"][f"toivanen_l{lamb}"], (name, lamb, "toivanen")
