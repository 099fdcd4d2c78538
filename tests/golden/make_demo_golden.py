"""Golden vectors from the reference's own sample data (its demos' inputs).

The reference's demos (FastGeodis ``samples/simpledemo2d.py`` and
``samples/simpledemo3d.py``) transform ``data/img2d.png`` (seed at row 100,
column 100) and a crop ``[18:38, 63:183, 93:233]`` of ``data/img3d.nii.gz``
(seed at ``[10, 60, 70]``, spacing from the file), with v = 1e10, 2
iterations, lamb 1.0 (geodesic) and 0.0 (Euclidean), by the raster scan and
by Toivanen's scan.  This script reads those files with
:mod:`fastgeodis_gb300.io` (the demos use PIL and SimpleITK), runs the
reference's own CPU build (``oracle/build_oracle.py:build_reference``) on the
demo configurations and writes ``demo/demo2d.npz`` / ``demo/demo3d.npz``: the demo's
input (in its stored integer type), the seed, the spacing, and per transform
the SHA-256 of the output's float32 bytes plus its middle row (2D) or slice
(3D) for diagnosis.  The tests compare the oracle and the GPU engine against
these digests, bit for bit.

Usage (where the reference tree is mounted):  python tests/golden/make_demo_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fastgeodis_gb300 import io as fgio  # noqa: E402
from oracle import build_oracle  # noqa: E402

REF_DATA = os.path.join(build_oracle.DEFAULT_REF_ROOT, "data")
V, ITERS = 1e10, 2
LAMBS = (1.0, 0.0)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def demo_inputs():
    """The demos' inputs: (name, image array (stored type), mask, spacing or None)."""
    img2d = fgio.read_png(os.path.join(REF_DATA, "img2d.png"))
    m2 = np.ones(img2d.shape, np.float32)
    m2[100, 100] = 0.0  # simpledemo2d.py:16
    vol, sp = fgio.read_nifti(os.path.join(REF_DATA, "img3d.nii.gz"))
    vol = vol[18:38, 63:183, 93:233]  # simpledemo3d.py:23
    m3 = np.ones(vol.shape, np.float32)
    m3[10, 60, 70] = 0.0  # simpledemo3d.py:15, 24-27 (mask = 1 - seed)
    return [("demo2d", img2d, m2, None), ("demo3d", vol, m3, [float(s) for s in sp])]


def main():
    import torch

    build_oracle.build_reference()
    ref = build_oracle.load_reference()
    if ref is None:
        raise SystemExit("reference sources not available; demo golden vectors cannot be regenerated here")
    for name, img, msk, sp in demo_inputs():
        ti = torch.from_numpy(np.asarray(img, np.float32))[None, None]
        tm = torch.from_numpy(msk)[None, None]
        out = {}
        for method in ("raster", "toivanen"):
            for lamb in LAMBS:
                if sp is None:
                    fn = ref.generalised_geodesic2d if method == "raster" else ref.generalised_geodesic2d_toivanen
                    r = fn(ti, tm, V, lamb, 1 - lamb, ITERS)
                else:
                    fn = ref.generalised_geodesic3d if method == "raster" else ref.generalised_geodesic3d_toivanen
                    r = fn(ti, tm, sp, V, lamb, 1 - lamb, ITERS)
                r = r[0, 0].numpy()
                key = f"{method}_l{lamb}"
                out[key] = digest(r)
                mid = r[r.shape[0] // 2]
                out[key + "_mid"] = mid
        params = {"v": V, "iter": ITERS, "lambs": list(LAMBS), "spacing": sp,
                  "digests": {k: v for k, v in out.items() if not k.endswith("_mid")}}
        arrays = {k: v for k, v in out.items() if k.endswith("_mid")}
        os.makedirs(os.path.join(HERE, "demo"), exist_ok=True)
        np.savez_compressed(os.path.join(HERE, "demo", name + ".npz"), image=img, mask=msk,
                            params=json.dumps(params), **arrays)
        print(name, img.shape, img.dtype, sp, params["digests"])


if __name__ == "__main__":
    main()
