"""Generate the golden input/output vectors in this directory.

The outputs come from the reference's own CPU implementation
(masadcv/FastGeodis 1.0.5, ``FastGeodis/fastgeodis_cpu.cpp`` and the
signed/GSF composition in ``FastGeodis/fastgeodis.cpp``), compiled from the
reference sources by ``oracle/build_oracle.py:build_reference``.  That build
only exists where the reference source tree is mounted, so this script is run
once there and its ``.npz`` outputs are committed; the tests only read them.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build_oracle  # noqa: E402


def smooth_noise(rng, shape, sigma, lo, hi):
    from scipy.ndimage import gaussian_filter

    x = rng.uniform(lo, hi, size=shape).astype(np.float32)
    return gaussian_filter(x, sigma=sigma, truncate=4.0).astype(np.float32)


def disks(rng, shape, count, radius):
    m = np.ones(shape, np.float32)
    grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    for _ in range(count):
        c = [rng.integers(0, n) for n in shape]
        r2 = sum((g - ci) ** 2 for g, ci in zip(grids, c))
        m[r2 <= radius * radius] = 0.0
    return m


def cases(rng):
    out = []
    # 2D plain, one channel, several weights and iteration counts
    img = (rng.random((1, 37, 53)) * 255).astype(np.float32)
    m = disks(rng, (37, 53), 3, 2)[None]
    for lamb in (0.0, 0.37, 1.0):
        for it in (1, 2):
            out.append(dict(name=f"g2d_c1_l{lamb}_i{it}", op="geodesic2d", image=img, mask=m,
                            v=1e10, lamb=lamb, iter=it))
    # 2D three channels, odd width
    img = (rng.random((3, 40, 17)) * 255).astype(np.float32)
    m = disks(rng, (40, 17), 2, 3)[None]
    out.append(dict(name="g2d_c3", op="geodesic2d", image=img, mask=m, v=1e10, lamb=0.5, iter=2))
    # 2D soft mask with two mask channels (only channel 0 is swept)
    img = (rng.random((2, 23, 29))).astype(np.float32)
    m = rng.random((2, 23, 29)).astype(np.float32)
    out.append(dict(name="g2d_softmask_cm2", op="geodesic2d", image=img, mask=m, v=3.0, lamb=0.75, iter=3))
    # degenerate extents
    img = (rng.random((1, 1, 19)) * 10).astype(np.float32)
    m = np.ones((1, 1, 19), np.float32); m[0, 0, 7] = 0
    out.append(dict(name="g2d_h1", op="geodesic2d", image=img, mask=m, v=1e10, lamb=0.5, iter=2))
    img = (rng.random((1, 21, 1)) * 10).astype(np.float32)
    m = np.ones((1, 21, 1), np.float32); m[0, 4, 0] = 0
    out.append(dict(name="g2d_w1", op="geodesic2d", image=img, mask=m, v=1e10, lamb=0.5, iter=2))
    # the 512x512 benchmark recipe, shrunk: smoothed [0,255] noise, r=4 disks
    img = smooth_noise(rng, (96, 80), 3.0, 0, 255)[None]
    m = disks(rng, (96, 80), 5, 4)[None]
    out.append(dict(name="g2d_smooth", op="geodesic2d", image=img, mask=m, v=1e10, lamb=1.0, iter=2))
    out.append(dict(name="s2d_smooth", op="signed2d", image=img, mask=m, v=1e10, lamb=0.6, iter=2))
    out.append(dict(name="gsf2d_smooth", op="gsf2d", image=img, mask=m, v=1e10, lamb=0.8, iter=2, theta=0.5))
    img3 = (rng.random((3, 30, 26)) * 255).astype(np.float32)
    m3 = disks(rng, (30, 26), 2, 3)[None]
    out.append(dict(name="s2d_c3", op="signed2d", image=img3, mask=m3, v=1e10, lamb=0.3, iter=1))
    # 3D plain, anisotropic spacing
    img = rng.random((1, 7, 9, 11)).astype(np.float32)
    m = np.ones((1, 7, 9, 11), np.float32); m[0, 2, 3, 4] = 0
    for lamb in (0.0, 0.5, 1.0):
        out.append(dict(name=f"g3d_l{lamb}", op="geodesic3d", image=img, mask=m, v=1e10, lamb=lamb,
                        iter=3, spacing=[2.0, 0.5, 0.7]))
    img = rng.random((2, 12, 5, 16)).astype(np.float32)
    m = disks(rng, (12, 5, 16), 2, 1)[None]
    out.append(dict(name="g3d_c2", op="geodesic3d", image=img, mask=m, v=1e10, lamb=0.5, iter=4,
                    spacing=[1.0, 1.0, 1.0]))
    img = smooth_noise(rng, (10, 14, 18), 2.0, 0, 1)[None]
    m = np.ones((1, 10, 14, 18), np.float32); m[0, 3:6, 4:7, 5:8] = 0
    out.append(dict(name="g3d_cube", op="geodesic3d", image=img, mask=m, v=1e10, lamb=0.5, iter=4,
                    spacing=[2.0, 0.5, 0.5]))
    out.append(dict(name="s3d_cube", op="signed3d", image=img, mask=m, v=1e10, lamb=1.0, iter=2,
                    spacing=[2.0, 0.5, 0.5]))
    out.append(dict(name="gsf3d_cube", op="gsf3d", image=img, mask=m, v=1e10, lamb=1.0, iter=2,
                    spacing=[2.0, 0.5, 0.5], theta=0.01))
    img = rng.random((1, 1, 6, 9)).astype(np.float32)
    m = np.ones((1, 1, 6, 9), np.float32); m[0, 0, 2, 2] = 0
    out.append(dict(name="g3d_d1", op="geodesic3d", image=img, mask=m, v=1e10, lamb=0.5, iter=2,
                    spacing=[1.0, 1.5, 0.5]))
    # Toivanen's raster scan (FastGeodis/geodis_toivanen.cpp), same families
    img = smooth_noise(rng, (45, 38), 3.0, 0, 255)[None]
    m = disks(rng, (45, 38), 3, 3)[None]
    for lamb in (0.0, 0.6, 1.0):
        out.append(dict(name=f"t2d_l{lamb}", op="toivanen2d", image=img, mask=m, v=1e10, lamb=lamb, iter=2))
    out.append(dict(name="ts2d", op="signed_toivanen2d", image=img, mask=m, v=1e10, lamb=0.7, iter=1))
    out.append(dict(name="tgsf2d", op="gsf_toivanen2d", image=img, mask=m, v=1e10, lamb=0.8, iter=2, theta=0.5))
    img = (rng.random((3, 20, 33)) * 255).astype(np.float32)
    m = rng.random((2, 20, 33)).astype(np.float32)
    out.append(dict(name="t2d_c3_cm2", op="toivanen2d", image=img, mask=m, v=4.0, lamb=0.5, iter=3))
    img = (rng.random((1, 1, 23)) * 10).astype(np.float32)
    m = np.ones((1, 1, 23), np.float32); m[0, 0, 9] = 0
    out.append(dict(name="t2d_h1", op="toivanen2d", image=img, mask=m, v=1e10, lamb=0.5, iter=2))
    img = smooth_noise(rng, (9, 12, 14), 2.0, 0, 1)[None]
    m = np.ones((1, 9, 12, 14), np.float32); m[0, 3:5, 4:6, 5:8] = 0
    for lamb in (0.0, 0.5, 1.0):
        out.append(dict(name=f"t3d_l{lamb}", op="toivanen3d", image=img, mask=m, v=1e10, lamb=lamb, iter=2,
                        spacing=[2.0, 0.5, 0.7]))
    out.append(dict(name="ts3d", op="signed_toivanen3d", image=img, mask=m, v=1e10, lamb=1.0, iter=2,
                    spacing=[1.0, 1.0, 1.0]))
    out.append(dict(name="tgsf3d", op="gsf_toivanen3d", image=img, mask=m, v=1e10, lamb=1.0, iter=1,
                    spacing=[2.0, 0.5, 0.5], theta=0.01))
    img = rng.random((2, 5, 7, 6)).astype(np.float32)
    m = disks(rng, (5, 7, 6), 1, 1)[None]
    out.append(dict(name="t3d_c2", op="toivanen3d", image=img, mask=m, v=1e10, lamb=0.5, iter=3,
                    spacing=[1.0, 1.5, 0.5]))
    # more than four image channels (the reference sums L1 over any count)
    img = (rng.random((5, 41, 37)) * 255).astype(np.float32)
    m = disks(rng, (41, 37), 2, 2)[None]
    out.append(dict(name="g2d_c5", op="geodesic2d", image=img, mask=m, v=1e10, lamb=0.6, iter=2))
    out.append(dict(name="s2d_c5", op="signed2d", image=img, mask=m, v=1e10, lamb=0.4, iter=2))
    img = (rng.random((8, 33, 70)) * 255).astype(np.float32)
    m = disks(rng, (33, 70), 3, 2)[None]
    out.append(dict(name="g2d_c8_l1.0", op="geodesic2d", image=img, mask=m, v=1e10, lamb=1.0, iter=2))
    out.append(dict(name="gsf2d_c8", op="gsf2d", image=img, mask=m, v=1e10, lamb=0.5, iter=1, theta=0.5))
    img = rng.random((5, 9, 10, 12)).astype(np.float32)
    m = disks(rng, (9, 10, 12), 2, 1)[None]
    out.append(dict(name="g3d_c5", op="geodesic3d", image=img, mask=m, v=1e10, lamb=0.5, iter=2,
                    spacing=[1.5, 0.8, 1.1]))
    img = rng.random((8, 7, 9, 13)).astype(np.float32)
    m = disks(rng, (7, 9, 13), 2, 1)[None]
    out.append(dict(name="g3d_c8_l1.0", op="geodesic3d", image=img, mask=m, v=1e10, lamb=1.0, iter=2,
                    spacing=[1.0, 1.0, 1.0]))
    out.append(dict(name="s3d_c8", op="signed3d", image=img, mask=m, v=1e10, lamb=0.7, iter=2,
                    spacing=[2.0, 0.5, 0.5]))
    # lamb outside [0, 1] (the reference does not restrict it): a negative
    # image weight, and a negative step-length weight
    img = smooth_noise(rng, (47, 53), 2.0, 0.0, 255.0)[None]
    m = disks(rng, (47, 53), 3, 2)[None]
    out.append(dict(name="g2d_lneg", op="geodesic2d", image=img, mask=m, v=1e10, lamb=-0.4, iter=2))
    out.append(dict(name="g2d_l1.5", op="geodesic2d", image=img, mask=m, v=1e10, lamb=1.5, iter=2))
    out.append(dict(name="s2d_lneg", op="signed2d", image=img, mask=m, v=1e10, lamb=-0.25, iter=2))
    img3 = (rng.random((3, 29, 31)) * 255).astype(np.float32)
    out.append(dict(name="g2d_c3_lneg", op="geodesic2d", image=img3, mask=disks(rng, (29, 31), 2, 2)[None],
                    v=1e10, lamb=-0.3, iter=2))
    img = rng.random((1, 11, 13, 12)).astype(np.float32)
    m = disks(rng, (11, 13, 12), 2, 1)[None]
    out.append(dict(name="g3d_lneg", op="geodesic3d", image=img, mask=m, v=1e10, lamb=-0.3, iter=2,
                    spacing=[1.5, 0.8, 1.1]))
    return out


def run_reference(ref, c):
    import torch

    img = torch.from_numpy(c["image"])[None]
    m = torch.from_numpy(c["mask"])[None]
    v, lamb, it = c["v"], c["lamb"], c["iter"]
    op = c["op"]
    # argument conventions of FastGeodis/__init__.py:37-162, 526-585
    if op == "geodesic2d":
        r = ref.generalised_geodesic2d(img, m, v, lamb, 1 - lamb, it)
    elif op == "geodesic3d":
        r = ref.generalised_geodesic3d(img, m, c["spacing"], v, lamb, 1 - lamb, it)
    elif op == "signed2d":
        r = ref.signed_generalised_geodesic2d(img, m, v, lamb, 1 - lamb, it)
    elif op == "signed3d":
        r = ref.signed_generalised_geodesic3d(img, m, c["spacing"], v, lamb, 1 - lamb, it)
    elif op == "gsf2d":
        r = ref.GSF2d(img, m, c["theta"], v, lamb, it)
    elif op == "gsf3d":
        r = ref.GSF3d(img, m, c["theta"], c["spacing"], v, lamb, it)
    elif op == "toivanen2d":
        r = ref.generalised_geodesic2d_toivanen(img, m, v, lamb, 1 - lamb, it)
    elif op == "toivanen3d":
        r = ref.generalised_geodesic3d_toivanen(img, m, c["spacing"], v, lamb, 1 - lamb, it)
    elif op == "signed_toivanen2d":
        r = ref.signed_generalised_geodesic2d_toivanen(img, m, v, lamb, 1 - lamb, it)
    elif op == "signed_toivanen3d":
        r = ref.signed_generalised_geodesic3d_toivanen(img, m, c["spacing"], v, lamb, 1 - lamb, it)
    elif op == "gsf_toivanen2d":
        r = ref.GSF2d_toivanen(img, m, c["theta"], v, lamb, it)
    elif op == "gsf_toivanen3d":
        r = ref.GSF3d_toivanen(img, m, c["theta"], c["spacing"], v, lamb, it)
    else:
        raise ValueError(op)
    return r[0].numpy()


def main():
    build_oracle.build_reference()
    ref = build_oracle.load_reference()
    if ref is None:
        raise SystemExit("reference sources not available; golden vectors cannot be regenerated here")
    rng = np.random.default_rng(20241203)
    for c in cases(rng):
        expected = run_reference(ref, c)
        params = {k: c[k] for k in c if k not in ("image", "mask")}
        path = os.path.join(HERE, c["name"] + ".npz")
        if os.path.exists(path):  # rewrite only what changed (the archive bytes are not reproducible)
            with np.load(path) as z:
                if all(z[k].tobytes() == np.ascontiguousarray(v).tobytes() and z[k].shape == np.shape(v)
                       for k, v in (("image", c["image"]), ("mask", c["mask"]), ("expected", expected))) \
                        and json.loads(str(z["params"])) == params:
                    print(c["name"], "unchanged")
                    continue
        np.savez_compressed(path, image=c["image"], mask=c["mask"], expected=expected, params=json.dumps(params))
        print(c["name"], c["op"], c["image"].shape, float(np.abs(expected).max()))


if __name__ == "__main__":
    main()
