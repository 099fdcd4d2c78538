"""The engine on the reference's own sample data (its demos' inputs, read by
fastgeodis_gb300.io into tests/golden/demo/): the raster scan and Toivanen's
scan, geodesic (lamb 1) and Euclidean (lamb 0), must reproduce the digests of
the reference's CPU outputs bit for bit."""
import hashlib
import json
import os

import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import io as fgio

pytestmark = pytest.mark.gpu

DEMO = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "demo")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["demo2d", "demo3d"])
def test_demo_data_bits(name):
    with np.load(os.path.join(DEMO, name + ".npz")) as z:
        img, msk, p = z["image"], z["mask"], json.loads(str(z["params"]))
        mids = {k: z[k] for k in z.files if k.endswith("_mid")}
    ti = fgio.as_image_tensor(img).cuda()
    tm = torch.from_numpy(msk)[None, None].cuda()
    for lamb in p["lambs"]:
        for method in ("raster", "toivanen"):
            if p["spacing"] is None:
                f = fg.generalised_geodesic2d if method == "raster" else fg.generalised_geodesic2d_toivanen
                out = f(ti, tm, p["v"], lamb, p["iter"])
            else:
                f = fg.generalised_geodesic3d if method == "raster" else fg.generalised_geodesic3d_toivanen
                out = f(ti, tm, p["spacing"], p["v"], lamb, p["iter"])
            got = out[0, 0].cpu().numpy()
            key = f"{method}_l{lamb}"
            mid = got[got.shape[0] // 2]
            assert digest(got) == p["digests"][key], (name, key, float(np.abs(mid - mids[key + "_mid"]).max()))
    fg.check_status()
