"""Loader for the committed golden vectors (tests/golden/*.npz), which were
produced by the reference's own CPU build (tests/golden/make_golden.py)."""
import glob
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_all():
    cases = []
    for path in sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))):
        with np.load(path) as z:
            params = json.loads(str(z["params"]))
            cases.append(dict(params, image=z["image"], mask=z["mask"], expected=z["expected"]))
    return cases


def names():
    return [os.path.basename(p)[:-4] for p in sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))]


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))
