"""bench.py helpers that run without a GPU."""
import numpy as np

import bench


def test_batch_cpu_sample_counts_plain_and_signed():
    rng = np.random.default_rng(5)
    imgs = [rng.random((C, H, W)).astype(np.float32) * 255 for C, H, W in [(1, 40, 52), (3, 36, 20), (1, 16, 64)]]
    masks = []
    for im in imgs:
        m = np.ones((1,) + im.shape[1:], np.float32)
        m[0, 3, 4] = 0
        masks.append(m)
    value, kind, cores, sample = bench.batch_cpu_sample(imgs, masks, [0.2, 0.7, 1.0], budget_s=0.0)
    assert kind == "port" and cores >= 1 and value > 0
    assert sample.startswith("1 images")  # one image then the budget is spent
    value, _, _, sample = bench.batch_cpu_sample(imgs, masks, [0.2, 0.7, 1.0], budget_s=1e9)
    assert sample.startswith("12 images")  # at most four rounds of the batch
