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


def test_spawned_ranks_report_the_world_size():
    """`bench.py --gpus 2` without torchrun launches two ranks itself; both
    arms report the real world size, and the time is the maximum over ranks
    (here gloo on the CPU: the multi-rank plumbing without a workload)."""
    import json
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    for extra in ([], ["--impl", "reference"]):
        out = subprocess.run([sys.executable, "bench.py", "--gpus", "2", "--dry-run", *extra], cwd=root, env=env,
                             capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stderr[-2000:]
        lines = [json.loads(ln) for ln in out.stdout.splitlines() if ln.startswith("{")]
        assert len(lines) == 1, out.stdout
        assert lines[0]["n_gpus"] == 2 and lines[0]["max_over_ranks"] == 2.0
        assert lines[0].get("impl") == ("reference" if extra else None)
