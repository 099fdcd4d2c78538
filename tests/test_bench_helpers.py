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


def test_sweep_kernel_names_follow_the_plans():
    """The bench line's kernel: the one-CTA kernel for a 2D image of fewer
    than 16384 cells, the planner's row tiles for 512 x 512, pinned plans'
    kinds."""
    from fastgeodis_gb300 import _lib

    w = bench.workload("c1")
    assert bench.sweep_kernel_name(w, None) == "fg_row_tile_kernel"
    small = dict(w, image=np.zeros((1, 1, 64, 200), np.float32))
    assert bench.sweep_kernel_name(small, None) == "fg_row2d_kernel"
    pinned = {"plans": {"1,1,512": [8, 1, 128, 0]}}
    assert bench.sweep_kernel_name(w, pinned) == "fg_pass_kernel"
    vol = dict(w, dims=3, image=np.zeros((1, 1, 16, 32, 32), np.float32))
    pinned = {"plans": {"2,32,32": [8, 16, 32, _lib.FG_PLAN_CLUSTER | _lib.FG_PLAN_RUNS2], "2,16,32": [0, 0, 0, 0]}}
    names = bench.sweep_kernel_name(vol, pinned).split(" + ")
    assert names[0] == "fg_sweep_cluster_kernel" and len(names) == 2
