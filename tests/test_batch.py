"""Host-side planning of the batched 2D transform (no GPU): the queue order
of the jobs and when a signed image is split over two CTAs."""
import pytest

from fastgeodis_gb300.batch import ITEM_DTYPE, job_cost, plan_jobs


def test_item_layout():
    assert ITEM_DTYPE.itemsize == 88
    assert ITEM_DTYPE.fields["flags"][1] == 68  # after 7 pointers and C, H, W


def test_jobs_largest_first_and_pairs_adjacent():
    shapes = [(1, 100, 100), (3, 2000, 1900), (1, 800, 600), (2, 50, 60)]
    signed = [False, True, True, False]
    jobs = plan_jobs(shapes, signed, 2, sms=152, split=True)
    assert sorted(i for i, p in jobs if p in (0, 1)) == [0, 1, 2, 3]
    for k, (i, p) in enumerate(jobs):
        if p == 1:
            assert jobs[k + 1] == (i, 2)
    assert jobs[0] == (1, 1)  # the largest image first
    assert [p for i, p in jobs if not signed[i]] == [0, 0]
    assert all(p == 0 for _, p in plan_jobs(shapes, signed, 2, sms=152, split=False))


def test_auto_split_only_the_critical_images():
    # one huge signed image among many small ones: it alone is split
    shapes = [(3, 2000, 2000)] + [(1, 200, 200)] * 40
    signed = [True] * 41
    jobs = plan_jobs(shapes, signed, 2, sms=152)
    assert jobs[:2] == [(0, 1), (0, 2)]
    assert all(p == 0 for _, p in jobs[2:])
    # more work than the GPU runs at once: splitting would only add work
    many = [(3, 1000, 1000)] * 1000
    assert all(p == 0 for _, p in plan_jobs(many, [True] * 1000, 2, sms=152))


def test_job_cost_monotone():
    assert job_cost(1, 512, 512, 1, 2) < job_cost(3, 512, 512, 1, 2) < job_cost(3, 512, 512, 2, 2)
    assert job_cost(1, 256, 256, 1, 2) < job_cost(1, 1024, 1024, 1, 2)
    assert job_cost(1, 256, 256, 1, 4) == pytest.approx(2 * job_cost(1, 256, 256, 1, 2))


def test_plan_tiles_splits_only_the_critical_images():
    from fastgeodis_gb300.batch import plan_tiles, tiled_cost, job_cost

    # one large 3-channel image among many small ones: it alone is tiled
    shapes = [(3, 2000, 1900)] + [(1, 300, 300)] * 60
    tl = plan_tiles(shapes, [False] * 61, 2, 152)
    assert list(tl) == [0] and 2 <= tl[0] <= 8
    assert tiled_cost(3, 2000, 1900, 1, 2, tl[0]) < job_cost(3, 2000, 1900, 1, 2)
    # a batch of equal images that fills the GPU: nothing to gain
    assert plan_tiles([(1, 1024, 1024)] * 400, [False] * 400, 2, 152) == {}
    # small images are never tiled
    assert plan_tiles([(1, 200, 200)] * 3, [True] * 3, 2, 152) == {}


def test_tiled_width():
    from fastgeodis_gb300.batch import tiled_width

    assert tiled_width(1968, 3) == 656 and tiled_width(1968, 3) % 4 == 0
    assert tiled_width(30, 8) == 32  # at least the halo (a hand-off every 32 steps)
    assert tiled_width(30, 8, 8) == 8
    assert tiled_width(2048, 2) == 1024


def test_split_pairs_and_tiled_costs():
    from fastgeodis_gb300.batch import _rest_bound, plan_jobs, tiled_cost

    shapes = [(1, 500, 500), (3, 900, 1200), (2, 64, 64)]
    signed = [True, True, False]
    jobs = plan_jobs(shapes, signed, 2, sms=152, split=True)
    assert sorted(jobs) == [(0, 1), (0, 2), (1, 1), (1, 2), (2, 0)]
    for k, (i, p) in enumerate(jobs):
        if p == 1:
            assert jobs[k + 1] == (i, 2)
    # more CTAs per strip shorten a large image's chain, with diminishing returns
    c = [tiled_cost(3, 1544, 1968, 1, 2, k) for k in (2, 4, 8)]
    assert c[0] > c[1] > c[2] and (c[0] - c[1]) > (c[1] - c[2])
    # fewer SMs never make the batch's lower bound shorter
    assert _rest_bound(shapes, signed, 2, 8) >= _rest_bound(shapes, signed, 2, 152)
