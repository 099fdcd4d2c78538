"""Autotuner: candidate plans respect the engine's tiling rules (CPU), pinned
plans round-trip through the C ABI and JSON (CPU), and tuned transforms give
the same bits as the oracle (GPU)."""
import numpy as np
import pytest
import torch

from fastgeodis_gb300 import _lib, tune


@pytest.mark.parametrize("cross,N1,N2", [(1, 1, 5), (1, 1, 300), (1, 1, 2048), (2, 7, 9), (2, 128, 256),
                                         (2, 256, 256), (2, 40, 600), (2, 2048, 8)])
@pytest.mark.parametrize("sms", [152, 8])
@pytest.mark.parametrize("lean", [False, True])
@pytest.mark.parametrize("fracs", [(1.0,), (1.0, 0.5, 0.34)])
def test_candidates_follow_the_tiling_rules(cross, N1, N2, sms, lean, fracs):
    cands = tune.candidates(cross, N1, N2, sms, lean=lean, tile_fracs=fracs)
    if cross == 1 or N1 * N2 <= sms * 512:
        assert cands, "a cross-section that fits the SMs has a plan"
    assert len(set(cands)) == len(cands)
    max_threads = tune.THREADS_LEAN if (lean and cross == 2) else tune.THREADS
    for S, T1, T2 in cands:
        assert S in (4, 8)
        t1, t2 = -(-N1 // T1), -(-N2 // T2)
        assert t1 * t2 <= sms
        assert 1 <= T2 <= N2 and 1 <= T1 <= max(N1, 1)
        if cross == 1:
            assert T1 == 1
        K1 = S if cross == 2 and t1 > 1 else 0
        K2 = S if t2 > 1 else 0
        if t2 > 1:
            assert T2 % 4 == 0 and T2 >= K2
        if t1 > 1:
            assert T1 >= K1
        R1 = T1 + 2 * K1 if cross == 2 else 1
        R2 = T2 + 2 * K2
        assert R1 * R2 <= 4 * max_threads and R1 * (-(-R2 // 4)) <= max_threads


def test_fewer_tile_candidates_for_concurrent_transforms():
    one = tune.candidates(2, 256, 256, 152, lean=True)
    conc = tune.candidates(2, 256, 256, 152, lean=True, tile_fracs=(1.0, 0.5, 0.34))
    assert set(one) <= set(conc)
    tiles = lambda c: -(-256 // c[1]) * -(-256 // c[2])  # noqa: E731
    assert min(tiles(c) for c in conc) <= 52 < min(tiles(c) for c in one)


@pytest.mark.parametrize("N1,N2", [(256, 256), (128, 256), (20, 27), (2, 8), (1, 64), (300, 300)])
def test_cluster_candidates_fit_the_kernel(N1, N2):
    for lean in (False, True):
        for S, T1, T2, flags in tune.cluster_candidates(2, N1, N2, lean_capable=lean):
            assert flags & _lib.FG_PLAN_CLUSTER and T2 == N2
            rpt = 2 if flags & _lib.FG_PLAN_RUNS2 else 1
            assert T1 % rpt == 0
            g = -(-N1 // T1)
            threads = T1 // rpt * -(-N2 // 4)
            assert 2 <= g <= 16 and threads <= (1024 if lean and rpt == 1 else 512)
            assert bool(flags & _lib.FG_PLAN_LEAN) == (threads > 512)
    for c in tune.cluster_candidates(2, N1, N2, one_channel=False):
        assert not c[3] & _lib.FG_PLAN_RUNS2
    assert tune.cluster_candidates(1, 1, 512) == []
    if N1 * -(-N2 // 4) > 16 * 512 * 2:  # 16 CTAs of 512 threads with 2 runs each
        assert tune.cluster_candidates(2, N1, N2) == []


@pytest.mark.parametrize("N2,C", [(128, 1), (300, 3), (512, 4), (5000, 1), (64, 1), (300, 5)])
def test_row_tile_candidates_pin_row_tiles(N2, C):
    """Each 2D row-tile candidate pins as a row-tile plan (T2 + 2 S threads
    at most 512, narrower than the row); none for volumes or 5+ channels."""
    L = _lib.load()
    cands = tune.row_tile_candidates(1, N2, 152, C)
    assert (cands == []) == (C > 4 or N2 <= 32)
    try:
        for S, T1, T2, flags in cands:
            clu = -(-N2 // T2) <= 16 and S <= T2
            assert flags in (_lib.FG_PLAN_ROWS, _lib.FG_PLAN_ROWS | _lib.FG_PLAN_CLUSTER)
            assert T1 == 1 and T2 < N2 and T2 + 2 * S <= 512 and (clu or flags == _lib.FG_PLAN_ROWS)
            _lib.check(L.fg_plan_override(1, 1, N2, S, T1, T2, flags))
            p = _lib.plan_describe(1, 1, N2, C=C)
            assert p["lean"] == flags and (p["S"], p["T2"]) == (S, T2), (S, T2, p)
        assert sum(f != _lib.FG_PLAN_ROWS for *_, f in cands) == sum(
            -(-N2 // T2) <= 16 and S <= T2 for S, _, T2, f in cands if f == _lib.FG_PLAN_ROWS)
    finally:
        _lib.check(L.fg_plan_override(1, 1, N2, 0, 0, 0, 0))
    assert tune.row_tile_candidates(2, 64, 64, 152) == []


def test_pass_keys():
    assert tune.pass_keys((5, 7)) == [(1, 1, 7), (1, 1, 5)]
    assert tune.pass_keys((6, 6)) == [(1, 1, 6)]
    assert tune.pass_keys((3, 4, 5)) == [(2, 4, 5), (2, 3, 5), (2, 3, 4)]
    assert tune.pass_keys((8, 8, 8)) == [(2, 8, 8)]
    with pytest.raises(ValueError):
        tune.pass_keys((1, 2, 3, 4))


def test_override_validation_and_round_trip(tmp_path):
    L = _lib.load()
    assert L.fg_plan_override(2, 64, 64, 3, 8, 8, 0) == _lib.FG_ERR_INVALID_ARGUMENT  # S not a power of two <= 8
    assert L.fg_plan_override(2, 64, 64, 4, 8, 6, 0) == _lib.FG_ERR_INVALID_ARGUMENT  # T2 not a multiple of 4
    assert L.fg_plan_override(3, 64, 64, 4, 8, 8, 0) == _lib.FG_ERR_INVALID_ARGUMENT
    res = {(2, 64, 64): (4, 8, 16, 1, 0.5), (1, 1, 100): (8, 1, 52, 0, 0.25), (2, 9, 9): (0, 0, 0, 0, 0.1)}
    path = str(tmp_path / "plans.json")
    tune.save(res, path)
    back = tune.load(path)
    assert back == res
    tune.clear((64, 64, 64))
    tune.clear((100, 100))


def _case(shape, C, seed):
    rng = np.random.default_rng(seed)
    img = rng.random((C,) + tuple(shape)).astype(np.float32)
    m = np.ones((1,) + tuple(shape), np.float32)
    for _ in range(3):
        m[(0,) + tuple(int(rng.integers(0, n)) for n in shape)] = 0
    return img, m


@pytest.mark.gpu
@pytest.mark.parametrize("shape,C", [((300, 517), 1), ((40, 72, 64), 2), ((24, 24, 24), 1), ((12, 160, 144), 1)])
def test_every_candidate_plan_gives_the_oracle_bits(shape, C):
    import fastgeodis_gb300 as fg
    from golden_cases import bits_equal
    from oracle import oracle

    img, m = _case(shape, C, 11)
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    if len(shape) == 2:
        want = oracle.geodesic2d(img, m, 1e10, 0.6, 2)
        run = lambda: fg.generalised_geodesic2d(ti, tm, 1e10, 0.6, 2)
    else:
        sp = [1.5, 0.8, 1.1]
        want = oracle.geodesic3d(img, m, sp, 1e10, 0.6, 2)
        run = lambda: fg.generalised_geodesic3d(ti, tm, sp, 1e10, 0.6, 2)
    L = _lib.load()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    try:
        for key in tune.pass_keys(shape):
            # fewer, larger tiles too: 1024-thread regions where the variant allows them
            for c in tune.candidates(*key, sms, lean=(C == 1), tile_fracs=(1.0, 0.3, 0.1), max_per_step=8):
                for lean in ((0, 1) if C == 1 and len(shape) == 3 else (0,)):  # both register budgets
                    _lib.check(L.fg_plan_override(*key, *c, lean))
                    got = run()[0].cpu().numpy()
                    assert bits_equal(got, want), (key, c, lean, np.abs(got - want).max())
            for c in tune.row_tile_candidates(*key[::2], sms, C):  # 2D: row tiles
                _lib.check(L.fg_plan_override(*key, *c))
                got = run()[0].cpu().numpy()
                assert bits_equal(got, want), (key, c, np.abs(got - want).max())
            _lib.check(L.fg_plan_override(*key, 0, 0, 0, 0))
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.gpu
def test_autotune_pins_plans_and_keeps_results():
    import fastgeodis_gb300 as fg
    from golden_cases import bits_equal
    from oracle import oracle

    shape = (36, 80, 96)
    try:
        # two modes (lamb 0: no image term; 0.5: general): one plan per cross-section and mode
        res = tune.autotune(shape, channels=1, lambs=[0.0, 0.5], iterations=1, repeats=2, max_per_step=4, per_mode=True)
        keys = tune.pass_keys(shape)
        assert set(res) == set(keys) | {k + (m,) for k in keys for m in (tune.MODE_GENERAL, tune.MODE_EUCLID)}
        for S, T1, T2, flags, ms in res.values():
            assert ms > 0 and S in (0, 4, 8)
            assert flags & ~(_lib.FG_PLAN_LEAN | _lib.FG_PLAN_CLUSTER | _lib.FG_PLAN_RUNS2) == 0
        img, m = _case(shape, 1, 5)
        for lamb in (0.0, 0.5):
            got = fg.generalised_geodesic3d(torch.from_numpy(img)[None].cuda(), torch.from_numpy(m)[None].cuda(),
                                            [1.0, 1.0, 1.0], 1e10, lamb, 2)[0].cpu().numpy()
            assert bits_equal(got, oracle.geodesic3d(img, m, [1.0, 1.0, 1.0], 1e10, lamb, 2)), lamb
        res1 = tune.autotune(shape, channels=1, lambs=[0.5, 0.5], iterations=1, repeats=1, max_per_step=2)
        assert set(res1) == set(tune.pass_keys(shape))  # one mode: plans for every mode
        fg.check_status()
    finally:
        tune.clear(shape)


def test_per_mode_overrides():
    """A plan pinned for one arithmetic mode serves that mode's passes only
    and wins over a plan pinned for every mode; clearing removes both."""
    L = _lib.load()
    key = (2, 256, 256)
    model = [_lib.plan_describe(*key, C=1, maps=1, mode=m) for m in range(3)]
    try:
        _lib.check(L.fg_plan_override(*key, 8, 16, 256, _lib.FG_PLAN_CLUSTER | _lib.FG_PLAN_RUNS2
                                      | _lib.FG_PLAN_MODE(tune.MODE_GENERAL)))
        _lib.check(L.fg_plan_override(*key, 4, 32, 64, 0))  # every mode
        general = _lib.plan_describe(*key, C=1, maps=1, mode=tune.MODE_GENERAL)
        assert general["tiles1"] == 16 and general["lean"] & _lib.FG_PLAN_CLUSTER
        for m in (tune.MODE_EUCLID, tune.MODE_GEO):
            p = _lib.plan_describe(*key, C=1, maps=1, mode=m)
            assert (p["S"], p["T1"], p["T2"]) == (4, 32, 64) and not p["lean"] & _lib.FG_PLAN_CLUSTER
        assert tune.mode_of(0.0) == tune.MODE_EUCLID and tune.mode_of(1.0) == tune.MODE_GEO
        assert tune.mode_of(0.5) == tune.MODE_GENERAL
    finally:
        tune.clear((256, 256, 256))
    assert [_lib.plan_describe(*key, C=1, maps=1, mode=m) for m in range(3)] == model
