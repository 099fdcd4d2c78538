"""CPU tests of the pass planner through fg_plan_describe: every plan it
returns respects the kernel's limits (region cells, threads, co-resident
tiles, shared memory) and the tiling rules, for 2D rows and 3D planes, and
honours plan overrides and tuning caps.  No kernel is launched."""
import os
import re

import pytest

from fastgeodis_gb300 import _lib

SMEM_LIMIT = 227 * 1024
SHAPES = [(1, 1, 1), (1, 1, 5), (1, 1, 300), (1, 1, 512), (1, 1, 2048), (1, 1, 4099),
          (2, 1, 1), (2, 3, 7), (2, 16, 16), (2, 64, 64), (2, 128, 256), (2, 256, 256), (2, 40, 600),
          (2, 2048, 8), (2, 300, 257)]


def max_threads(cross, C, maps, mode):
    """1024 for the 64-register volume variants (one image channel or none, one map), else 512."""
    cimg = 0 if mode == 1 else C
    return 1024 if (cross == 2 and cimg <= 1 and maps == 1) else 512


def ring_pitch(f):
    f = (f + 3) // 4 * 4
    return f + (36 - f % 32) % 32


def cluster_smem(C, M, T1, N2, NT, rpt, depth):
    """Shared-memory bytes of a cluster sweep CTA (the layout of ClusterLayout:
    two rows of each ring; the passes write in place)."""
    rpr = -(-N2 // 4)
    rowf = ring_pitch((T1 + 2) * (4 * rpr + 8))
    edgef = ring_pitch((T1 + 2) * (rpr + 2) * 2)
    floats = (2 * M + 2 * C) * (rowf + edgef) + depth * (M + C) * rpt * NT * 4
    return floats * 4 + 16


def check_plan(cross, N1, N2, p, sms, C=1, maps=1, mode=0):
    S, T1, T2, K1, K2, t1, t2, nt, depth, smem, lean = (p[k] for k in _lib.PLAN_FIELDS)
    assert S in (1, 2, 4, 8, 16, 32) and depth in (2, 4, 8)
    assert t1 == -(-N1 // T1) and t2 == -(-N2 // T2)
    assert t1 * t2 <= sms, "all tiles must be co-resident"
    if cross == 1:
        assert T1 == 1 and K1 == 0
    assert K1 == (S if t1 > 1 else 0) and K2 == (S if t2 > 1 else 0)
    if t2 > 1:
        assert T2 % 4 == 0, "runs of 4 must not straddle tiles"
    assert T1 >= K1 and T2 >= K2, "a halo reaches only the adjacent tiles"
    R1 = T1 + 2 * K1 if cross == 2 else 1
    R2 = T2 + 2 * K2
    if lean & _lib.FG_PLAN_ROWS:
        # row tiles: 2D, one thread per cell of a tile and its halos, at most
        # 512; as one thread-block cluster: 2 to 16 tiles, halos within a tile
        assert lean in (_lib.FG_PLAN_ROWS, _lib.FG_PLAN_ROWS | _lib.FG_PLAN_CLUSTER)
        assert cross == 1 and C <= 4 and R2 <= nt <= 512 and nt % 32 == 0
        if lean & _lib.FG_PLAN_CLUSTER:
            assert t2 <= 16 and K2 == S <= T2
        assert smem <= SMEM_LIMIT
        return
    runs = R1 * (-(-R2 // 4))
    mt = max_threads(cross, C, maps, mode)
    assert R1 * R2 <= 4 * mt and runs <= nt <= mt and nt % 32 == 0
    assert lean in (0, 1)
    if lean:
        assert mt == 1024, "only lean-capable variants use the 64-register kernel"
    else:
        assert nt <= 512, "the 128-register kernel stops at 512 threads"
    assert smem <= SMEM_LIMIT


@pytest.mark.parametrize("cross,N1,N2", SHAPES)
@pytest.mark.parametrize("C,maps,mode", [(1, 1, 0), (1, 1, 1), (1, 1, 2), (3, 1, 0), (4, 2, 0), (1, 2, 1)])
@pytest.mark.parametrize("wt", [False, True])
def test_plans_respect_kernel_limits(cross, N1, N2, C, maps, mode, wt):
    try:
        p = _lib.plan_describe(cross, N1, N2, C, maps, mode, wt, 152)
    except RuntimeError:
        # only cross-sections larger than the SMs' regions may lack a plan
        assert N1 * N2 > 152 * 1024
        return
    check_plan(cross, N1, N2, p, 152, C, maps, mode)


@pytest.mark.parametrize("sms", [1, 8, 76, 152])
def test_plans_scale_with_sm_count(sms):
    for cross, N1, N2 in [(1, 1, 2048), (2, 64, 64), (2, 30, 40)]:
        try:
            p = _lib.plan_describe(cross, N1, N2, 1, 1, 0, False, sms)
        except RuntimeError:
            assert N1 * N2 > sms * 1024
            continue
        check_plan(cross, N1, N2, p, sms)


def test_override_is_used_and_cleared():
    L = _lib.load()
    base = _lib.plan_describe(2, 256, 256)
    _lib.check(L.fg_plan_override(2, 256, 256, 4, 20, 24, 0))
    try:
        p = _lib.plan_describe(2, 256, 256)
        assert (p["S"], p["T1"], p["T2"]) == (4, 20, 24)
        check_plan(2, 256, 256, p, 152)
    finally:
        _lib.check(L.fg_plan_override(2, 256, 256, 0, 0, 0, 0))
    assert _lib.plan_describe(2, 256, 256) == base


def test_lean_override():
    L = _lib.load()
    _lib.check(L.fg_plan_override(2, 256, 256, 8, 14, 32, 1))
    try:
        p = _lib.plan_describe(2, 256, 256)          # one channel, one map: lean-capable
        assert p["lean"] == 1 and p["threads"] <= 512
        q = _lib.plan_describe(2, 256, 256, C=3)     # three channels: no 64-register kernel
        assert q["lean"] == 0
    finally:
        _lib.check(L.fg_plan_override(2, 256, 256, 0, 0, 0, 0))
    assert _lib.plan_describe(2, 256, 256)["lean"] == 0 or _lib.plan_describe(2, 256, 256)["threads"] > 512


def test_override_that_does_not_fit_falls_back_to_the_model():
    L = _lib.load()
    base = _lib.plan_describe(2, 256, 256)
    _lib.check(L.fg_plan_override(2, 256, 256, 8, 64, 64, 0))  # region 80 x 80 > 2048 cells
    try:
        assert _lib.plan_describe(2, 256, 256) == base
    finally:
        _lib.check(L.fg_plan_override(2, 256, 256, 0, 0, 0, 0))


def test_tuning_caps_region_and_tiles():
    L = _lib.load()
    _lib.check(L.fg_set_tuning(200, 40))
    try:
        p = _lib.plan_describe(2, 64, 64)
        R1 = p["T1"] + 2 * p["K1"]
        R2 = p["T2"] + 2 * p["K2"]
        assert R1 * R2 <= 200 and p["tiles1"] * p["tiles2"] <= 40
    finally:
        _lib.check(L.fg_set_tuning(0, 0))


def test_bad_queries():
    with pytest.raises(ValueError):
        _lib.plan_describe(3, 4, 4)
    with pytest.raises(ValueError):
        _lib.plan_describe(2, 4, 4, maps=3)


@pytest.mark.parametrize("N1,N2", [(256, 256), (128, 256), (20, 27), (64, 64), (9, 100), (2, 8)])
@pytest.mark.parametrize("C,maps,mode", [(1, 1, 0), (1, 1, 1), (3, 1, 0), (1, 2, 2)])
@pytest.mark.parametrize("wt", [False, True])
@pytest.mark.parametrize("G", [2, 4, 16])
def test_cluster_plans(N1, N2, C, maps, mode, wt, G):
    L = _lib.load()
    T1 = -(-N1 // G)
    _lib.check(L.fg_plan_override(2, N1, N2, 8, T1, N2, _lib.FG_PLAN_CLUSTER))
    try:
        p = _lib.plan_describe(2, N1, N2, C, maps, mode, wt)
    finally:
        _lib.check(L.fg_plan_override(2, N1, N2, 0, 0, 0, 0))
    runs = T1 * -(-N2 // 4)
    g = -(-N1 // T1)
    mt = max_threads(2, C, maps, mode)
    if not p["lean"] & _lib.FG_PLAN_CLUSTER:
        # no cluster plan: one strip too many threads, or a single strip
        assert runs > mt or g < 2
        return
    assert (p["tiles1"], p["tiles2"], p["K1"], p["K2"], p["T1"], p["T2"]) == (g, 1, 0, 0, T1, N2)
    assert 2 <= g <= 16 and runs <= p["threads"] <= mt and p["threads"] % 32 == 0
    assert p["smem"] <= SMEM_LIMIT and p["depth"] in (2, 4, 8)
    if wt:
        assert p["S"] in (2, 4, 8)  # the apron rings hold two steps at least
    if p["threads"] > 512:
        assert p["lean"] & _lib.FG_PLAN_LEAN


def test_cluster_override_validation():
    L = _lib.load()
    assert L.fg_plan_override(1, 1, 256, 8, 1, 256, _lib.FG_PLAN_CLUSTER) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_plan_override(2, 64, 64, 1, 8, 64, _lib.FG_PLAN_CLUSTER) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_plan_override(2, 64, 64, 4, 8, 64, 4) == _lib.FG_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("N1,N2", [(256, 256), (128, 256), (20, 27), (100, 64), (9, 100)])
@pytest.mark.parametrize("C,maps,mode", [(1, 1, 0), (1, 1, 1), (1, 2, 2), (3, 1, 1), (3, 1, 0)])
@pytest.mark.parametrize("wt", [False, True])
@pytest.mark.parametrize("rpt,flag", [(2, 4)])
def test_cluster_sweep_plans(N1, N2, C, maps, mode, wt, rpt, flag):
    L = _lib.load()
    G = 16
    _lib.check(L.fg_plan_override(2, N1, N2, 8, -(-N1 // G), N2, _lib.FG_PLAN_CLUSTER | flag))
    try:
        p = _lib.plan_describe(2, N1, N2, C, maps, mode, wt)
    finally:
        _lib.check(L.fg_plan_override(2, N1, N2, 0, 0, 0, 0))
    cimg = 0 if mode == 1 else C
    T1 = -(-(-(-N1 // G)) // rpt) * rpt
    g = -(-N1 // T1)
    threads = T1 // rpt * -(-N2 // 4)
    nt = -(-threads // 32) * 32
    fits = cluster_smem(cimg, maps, T1, N2, nt, rpt, 2) <= 227 * 1024 - 1024
    if cimg > 1 or g < 2 or threads > 512 or not fits:
        assert not p["lean"] & _lib.FG_PLAN_RUNS2  # the planner's own plan
        return
    assert p["lean"] == _lib.FG_PLAN_CLUSTER | flag
    assert (p["tiles1"], p["tiles2"], p["T1"], p["T2"], p["K1"], p["K2"]) == (g, 1, T1, N2, 0, 0)
    assert threads <= p["threads"] <= 512 and p["threads"] % 32 == 0
    assert p["smem"] <= SMEM_LIMIT and p["depth"] in (2, 4, 8)
    # the layout-changing passes of a cluster plan write in place (a transpose follows): no flush rings
    assert p["smem"] == cluster_smem(cimg, maps, T1, N2, p["threads"], rpt, p["depth"])


def test_runs_flags_validation():
    L = _lib.load()
    assert L.fg_plan_override(2, 64, 64, 8, 8, 64, _lib.FG_PLAN_RUNS2) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_plan_override(2, 64, 64, 8, 8, 64, _lib.FG_PLAN_CLUSTER | 8) == _lib.FG_ERR_INVALID_ARGUMENT


def test_cluster_capacity_arguments():
    import ctypes
    L = _lib.load()
    n = ctypes.c_int()
    assert L.fg_cluster_capacity(0, 512, 1024, ctypes.byref(n)) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_cluster_capacity(17, 512, 1024, ctypes.byref(n)) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_cluster_capacity(16, 1024, 1024, ctypes.byref(n)) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_cluster_capacity(16, 512, 1024, None) == _lib.FG_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("cross,N1,N2,C,maps,mode", [(2, 1024, 1024, 1, 1, 0), (2, 800, 900, 1, 2, 2),
                                                     (2, 2048, 2048, 3, 1, 0), (2, 1024, 1024, 9, 1, 0),
                                                     (1, 1, 800000, 1, 1, 0)])
def test_chunked_plan_for_sections_beyond_the_resident_tiles(cross, N1, N2, C, maps, mode):
    """A cross-section whose tiles cannot all be resident gets a chunked plan
    (one ordinary launch per chunk of S steps): more tiles than SMs, each
    region within the kernel's limits, halos of S."""
    p = _lib.plan_describe(cross, N1, N2, C=C, maps=maps, mode=mode)
    assert p["lean"] & _lib.FG_PLAN_CHUNKED and not p["lean"] & _lib.FG_PLAN_CLUSTER
    t1, t2 = -(-N1 // p["T1"]), -(-N2 // p["T2"])
    assert (t1, t2) == (p["tiles1"], p["tiles2"]) and t1 * t2 > 152
    assert p["K2"] == p["S"] and p["K1"] == (p["S"] if cross == 2 and t1 > 1 else 0)
    R1 = p["T1"] + 2 * p["K1"] if cross == 2 else 1
    assert R1 * (p["T2"] + 2 * p["K2"]) <= 4096 and p["smem"] <= 227 * 1024
    assert p["T2"] % 4 == 0 and p["T1"] >= p["K1"] and p["T2"] >= p["K2"]


def test_sections_that_fit_keep_cooperative_plans():
    for key in [(2, 256, 256), (2, 512, 512), (2, 128, 1024), (1, 1, 4096)]:
        assert not _lib.plan_describe(*key)["lean"] & _lib.FG_PLAN_CHUNKED, key


def test_chunked_override():
    L = _lib.load()
    CH = _lib.FG_PLAN_CHUNKED
    assert L.fg_plan_override(2, 64, 64, 4, 16, 16, CH | _lib.FG_PLAN_CLUSTER) == _lib.FG_ERR_INVALID_ARGUMENT
    try:
        _lib.check(L.fg_plan_override(2, 64, 64, 4, 16, 16, CH))
        p = _lib.plan_describe(2, 64, 64)
        assert p["lean"] & CH and (p["T1"], p["T2"], p["tiles1"], p["tiles2"]) == (16, 16, 4, 4)
        # a chunked override may use more tiles than the SMs
        _lib.check(L.fg_plan_override(2, 64, 64, 2, 4, 4, CH))
        p = _lib.plan_describe(2, 64, 64, sms=8)
        assert p["lean"] & CH and p["tiles1"] * p["tiles2"] == 256
    finally:
        _lib.check(L.fg_plan_override(2, 64, 64, 0, 0, 0, 0))
    assert not _lib.plan_describe(2, 64, 64)["lean"] & CH


@pytest.mark.parametrize("N2,T2", [(33, 32), (40, 32), (64, 32), (100, 32), (128, 32), (300, 32), (512, 32), (513, 64),
                                   (600, 64), (1024, 64), (1025, 32),
                                   (4864, 32), (4865, 64), (8192, 64), (9729, 128), (19456, 128)])
def test_long_rows_take_row_tiles_with_32_step_chunks(N2, T2):
    """2D rows of more than 32 cells: row tiles (one thread per cell of a
    tile and its halos), a hand-off every 32 steps (the measured optimum).
    Rows up to 1024 cells: one thread-block cluster of at most 16 tiles (32
    cells up to 512, else 64); longer rows: the narrowest of 32, 64, 128
    cells that fits the SMs, handing over through global memory."""
    p = _lib.plan_describe(1, 1, N2)
    assert (p["S"], p["T1"], p["T2"], p["K2"]) == (32, 1, T2, 32)
    assert p["tiles2"] == -(-N2 // T2) <= 152 and p["threads"] == T2 + 64
    clu = _lib.FG_PLAN_CLUSTER if N2 <= 1024 else 0
    assert p["lean"] == _lib.FG_PLAN_ROWS | clu and (not clu or p["tiles2"] <= 16)
    # more than 4 channels take the pass kernel on 128-cell tiles
    q = _lib.plan_describe(1, 1, N2, C=6)
    assert not q["lean"] & _lib.FG_PLAN_ROWS and q["T2"] in (128, T2) or q["S"] <= 8
    # rows wider than 152 tiles of 128 keep the cost model's plan
    assert _lib.plan_describe(1, 1, 19457)["S"] <= 8


@pytest.mark.parametrize("N2", [1, 2, 5, 17, 32])
def test_short_rows_take_one_row_tile(N2):
    """Rows of up to 32 cells: one row tile of the whole row, one warp, no
    halos and no hand-off (images of 1 to 4 channels)."""
    for C, maps in ((1, 1), (4, 2)):
        p = _lib.plan_describe(1, 1, N2, C=C, maps=maps)
        assert p["lean"] == _lib.FG_PLAN_ROWS and (p["T2"], p["K2"], p["tiles2"], p["threads"]) == (N2, 0, 1, 32)
    assert not _lib.plan_describe(1, 1, N2, C=5)["lean"] & _lib.FG_PLAN_ROWS


def test_one_launch_rule():
    """The per-call path's one-CTA launch: fewer than 16384 cells, sides up
    to 512."""
    assert _lib.FG_ONE_LAUNCH_SIDE == 512
    assert _lib.FG_ONE_LAUNCH_CELLS == 16384
    assert _lib.runs_in_one_launch((64, 96)) and _lib.runs_in_one_launch((512, 31))
    assert _lib.runs_in_one_launch((1, 5)) and _lib.runs_in_one_launch((127, 128))
    for shape in [(128, 128), (512, 512), (127, 513), (256, 300), (64, 512), (20, 600)]:
        assert not _lib.runs_in_one_launch(shape), shape
    header = open(os.path.join(os.path.dirname(__file__), "..", "include", "fastgeodis_gb300.h")).read()
    for name in ("FG_ONE_LAUNCH_SIDE", "FG_ONE_LAUNCH_CELLS"):
        assert re.search(rf"#define {name} (\d+)", header).group(1) == str(getattr(_lib, name))


def test_row_tile_override_validation():
    L = _lib.load()
    ROWS = _lib.FG_PLAN_ROWS
    assert L.fg_plan_override(2, 64, 64, 8, 8, 8, ROWS) == _lib.FG_ERR_INVALID_ARGUMENT  # 2D only
    assert L.fg_plan_override(1, 1, 300, 8, 1, 64, ROWS | _lib.FG_PLAN_CHUNKED) == _lib.FG_ERR_INVALID_ARGUMENT
    try:
        _lib.check(L.fg_plan_override(1, 1, 300, 8, 1, 64, ROWS))
        p = _lib.plan_describe(1, 1, 300)
        assert p["lean"] == ROWS and (p["S"], p["T2"], p["tiles2"], p["threads"]) == (8, 64, 5, 96)
        # one tile of the whole row: no halos and no hand-off
        _lib.check(L.fg_plan_override(1, 1, 300, 8, 1, 496, ROWS))
        p = _lib.plan_describe(1, 1, 300)
        assert p["lean"] == ROWS and (p["T2"], p["K2"], p["tiles2"], p["threads"]) == (300, 0, 1, 320)
        # a region beyond 512 cells stays on the pass kernel
        _lib.check(L.fg_plan_override(1, 1, 600, 8, 1, 600, ROWS))
        assert not _lib.plan_describe(1, 1, 600)["lean"] & ROWS
    finally:
        _lib.check(L.fg_plan_override(1, 1, 300, 0, 0, 0, 0))
        _lib.check(L.fg_plan_override(1, 1, 600, 0, 0, 0, 0))


@pytest.mark.parametrize("N2,S,T2,clu", [(512, 32, 32, True), (211, 4, 20, True), (1024, 32, 64, True),
                                         (1024, 32, 32, False), (492, 32, 32, True), (300, 8, 16, False),
                                         (300, 8, 300, False)])
def test_cluster_row_tile_overrides(N2, S, T2, clu):
    """FG_PLAN_ROWS | FG_PLAN_CLUSTER: row tiles as one thread-block cluster
    when there are 2 to 16 tiles with halos no wider than a tile; otherwise
    the same row tiles with the hand-off through global memory (or the
    planner's plan for one tile).  The cluster form adds its receive rows and
    two mbarriers to the shared memory."""
    L = _lib.load()
    ROWS, CLU = _lib.FG_PLAN_ROWS, _lib.FG_PLAN_CLUSTER
    try:
        for maps, wt in ((1, False), (2, True)):
            _lib.check(L.fg_plan_override(1, 1, N2, S, 1, T2, ROWS | CLU))
            p = _lib.plan_describe(1, 1, N2, maps=maps, transposed_write=wt)
            _lib.check(L.fg_plan_override(1, 1, N2, S, 1, T2, ROWS))
            q = _lib.plan_describe(1, 1, N2, maps=maps, transposed_write=wt)
            if T2 >= N2:  # one tile of the whole row: no halos, no cluster
                assert p["lean"] == q["lean"] == ROWS and p["tiles2"] == 1 and p["K2"] == 0
                continue
            assert p["lean"] == (ROWS | CLU if clu else ROWS) and q["lean"] == ROWS
            assert (p["tiles2"], p["threads"]) == (q["tiles2"], q["threads"])
            assert p["smem"] - q["smem"] == ((4 * maps * S + 4) * 4 if clu else 0)
            if clu:
                assert 2 <= p["tiles2"] <= 16 and S <= T2
    finally:
        _lib.check(L.fg_plan_override(1, 1, N2, 0, 0, 0, 0))
    # no runs per thread or chunks with row tiles; a cluster flag alone stays a volume plan
    assert L.fg_plan_override(1, 1, 300, 8, 1, 64, ROWS | CLU | _lib.FG_PLAN_RUNS2) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_plan_override(1, 1, 300, 8, 1, 64, ROWS | CLU | _lib.FG_PLAN_CHUNKED) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_plan_override(1, 1, 300, 8, 1, 64, CLU) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_plan_override(2, 64, 64, 8, 8, 8, ROWS | CLU) == _lib.FG_ERR_INVALID_ARGUMENT
