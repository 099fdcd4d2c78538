"""Accuracy harness against fast marching (oracle/fastmarch.py): the speed
field restatement, the vendored solver on known answers (constant speed ->
Euclidean distance, isotropic and anisotropic), and the raster scan's
agreement with fast marching on a smoothed image, pinned."""
import numpy as np
import pytest

from golden_cases import load_all
from oracle import fastmarch, oracle

pytestmark = pytest.mark.skipif(not fastmarch.available(), reason="the vendored fast-marching header is not available")


def test_speed_field_matches_the_reference_formula():
    img = np.array([[[1, 2], [4, 8]]], np.float32)
    got = fastmarch.speed_field(img, 0.5, 0.5)
    # 0.5 * (|dx| + |dy|) with zero beyond the edge: 2, 4, 4, 8
    grad = np.array([[2.0, 4.0], [4.0, 8.0]], np.float32)
    want = np.float32(1) / (np.float32(0.5) * grad + np.float32(0.5) + fastmarch.FEPS)
    assert np.array_equal(got, want)
    vol = np.arange(8, dtype=np.float32).reshape(1, 2, 2, 2)  # 3D: (|dx| + |dy|) / 3, no z term
    g3 = (np.float32(1.0 / 3.0) * (fastmarch._fwd_diff_abs(vol, 3) + fastmarch._fwd_diff_abs(vol, 2)))[0]
    assert np.array_equal(fastmarch.speed_field(vol, 1.0, 0.0), np.float32(1) / (g3 + fastmarch.FEPS))


def test_constant_speed_gives_the_euclidean_distance():
    H, W = 64, 64
    img = np.zeros((1, H, W), np.float32)
    m = np.ones((1, H, W), np.float32)
    m[0, 20, 30] = 0
    t = fastmarch.fastmarch(img, m, 0.0)
    yy, xx = np.mgrid[:H, :W]
    e = np.sqrt((yy - 20.0) ** 2 + (xx - 30.0) ** 2)
    far = e > 5
    rel = np.abs(t - e)[far] / e[far]
    assert t[20, 30] == 0 and rel.max() < 0.06 and rel.mean() < 0.012


def test_constant_speed_anisotropic_volume():
    D, H, W = 12, 20, 24
    img = np.zeros((1, D, H, W), np.float32)
    m = np.ones((1, D, H, W), np.float32)
    m[0, 5, 9, 11] = 0
    sp = [2.0, 0.5, 1.0]
    t = fastmarch.fastmarch(img, m, 0.0, sp)
    zz, yy, xx = np.mgrid[:D, :H, :W]
    e = np.sqrt(((zz - 5) * 2.0) ** 2 + ((yy - 9) * 0.5) ** 2 + ((xx - 11) * 1.0) ** 2)
    far = e > 3
    assert (np.abs(t - e)[far] / e[far]).mean() < 0.07


def test_raster_scan_against_fast_marching_pinned():
    """The raster scan (the engine's bits: the oracle equals them) against fast
    marching on the reference's smoothed-noise golden input: the agreement
    figures of this harness, pinned (both computations are deterministic)."""
    c = {x["name"]: x for x in load_all()}["g2d_smooth"]
    img, m = c["image"], c["mask"]
    t = fastmarch.fastmarch(img, m, 0.5)
    d = oracle.geodesic2d(img, m, 1e10, 0.5, 2)[0]
    r = fastmarch.compare(d, t, m[0])
    assert r["cells"] == int((m[0] != 0).sum())
    # measured: Pearson 0.874, mean relative difference 0.157 (short paths
    # around five seed disks on a 96 x 80 image; longer ones agree better)
    assert r["pearson"] == pytest.approx(0.874, abs=0.01)
    assert r["mean_rel_diff"] == pytest.approx(0.157, abs=0.01)
    ref = fastmarch.compare(oracle.geodesic2d(img, m, 1e10, 0.0, 2)[0], fastmarch.fastmarch(img, m, 0.0), m[0])
    # lamb 0: the 3 x 3 raster scan's chamfer metric against Euclidean arrival (measured 0.083, 0.9984)
    assert ref["mean_rel_diff"] == pytest.approx(0.083, abs=0.005) and ref["pearson"] > 0.998
