"""GPU parity tests: the CUDA engine (through the drop-in API and its C ABI)
against the reference's golden vectors and against the C oracle, bit for bit.

Bit-exactness is the bar because both sides evaluate the same float32
operations in the same order; a tolerance of 1e-5 relative / 1e-4 absolute
is additionally asserted where the comparison is against the float64 scan."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib
from golden_cases import bits_equal, load_all, names
from oracle import oracle

pytestmark = pytest.mark.gpu

CASES = {c["name"]: c for c in load_all()}
DEV = "cuda"


def t(a):
    return torch.from_numpy(np.ascontiguousarray(a))[None].to(DEV)


def run_gpu(c):
    img, m, v, lamb, it = t(c["image"]), t(c["mask"]), c["v"], c["lamb"], c["iter"]
    op = c["op"]
    if op == "geodesic2d":
        r = fg.generalised_geodesic2d(img, m, v, lamb, it)
    elif op == "geodesic3d":
        r = fg.generalised_geodesic3d(img, m, c["spacing"], v, lamb, it)
    elif op == "signed2d":
        r = fg.signed_generalised_geodesic2d(img, m, v, lamb, it)
    elif op == "signed3d":
        r = fg.signed_generalised_geodesic3d(img, m, c["spacing"], v, lamb, it)
    elif op == "gsf2d":
        r = fg.GSF2d(img, m, c["theta"], v, lamb, it)
    elif op == "gsf3d":
        r = fg.GSF3d(img, m, c["theta"], c["spacing"], v, lamb, it)
    elif op == "toivanen2d":
        r = fg.generalised_geodesic2d_toivanen(img, m, v, lamb, it)
    elif op == "toivanen3d":
        r = fg.generalised_geodesic3d_toivanen(img, m, c["spacing"], v, lamb, it)
    elif op == "signed_toivanen2d":
        r = fg.signed_generalised_geodesic2d_toivanen(img, m, v, lamb, it)
    elif op == "signed_toivanen3d":
        r = fg.signed_generalised_geodesic3d_toivanen(img, m, c["spacing"], v, lamb, it)
    elif op == "gsf_toivanen2d":
        r = fg.GSF2d_toivanen(img, m, c["theta"], v, lamb, it)
    else:
        r = fg.GSF3d_toivanen(img, m, c["theta"], c["spacing"], v, lamb, it)
    return r[0].cpu().numpy()


@pytest.fixture
def tuning():
    L = _lib.load()
    yield lambda region, tiles=0: _lib.check(L.fg_set_tuning(region, tiles))
    _lib.check(L.fg_set_tuning(0, 0))


@pytest.mark.parametrize("name", names())
def test_golden_bits(name):
    c = CASES[name]
    got = run_gpu(c)
    assert bits_equal(got, c["expected"]), f"{name}: max abs diff {np.abs(got - c['expected']).max()}"
    fg.check_status()


@pytest.mark.parametrize("region", [24, 40, 64])
@pytest.mark.parametrize("name", ["g2d_c1_l0.37_i2", "g2d_c3", "g2d_smooth", "s2d_smooth", "gsf2d_smooth",
                                  "g3d_cube", "g3d_c2", "gsf3d_cube"])
def test_golden_bits_multi_tile(name, region, tuning):
    """Small per-CTA regions force many tiles, halos and flag hand-offs."""
    tuning(region)
    c = CASES[name]
    got = run_gpu(c)
    assert bits_equal(got, c["expected"]), f"{name}: max abs diff {np.abs(got - c['expected']).max()}"
    fg.check_status()


def rand_case(rng, shape, C, nseeds=3):
    img = (rng.random((C,) + shape) * 255).astype(np.float32)
    m = np.ones((1,) + shape, np.float32)
    for _ in range(nseeds):
        m[(0,) + tuple(rng.integers(0, n) for n in shape)] = 0
    return img, m


SHAPES2D = [(1, 1), (1, 70), (70, 1), (2, 3), (17, 31), (64, 64), (33, 130), (130, 33), (257, 511), (512, 512)]


@pytest.mark.parametrize("shape", SHAPES2D)
@pytest.mark.parametrize("C", [1, 3])
def test_2d_vs_oracle(shape, C):
    rng = np.random.default_rng(hash((shape, C)) % 2**32)
    img, m = rand_case(rng, shape, C)
    for lamb, it in [(0.0, 1), (0.6, 2), (1.0, 2)]:
        got = fg.generalised_geodesic2d(t(img), t(m), 1e10, lamb, it)[0].cpu().numpy()
        want = oracle.geodesic2d(img, m, 1e10, lamb, it)
        assert bits_equal(got, want), (shape, C, lamb, it, np.abs(got - want).max())


@pytest.mark.parametrize("shape", [(1, 5), (31, 33), (96, 150), (512, 30), (31, 512), (127, 128)])
@pytest.mark.parametrize("C", [1, 2, 3, 4])
def test_one_launch_forms_vs_oracle(shape, C):
    """Images of fewer than 16384 cells, up to 512 per side, run in one launch
    (one thread per cell of a row), compiled per channel count and lamb form
    (0: no image term, 1: no spatial term, else general): plain and signed
    against the oracle."""
    assert _lib.runs_in_one_launch(shape)
    rng = np.random.default_rng(hash((shape, C, "one")) % 2**32)
    img, m = rand_case(rng, shape, C)
    for lamb in (0.0, 1.0, 0.37):
        got = fg.generalised_geodesic2d(t(img), t(m), 1e10, lamb, 2)[0].cpu().numpy()
        assert bits_equal(got, oracle.geodesic2d(img, m, 1e10, lamb, 2)), (shape, C, lamb)
        got = fg.signed_generalised_geodesic2d(t(img), t(m), 1e10, lamb, 2)[0].cpu().numpy()
        assert bits_equal(got, oracle.signed2d(img, m, 1e10, lamb, 2)), (shape, C, lamb, "signed")


@pytest.mark.parametrize("shape", [(300, 257), (64, 2000), (2048, 96)])
@pytest.mark.parametrize("region", [40, 200])
def test_2d_vs_oracle_multi_tile(shape, region, tuning):
    tuning(region)
    rng = np.random.default_rng(7)
    img, m = rand_case(rng, shape, 1, nseeds=5)
    got = fg.generalised_geodesic2d(t(img), t(m), 1e10, 0.75, 2)[0].cpu().numpy()
    want = oracle.geodesic2d(img, m, 1e10, 0.75, 2)
    assert bits_equal(got, want), np.abs(got - want).max()
    fg.check_status()


SHAPES3D = [(1, 1, 1), (1, 9, 13), (9, 1, 13), (9, 13, 1), (5, 6, 7), (16, 16, 16), (33, 20, 47), (40, 64, 36)]


@pytest.mark.parametrize("shape", SHAPES3D)
@pytest.mark.parametrize("C", [1, 2])
def test_3d_vs_oracle(shape, C):
    rng = np.random.default_rng(hash((shape, C, 3)) % 2**32)
    img = rng.random((C,) + shape).astype(np.float32)
    m = np.ones((1,) + shape, np.float32)
    m[(0,) + tuple(n // 2 for n in shape)] = 0
    for sp, lamb, it in [([1.0, 1.0, 1.0], 0.0, 1), ([2.0, 0.5, 0.7], 0.5, 2), ([0.6, 1.3, 2.2], 1.0, 3)]:
        got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, it)[0].cpu().numpy()
        want = oracle.geodesic3d(img, m, sp, 1e10, lamb, it)
        assert bits_equal(got, want), (shape, C, sp, lamb, it, np.abs(got - want).max())
    fg.check_status()


def test_signed_and_gsf_vs_oracle():
    rng = np.random.default_rng(11)
    img, m = rand_case(rng, (150, 170), 2, nseeds=4)
    m[0, 40:70, 50:90] = 0
    got = fg.signed_generalised_geodesic2d(t(img), t(m), 1e10, 0.7, 2)[0].cpu().numpy()
    want = oracle.signed2d(img, m, 1e10, 0.7, 2)
    assert bits_equal(got, want)
    assert np.array_equal(np.signbit(got), np.signbit(want))
    got = fg.GSF2d(t(img), t(m), 20.0, 1e10, 0.9, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.gsf2d(img, m, 20.0, 1e10, 0.9, 2))
    vol = rng.random((1, 20, 30, 26)).astype(np.float32)
    vm = np.ones((1, 20, 30, 26), np.float32)
    vm[0, 5:12, 8:15, 6:20] = 0
    sp = [1.5, 0.8, 0.8]
    got = fg.signed_generalised_geodesic3d(t(vol), t(vm), sp, 1e10, 0.5, 3)[0].cpu().numpy()
    assert bits_equal(got, oracle.signed3d(vol, vm, sp, 1e10, 0.5, 3))
    got = fg.GSF3d(t(vol), t(vm), 0.5, sp, 1e10, 0.5, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.gsf3d(vol, vm, 0.5, sp, 1e10, 0.5, 2))
    fg.check_status()


@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("base", [16, 32, 64])
def test_known_answers(dims, base):
    """Reference tests/test_fastgeodis.py:116-210, 326-371 on the GPU."""
    import math

    shape = [1, 1] + [base] * dims
    z = torch.zeros(shape, device=DEV)
    o = torch.ones(shape, device=DEV)
    if dims == 2:
        f = lambda i, m, l: fg.generalised_geodesic2d(i, m, 1e10, l, 2)  # noqa: E731
        s = lambda i, m, l: fg.signed_generalised_geodesic2d(i, m, 1e10, l, 2)  # noqa: E731
    else:
        f = lambda i, m, l: fg.generalised_geodesic3d(i, m, [1.0] * 3, 1e10, l, 2)  # noqa: E731
        s = lambda i, m, l: fg.signed_generalised_geodesic3d(i, m, [1.0] * 3, 1e10, l, 2)  # noqa: E731
    assert torch.all(f(z, z, 1.0) == 0)
    assert torch.all(f(z, o, 1.0) == 1e10)
    assert torch.all(s(z, z, 1.0) == -1e10)
    assert torch.all(s(z, o, 1.0) == 1e10)
    m = o.clone()
    m.view(-1)[0] = 0
    d = f(o, m, 0.0)
    exp = math.sqrt(dims * base ** 2)
    tol = 10 if dims == 2 else 100
    assert exp - tol < float(d.max()) < exp + tol
    # GSF runs (reference :416-436 is a smoke test)
    if dims == 2:
        fg.GSF2d(o, m, 0.0, 1e10, 1.0, 2)
    else:
        fg.GSF3d(o, m, 0.0, [1.0] * 3, 1e10, 1.0, 2)


def test_device_mismatch_and_batch_on_cuda():
    # reference tests/test_fastgeodis.py:233-252
    for dims in (2, 3):
        img = torch.rand([1, 1] + [16] * dims, device=DEV)
        with pytest.raises(ValueError):
            if dims == 2:
                fg.generalised_geodesic2d(img, torch.rand([2, 1] + [16] * dims, device=DEV), 1e10, 1.0, 2)
            else:
                fg.generalised_geodesic3d(img, torch.rand([2, 1] + [16] * dims, device=DEV), [1.0] * 3, 1e10, 1.0, 2)
        with pytest.raises(ValueError):
            fg.generalised_geodesic2d(torch.rand(1, 1, 8, 8, device=DEV), torch.rand(1, 1, 8, 8), 1e10, 1.0)


def test_host_tensors_roundtrip():
    rng = np.random.default_rng(3)
    img, m = rand_case(rng, (90, 77), 1)
    got = fg.generalised_geodesic2d(torch.from_numpy(img)[None], torch.from_numpy(m)[None], 1e10, 0.5, 2)
    assert got.device.type == "cpu"
    assert bits_equal(got[0].numpy(), oracle.geodesic2d(img, m, 1e10, 0.5, 2))


def test_multichannel_mask_unswept_channels():
    c = CASES["g2d_softmask_cm2"]
    assert bits_equal(run_gpu(c), c["expected"])
    rng = np.random.default_rng(5)
    img = rng.random((1, 30, 40)).astype(np.float32)
    m = rng.random((3, 30, 40)).astype(np.float32)
    got = fg.GSF2d(t(img), t(m), 0.2, 2.0, 0.5, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.gsf2d(img, m, 0.2, 2.0, 0.5, 2))
    got = fg.signed_generalised_geodesic2d(t(img), t(m), 2.0, 0.5, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.signed2d(img, m, 2.0, 0.5, 2))


def test_determinism_repeated_runs():
    rng = np.random.default_rng(9)
    vol = rng.random((1, 48, 64, 80)).astype(np.float32)
    vm = np.ones((1, 48, 64, 80), np.float32)
    vm[0, 20, 30, 40] = 0
    outs = [fg.generalised_geodesic3d(t(vol), t(vm), [1.0, 1.0, 1.0], 1e10, 0.5, 2) for _ in range(5)]
    for o in outs[1:]:
        assert torch.equal(o.view(torch.int32), outs[0].view(torch.int32))
    fg.check_status()


def test_inputs_not_modified_and_zero_iterations():
    img = torch.rand(1, 1, 20, 30, device=DEV)
    m = torch.rand(1, 1, 20, 30, device=DEV)
    i0, m0 = img.clone(), m.clone()
    d = fg.generalised_geodesic2d(img, m, 3.0, 0.5, 0)
    assert torch.equal(d, 3.0 * m0)
    fg.generalised_geodesic2d(img, m, 3.0, 0.5, 2)
    assert torch.equal(img, i0) and torch.equal(m, m0)
    e = fg.generalised_geodesic2d(torch.rand(1, 1, 0, 5, device=DEV), torch.rand(1, 1, 0, 5, device=DEV), 1.0, 0.5)
    assert e.shape == (1, 1, 0, 5)


def test_float64_error_report_2d():
    """The float32 scan stays within 1e-5 relative / 1e-4 absolute of the
    same scan in float64 (the tolerance of the parity contract)."""
    rng = np.random.default_rng(21)
    from scipy.ndimage import gaussian_filter

    img = gaussian_filter(rng.uniform(0, 255, (256, 256)).astype(np.float32), 3)[None].astype(np.float32)
    m = np.ones((1, 256, 256), np.float32)
    m[0, 100:104, 50:54] = 0
    got = fg.generalised_geodesic2d(t(img), t(m), 1e10, 1.0, 2)[0].cpu().numpy().astype(np.float64)
    ref64 = oracle.geodesic2d_f64(img, m, 1e10, 1.0, 2)
    np.testing.assert_allclose(got, ref64, rtol=1e-5, atol=1e-4)


def test_small_images_run_in_one_launch_unless_plans_are_pinned():
    L = _lib.load()
    rng = np.random.default_rng(21)
    img = rng.random((1, 64, 96)).astype(np.float32)
    m = np.ones((1, 64, 96), np.float32)
    m[0, 10, 20] = 0
    ti, tm = t(img), t(m)
    want = oracle.geodesic2d(img, m, 1e10, 0.5, 2)

    def launches(fn):
        torch.cuda.synchronize()
        _lib.profile_begin()
        out = fn()
        torch.cuda.synchronize()
        _, n, _ = _lib.profile_end()
        return n, out

    n, out = launches(lambda: fg.generalised_geodesic2d(ti, tm, 1e10, 0.5, 2))
    assert n == 1 and bits_equal(out[0].cpu().numpy(), want)  # the whole transform in one launch
    n, out = launches(lambda: fg.signed_generalised_geodesic2d(ti, tm, 1e10, 0.5, 2))
    assert n == 1
    _lib.check(L.fg_plan_override(1, 1, 96, 8, 1, 96, 0))  # a pinned plan: one launch per pass
    try:
        n, out = launches(lambda: fg.generalised_geodesic2d(ti, tm, 1e10, 0.5, 2))
        assert n == 8 and bits_equal(out[0].cpu().numpy(), want)
    finally:
        _lib.check(L.fg_plan_override(1, 1, 96, 0, 0, 0, 0))
    _lib.check(L.fg_set_tuning(64, 0))  # planner limits: one launch per pass too
    try:
        n, out = launches(lambda: fg.generalised_geodesic2d(ti, tm, 1e10, 0.5, 2))
        assert n == 8 and bits_equal(out[0].cpu().numpy(), want)
    finally:
        _lib.check(L.fg_set_tuning(0, 0))
    fg.check_status()


# More than four image channels: the wide pass variant (channels streamed from
# the shared rings, L1 summed in channel order), on the planner's tiles and on
# forced small regions (many tiles, halo hand-offs).
@pytest.mark.parametrize("C", [5, 8])
@pytest.mark.parametrize("region", [0, 48])
@pytest.mark.parametrize("shape", [(64, 77), (300, 257), (1, 40), (520, 9)])
def test_2d_wide_channels_vs_oracle(shape, C, region, tuning):
    if region:
        tuning(region)
    rng = np.random.default_rng(C * 1000 + shape[0] * 7 + shape[1] + region)
    img, m = rand_case(rng, shape, C)
    for lamb in (0.0, 0.45, 1.0):
        got = fg.generalised_geodesic2d(t(img), t(m), 1e10, lamb, 2)[0].cpu().numpy()
        want = oracle.geodesic2d(img, m, 1e10, lamb, 2)
        assert bits_equal(got, want), (shape, C, region, lamb, np.abs(got - want).max())
    got = fg.signed_generalised_geodesic2d(t(img), t(m), 1e10, 0.7, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.signed2d(img, m, 1e10, 0.7, 2)), (shape, C, region, "signed")
    fg.check_status()


@pytest.mark.parametrize("C", [5, 8])
@pytest.mark.parametrize("region", [0, 64])
@pytest.mark.parametrize("shape", [(9, 23, 31), (24, 40, 36), (1, 12, 17)])
def test_3d_wide_channels_vs_oracle(shape, C, region, tuning):
    if region:
        tuning(region)
    rng = np.random.default_rng(C * 1000 + sum(shape) + region)
    img = rng.random((C,) + shape).astype(np.float32)
    m = np.ones((1,) + shape, np.float32)
    m[(0,) + tuple(n // 2 for n in shape)] = 0
    sp = [1.3, 0.7, 0.9]
    for lamb in (0.0, 0.5, 1.0):
        got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, 2)[0].cpu().numpy()
        want = oracle.geodesic3d(img, m, sp, 1e10, lamb, 2)
        assert bits_equal(got, want), (shape, C, region, lamb, np.abs(got - want).max())
    got = fg.signed_generalised_geodesic3d(t(img), t(m), sp, 1e10, 0.3, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.signed3d(img, m, sp, 1e10, 0.3, 2)), (shape, C, region, "signed")
    got = fg.GSF3d(t(img), t(m), 0.5, sp, 1e10, 0.6, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.gsf3d(img, m, 0.5, sp, 1e10, 0.6, 1)), (shape, C, region, "gsf")
    fg.check_status()


@pytest.mark.parametrize("lamb", [-0.4, 1.5])
def test_lamb_outside_the_unit_interval(lamb):
    """The reference does not restrict lamb to [0, 1]: with a negative image
    weight (lamb < 0) the image term l_grad * |d| is negative, and with lamb
    > 1 the step-length term is.  Every sweep form gives the oracle's bits:
    the one-CTA launch, row tiles (clustered and through global memory),
    volume tile plans and the cluster sweep kernel."""
    from fastgeodis_gb300 import tune

    rng = np.random.default_rng(91)
    for shape, C in (((60, 70), 1), ((300, 400), 1), ((150, 1100), 3)):
        img, m = rand_case(rng, shape, C)
        got = fg.generalised_geodesic2d(t(img), t(m), 1e10, lamb, 2)[0].cpu().numpy()
        assert bits_equal(got, oracle.geodesic2d(img, m, 1e10, lamb, 2)), (shape, C)
        got = fg.signed_generalised_geodesic2d(t(img), t(m), 1e10, lamb, 1)[0].cpu().numpy()
        assert bits_equal(got, oracle.signed2d(img, m, 1e10, lamb, 1)), (shape, C, "signed")
    shape = (20, 48, 40)
    img, m = rand_case(rng, shape, 1)
    sp = [1.5, 0.8, 1.1]
    want = oracle.geodesic3d(img, m, sp, 1e10, lamb, 2)
    got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, 2)[0].cpu().numpy()
    assert bits_equal(got, want), "tile plans"
    try:
        tune.pin({k: (8, -(-k[1] // 4), k[2], _lib.FG_PLAN_CLUSTER | _lib.FG_PLAN_RUNS2) for k in tune.pass_keys(shape)})
        got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, 2)[0].cpu().numpy()
        assert bits_equal(got, want), "cluster plans"
    finally:
        tune.clear(shape)
    fg.check_status()


def test_gsf_side_stream_eager_threads_and_graph():
    """GSF runs the two signed transforms of its second stage at once, the
    second on a side stream of the calling thread: the oracle's bits from
    two host threads on their own streams, and from a CUDA graph (captured
    calls keep both on the captured stream)."""
    import threading

    rng = np.random.default_rng(77)
    cases = [rand_case(rng, (150, 300), 1), rand_case(rng, (12, 40, 36), 1)]
    wants = [oracle.gsf2d(*cases[0], 0.5, 1e10, 0.8, 2), oracle.gsf3d(*cases[1], 0.5, [1.2, 0.9, 1.0], 1e10, 0.8, 2)]
    outs = [None, None]

    def run(k):
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            img, m = (t(a) for a in cases[k])
            r = fg.GSF2d(img, m, 0.5, 1e10, 0.8, 2) if k == 0 else fg.GSF3d(img, m, 0.5, [1.2, 0.9, 1.0], 1e10, 0.8, 2)
            outs[k] = r[0].cpu().numpy()

    threads = [threading.Thread(target=run, args=(k,)) for k in range(2)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for k in range(2):
        assert bits_equal(outs[k], wants[k]), k
    img, m = (t(a) for a in cases[0])
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        fg.GSF2d(img, m, 0.5, 1e10, 0.8, 2)  # plans, attributes and workspace set up before capture
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        out = fg.GSF2d(img, m, 0.5, 1e10, 0.8, 2)
    g.replay()
    torch.cuda.synchronize()
    assert bits_equal(out[0].cpu().numpy(), wants[0])
    fg.check_status()
