"""CPU tests of the drop-in boundary: argument validation with the
reference's exception types (FastGeodis/common.h, FastGeodis/fastgeodis.cpp),
and the C ABI library (loads, exports every declared symbol, argument
errors) -- no kernel is launched here."""
import ctypes
import os
import re

import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            names |= set(re.findall(r"FG_API\s+[\w\s\*]*?\b(fg_\w+)\s*\(", open(os.path.join(inc, f)).read()))
    return names


def test_header_declares_the_exported_list():
    assert declared_symbols() == set(_lib.EXPORTED)


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    for name in declared_symbols():
        assert hasattr(L, name), name
    assert L.fg_abi_version() == 1


def test_workspace_sizes():
    L = _lib.load()
    P = 7 * 9 * 11
    plain = L.fg_workspace_bytes(_lib.FG_OP_PLAIN, 1, 7, 9, 11)
    signed = L.fg_workspace_bytes(_lib.FG_OP_SIGNED, 1, 7, 9, 11)
    gsf = L.fg_workspace_bytes(_lib.FG_OP_GSF, 1, 7, 9, 11)
    assert 0 < plain < signed < gsf
    assert signed - plain >= P * 4 and gsf - plain >= 4 * P * 4
    assert L.fg_workspace_bytes(9, 1, 1, 1, 1) == 0


def test_c_abi_argument_errors_without_launch():
    L = _lib.load()
    buf = (ctypes.c_float * 64)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    # null workspace
    rc = L.fg_generalised_geodesic2d(p, 1, 4, 4, p, 1, p, 1.0, 1.0, 0.0, 1, None, 0, None)
    assert rc == _lib.FG_ERR_WORKSPACE and "workspace" in _lib.last_error()
    # bad channel count
    rc = L.fg_generalised_geodesic2d(p, 0, 4, 4, p, 1, p, 1.0, 1.0, 0.0, 1, None, 0, None)
    assert rc == _lib.FG_ERR_INVALID_ARGUMENT
    # null spacing
    rc = L.fg_generalised_geodesic3d(p, 1, 2, 2, 2, p, 1, None, p, 1.0, 1.0, 0.0, 1, None, 0, None)
    assert rc == _lib.FG_ERR_INVALID_ARGUMENT
    # too-small workspace (unaligned sizes are refused before any CUDA call)
    rc = L.fg_signed_generalised_geodesic2d(p, 1, 4, 4, p, 1, p, 1.0, 1.0, 0.0, 1, p, 16, None)
    assert rc == _lib.FG_ERR_WORKSPACE
    assert L.fg_set_tuning(-1, 0) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_set_tuning(0, 0) == _lib.FG_OK
    with pytest.raises(ValueError):
        _lib.check(_lib.FG_ERR_INVALID_ARGUMENT)
    with pytest.raises(RuntimeError):
        _lib.check(_lib.FG_ERR_TIMEOUT)


FUNCS2D = [
    lambda i, m: fg.generalised_geodesic2d(i, m, 1e10, 1.0, 2),
    lambda i, m: fg.signed_generalised_geodesic2d(i, m, 1e10, 1.0, 2),
    lambda i, m: fg.GSF2d(i, m, 0.0, 1e10, 1.0, 2),
]
FUNCS3D = [
    lambda i, m, sp=[1.0, 1.0, 1.0]: fg.generalised_geodesic3d(i, m, sp, 1e10, 1.0, 2),
    lambda i, m, sp=[1.0, 1.0, 1.0]: fg.signed_generalised_geodesic3d(i, m, sp, 1e10, 1.0, 2),
    lambda i, m, sp=[1.0, 1.0, 1.0]: fg.GSF3d(i, m, 0.0, sp, 1e10, 1.0, 2),
]


@pytest.mark.parametrize("f", FUNCS2D)
@pytest.mark.parametrize("base", [16, 32, 64])
def test_ill_shape_2d(f, base):
    # reference tests/test_fastgeodis.py:48-91
    good = [1, 1, base, base]
    with pytest.raises(ValueError):
        f(torch.rand(good), torch.rand([2, 1, base, base]))
    with pytest.raises(ValueError):
        f(torch.rand([2, 1, base, base]), torch.rand([2, 1, base, base]))
    with pytest.raises(ValueError):
        f(torch.rand([1, 1, base, 12]), torch.rand(good))
    with pytest.raises(ValueError):
        f(torch.rand(good + [16]), torch.rand(good + [16]))


@pytest.mark.parametrize("f", FUNCS3D)
@pytest.mark.parametrize("base", [16, 32])
def test_ill_shape_3d(f, base):
    good = [1, 1, base, base, base]
    with pytest.raises(ValueError):
        f(torch.rand(good), torch.rand([2, 1, base, base, base]))
    with pytest.raises(ValueError):
        f(torch.rand([1, 1, base, base, 12]), torch.rand(good))
    with pytest.raises(ValueError):
        f(torch.rand([1, 1, base, base]), torch.rand([1, 1, base, base]))


@pytest.mark.parametrize("f", FUNCS3D)
def test_ill_spacing(f):
    # reference tests/test_fastgeodis.py:214-230
    z = torch.zeros([1, 1, 16, 16, 16])
    with pytest.raises(ValueError):
        f(z, z, [1.0, 1.0])


def test_dtype_is_runtime_error():
    with pytest.raises(RuntimeError):
        fg.generalised_geodesic2d(torch.rand([1, 1, 8, 8], dtype=torch.float64), torch.rand([1, 1, 8, 8]), 1e10, 1.0)


def test_messages_match_reference():
    with pytest.raises(ValueError, match="single batch"):
        fg.generalised_geodesic2d(torch.rand([2, 1, 8, 8]), torch.rand([2, 1, 8, 8]), 1e10, 1.0)
    with pytest.raises(ValueError, match="shapes of input tensors do not match"):
        fg.generalised_geodesic2d(torch.rand([1, 1, 8, 8]), torch.rand([1, 1, 8, 9]), 1e10, 1.0)
    with pytest.raises(ValueError, match="3D spacing"):
        fg.generalised_geodesic3d(torch.rand([1, 1, 4, 4, 4]), torch.rand([1, 1, 4, 4, 4]), [1.0], 1e10, 1.0)


def test_defaults_match_reference_signatures():
    import inspect

    assert inspect.signature(fg.generalised_geodesic2d).parameters["iter"].default == 2
    assert inspect.signature(fg.generalised_geodesic3d).parameters["iter"].default == 4
    assert inspect.signature(fg.signed_generalised_geodesic2d).parameters["iter"].default == 2
    assert inspect.signature(fg.signed_generalised_geodesic3d).parameters["iter"].default == 4
    assert list(inspect.signature(fg.GSF3d).parameters) == ["image", "softmask", "theta", "spacing", "v", "lamb", "iter"]


def test_tiled_batch_arguments_without_launch():
    """The tiled batch entry refuses bad arguments before any CUDA call."""
    L = _lib.load()
    buf = (ctypes.c_float * 64)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    tiles = (ctypes.c_int * 2)(4, 6)
    need = L.fg_batch2d_tiled_scratch_bytes(2, 1000)
    assert need >= 2 * 4 * 1000 * 8  # exchange words: 2 parities x 2 maps per cell of the longest side
    assert L.fg_batch2d_tiled_scratch_bytes(-1, 10) == 0 and L.fg_batch2d_tiled_scratch_bytes(1, 0) == 0
    assert L.fg_batch_geodesic2d_tiled(p, tiles, 0, 1, 100, 2, p, need, p, None) == _lib.FG_OK  # nothing to do
    assert L.fg_batch_geodesic2d_tiled(p, tiles, 33, 1, 100, 2, p, need, p, None) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_batch_geodesic2d_tiled(p, tiles, 2, 1, 100, 2, None, need, p, None) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_batch_geodesic2d_tiled(p, tiles, 2, 5, 100, 2, p, need, p, None) == _lib.FG_ERR_UNSUPPORTED
    assert L.fg_batch_geodesic2d_tiled(p, tiles, 2, 1, 4096, 2, p, need, p, None) == _lib.FG_ERR_UNSUPPORTED
    assert L.fg_batch_geodesic2d_tiled(p, tiles, 2, 1, 1000, 2, p, need - 8, p, None) == _lib.FG_ERR_WORKSPACE
    bad = (ctypes.c_int * 2)(4, 1)
    assert L.fg_batch_geodesic2d_tiled(p, bad, 2, 1, 1000, 2, p, need, p, None) == _lib.FG_ERR_INVALID_ARGUMENT


def test_header_constants_match_the_binding():
    """Every integer constant of the C header that the Python binding also
    names (status codes, operations, plan flags, one-launch limits, batch
    flags) has the same value on both sides."""
    header = open(os.path.join(ROOT, "include", "fastgeodis_gb300.h")).read()
    defines = {name: int(val, 0) for name, val in re.findall(r"#define (FG_\w+) (0x[0-9a-fA-F]+|\d+)\b", header)}
    named = {n: v for n, v in defines.items() if hasattr(_lib, n)}
    assert {"FG_OK", "FG_ERR_TIMEOUT", "FG_OP_GSF", "FG_PLAN_ROWS", "FG_PLAN_CHUNKED", "FG_ONE_LAUNCH_CELLS"} <= set(named)
    for name, value in named.items():
        assert getattr(_lib, name) == value, name
    for name in defines:  # every status code, operation and plan flag is bound
        if name.startswith(("FG_ERR_", "FG_OP_", "FG_PLAN_")) and name != "FG_PLAN_MODE_MASK":
            assert hasattr(_lib, name), name
    for m in range(3):
        assert _lib.FG_PLAN_MODE(m) == (m + 1) << 4


def test_batch_flags_match_the_header():
    from fastgeodis_gb300 import batch, batch3d

    header = open(os.path.join(ROOT, "include", "fastgeodis_gb300.h")).read()
    defines = dict((n, int(v)) for n, v in re.findall(r"#define (FG_BATCH_\w+) (\d+)\b", header))
    assert defines == {"FG_BATCH_SIGNED": batch.FG_BATCH_SIGNED, "FG_BATCH_SPLIT": batch.FG_BATCH_SPLIT,
                       "FG_BATCH_SECOND": batch.FG_BATCH_SECOND}
    assert batch3d.FG_BATCH_SIGNED == defines["FG_BATCH_SIGNED"]
