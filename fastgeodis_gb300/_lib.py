"""ctypes binding of the engine's C ABI (``include/fastgeodis_gb300.h``).

The shared library ``fastgeodis_gb300/_fg.so`` is built in-tree by
``fastgeodis_gb300/_build.py`` (``__graft_entry__.build()`` runs it).  There
is no fallback: if the library is missing or does not load, every call raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_fg.so")

FG_OK = 0
FG_ERR_INVALID_ARGUMENT = 1
FG_ERR_CUDA = 2
FG_ERR_WORKSPACE = 3
FG_ERR_TIMEOUT = 4
FG_ERR_UNSUPPORTED = 5

FG_OP_PLAIN = 0
FG_OP_SIGNED = 1
FG_OP_GSF = 2

# every symbol include/fastgeodis_gb300.h declares
EXPORTED = (
    "fg_abi_version", "fg_last_error", "fg_set_tuning", "fg_plan_override", "fg_plan_describe",
    "fg_profile_begin", "fg_profile_end", "fg_profile_launch_times", "fg_profile_aux_launches",
    "fg_workspace_bytes", "fg_workspace_status", "fg_selftest_wait", "fg_cluster_capacity",
    "fg_generalised_geodesic2d", "fg_generalised_geodesic3d",
    "fg_signed_generalised_geodesic2d", "fg_signed_generalised_geodesic3d",
    "fg_GSF2d", "fg_GSF3d", "fg_batch2d_smem_bytes", "fg_batch_geodesic2d",
    "fg_batch2d_tiled_scratch_bytes", "fg_batch_geodesic2d_tiled",
    "fg_grad_geodesic2d_forward", "fg_grad_geodesic2d_backward",
    "fg_grad_geodesic2d_forward_pass", "fg_grad_geodesic2d_backward_pass",
    "fg_generalised_geodesic2d_noalloc", "fg_noalloc_status", "fg_click_mask",
    "fg_generalised_geodesic2d_toivanen", "fg_generalised_geodesic3d_toivanen",
    "fg_signed_generalised_geodesic2d_toivanen", "fg_signed_generalised_geodesic3d_toivanen",
    "fg_GSF2d_toivanen", "fg_GSF3d_toivanen",
    "fg_batch3d_job_bytes", "fg_batch3d_plan", "fg_batch3d_launch", "fg_batch3d_capacity",
)

_lib = None


class EngineError(RuntimeError):
    """A non-argument failure reported by the engine (CUDA error, timeout...)."""


def load():
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"fastgeodis_gb300 engine library not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python fastgeodis_gb300/_build.py`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i, f, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_size_t
    fp = ctypes.POINTER(ctypes.c_float)
    L.fg_abi_version.restype = i
    L.fg_last_error.restype = ctypes.c_char_p
    L.fg_workspace_bytes.argtypes = [i, i, i, i, i]
    L.fg_workspace_bytes.restype = sz
    L.fg_profile_begin.argtypes = []
    L.fg_profile_end.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_double)]
    L.fg_profile_launch_times.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int), i,
                                          ctypes.POINTER(ctypes.c_int)]
    L.fg_profile_aux_launches.argtypes = [ctypes.POINTER(ctypes.c_int)]
    L.fg_click_mask.argtypes = [vp, i, i, i, ctypes.POINTER(ctypes.c_int), i, i, vp]
    L.fg_set_tuning.argtypes = [i, i]
    L.fg_plan_override.argtypes = [i, i, i, i, i, i, i]
    L.fg_plan_describe.argtypes = [i, i, i, i, i, i, i, i, ctypes.POINTER(ctypes.c_int)]
    L.fg_plan_override.restype = i
    L.fg_set_tuning.restype = i
    L.fg_workspace_status.argtypes = [vp, vp]
    L.fg_selftest_wait.argtypes = [i, vp, sz, vp]
    L.fg_cluster_capacity.argtypes = [i, i, sz, ctypes.POINTER(ctypes.c_int)]
    L.fg_workspace_status.restype = i
    L.fg_generalised_geodesic2d.argtypes = [vp, i, i, i, vp, i, vp, f, f, f, i, vp, sz, vp]
    L.fg_signed_generalised_geodesic2d.argtypes = L.fg_generalised_geodesic2d.argtypes
    L.fg_generalised_geodesic3d.argtypes = [vp, i, i, i, i, vp, i, fp, vp, f, f, f, i, vp, sz, vp]
    L.fg_signed_generalised_geodesic3d.argtypes = L.fg_generalised_geodesic3d.argtypes
    L.fg_GSF2d.argtypes = [vp, i, i, i, vp, i, f, f, f, i, vp, vp, sz, vp]
    L.fg_generalised_geodesic2d_noalloc.argtypes = [vp, i, i, i, vp, i, vp, f, f, f, i, vp]
    L.fg_noalloc_status.argtypes = [vp]
    L.fg_batch2d_smem_bytes.argtypes = [i, i, i]
    L.fg_batch2d_smem_bytes.restype = sz
    L.fg_batch_geodesic2d.argtypes = [vp, i, i, i, i, i, vp, vp, i, vp]
    L.fg_batch2d_tiled_scratch_bytes.argtypes = [i, i]
    L.fg_batch2d_tiled_scratch_bytes.restype = sz
    L.fg_batch_geodesic2d_tiled.argtypes = [vp, ctypes.POINTER(ctypes.c_int), i, i, i, i, vp, sz, vp, vp]
    L.fg_grad_geodesic2d_forward.argtypes = [vp, i, i, i, i, vp, vp, vp]
    L.fg_grad_geodesic2d_backward.argtypes = [vp, i, i, i, i, vp, vp, vp]
    L.fg_grad_geodesic2d_forward_pass.argtypes = [vp, i, i, i, i, vp, vp, vp]
    L.fg_grad_geodesic2d_backward_pass.argtypes = [vp, i, i, i, i, i, i, vp, vp]
    L.fg_GSF3d.argtypes = [vp, i, i, i, i, vp, i, f, fp, f, f, i, vp, vp, sz, vp]
    L.fg_batch3d_job_bytes.argtypes = []
    L.fg_batch3d_job_bytes.restype = sz
    L.fg_batch3d_plan.argtypes = [vp, i, i, i, vp, vp, sz, ctypes.POINTER(ctypes.c_int)]
    L.fg_batch3d_launch.argtypes = [vp, i, i, i, i, i, i, sz, vp, vp, vp]
    L.fg_batch3d_capacity.argtypes = [i, i, i, i, sz, ctypes.POINTER(ctypes.c_int)]
    for name in ("fg_generalised_geodesic2d", "fg_generalised_geodesic3d", "fg_signed_generalised_geodesic2d",
                 "fg_signed_generalised_geodesic3d", "fg_GSF2d", "fg_GSF3d"):
        getattr(L, name + "_toivanen").argtypes = getattr(L, name).argtypes  # same arguments
    for name in EXPORTED:
        if name not in ("fg_last_error",):
            getattr(L, name).restype = getattr(L, name).restype or i
    if L.fg_abi_version() != 1:
        raise ImportError("fastgeodis_gb300 engine ABI mismatch")
    _lib = L
    return L


def profile_begin() -> None:
    check(load().fg_profile_begin())


def profile_end():
    """Returns (summed pass-kernel ms, launches, voxel-passes) since profile_begin()."""
    ms, n, vp = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
    check(load().fg_profile_end(ctypes.byref(ms), ctypes.byref(n), ctypes.byref(vp)))
    return ms.value, n.value, vp.value


def profile_aux_launches() -> int:
    """Kernel launches of the window closed by profile_end() besides one per
    pass (chunk launches after a pass's first, map transposes)."""
    n = ctypes.c_int()
    check(load().fg_profile_aux_launches(ctypes.byref(n)))
    return n.value


def profile_launch_times():
    """[(ms, steps)] of every pass launch of the window closed by profile_end()."""
    L = load()
    n = ctypes.c_int()
    check(L.fg_profile_launch_times(None, None, 0, ctypes.byref(n)))
    ms = (ctypes.c_float * max(1, n.value))()
    st = (ctypes.c_int * max(1, n.value))()
    check(L.fg_profile_launch_times(ms, st, n.value, ctypes.byref(n)))
    return [(float(ms[i]), int(st[i])) for i in range(n.value)]


FG_ONE_LAUNCH_SIDE = 512  # the one-launch 2D kernel's largest side
FG_ONE_LAUNCH_CELLS = 16384  # the per-call path runs images of fewer cells in one launch


def runs_in_one_launch(shape) -> bool:
    """Whether the per-call path runs a plain or signed 2D transform of an
    image of this (H, W) in one launch (no pinned plans or planner limits):
    fewer than FG_ONE_LAUNCH_CELLS cells, sides up to FG_ONE_LAUNCH_SIDE."""
    H, W = (int(x) for x in shape)
    return max(H, W) <= FG_ONE_LAUNCH_SIDE and H * W < FG_ONE_LAUNCH_CELLS
FG_PLAN_LEAN = 1      # plan flag: the 64-register kernel
FG_PLAN_CLUSTER = 2   # plan flag: one thread-block cluster owns the cross-section
FG_PLAN_RUNS2 = 4     # plan flag: cluster sweep kernel, 2 runs of 4 cells per thread
FG_PLAN_CHUNKED = 8   # plan flag: one ordinary launch per chunk of S steps (tiles need not all be resident)
FG_PLAN_ROWS = 64     # plan flag: 2D tiles on the row-tile kernel (one thread per cell)


def FG_PLAN_MODE(m: int) -> int:
    """fg_plan_override flag: the plan applies to passes of arithmetic mode m only."""
    return (m + 1) << 4
# the last field holds the plan flags (FG_PLAN_LEAN | FG_PLAN_CLUSTER)
PLAN_FIELDS = ("S", "T1", "T2", "K1", "K2", "tiles1", "tiles2", "threads", "depth", "smem", "lean")


def plan_describe(cross, N1, N2, C=1, maps=1, mode=0, transposed_write=False, sms=152) -> dict:
    """The engine's plan for one pass (see fg_plan_describe); needs no GPU."""
    out = (ctypes.c_int * len(PLAN_FIELDS))()
    check(load().fg_plan_describe(cross, N1, N2, C, maps, mode, int(transposed_write), sms, out))
    return dict(zip(PLAN_FIELDS, list(out)))


def cluster_capacity(cluster_size: int, threads: int, smem: int) -> int:
    """Clusters of this shape of the cluster sweep kernel the current device runs at once."""
    n = ctypes.c_int()
    check(load().fg_cluster_capacity(cluster_size, threads, smem, ctypes.byref(n)))
    return n.value


def last_error() -> str:
    msg = load().fg_last_error()
    return msg.decode() if msg else ""


def check(rc: int) -> None:
    """Map an engine status code onto the reference's exception types."""
    if rc == FG_OK:
        return
    msg = last_error()
    if rc == FG_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise EngineError(f"fastgeodis_gb300 engine error {rc}: {msg}")
