"""Build recipes for the CPU oracle (test infrastructure only).

Three artefacts are produced here; none is part of the shipped product:

* ``oracle/_build/libfg_oracle.so`` -- the plain-C restatement of FastGeodis'
  raster scan (``oracle/fg_oracle.c``), compiled with ``gcc`` and OpenMP.  It
  runs on any host (x86 or Arm) and is the oracle of the parity tests and
  the timed CPU baseline.
* ``oracle/_ref/libfg_fastmarch.so`` -- the fast-marching accuracy harness
  (``oracle/fg_fastmarch.cpp``) over the reference's vendored solver header
  (``dependency/fmm``), compiled where that header is available.
* ``oracle/_ref/fastgeodis_ref_cpu*.so`` -- the reference's own CPU sources
  (``FastGeodis/*.cpp`` of masadcv/FastGeodis 1.0.5), compiled file by file with
  ``g++`` against the installed torch headers, without running the reference's
  ``setup.py``.  It only exists where the reference source tree is mounted and
  is used to generate the committed golden vectors under ``tests/golden/``.

The unmodified reference as its users install it -- its ``FastGeodis``
Python package over a ``FastGeodisCpp`` extension with the OpenMP CPU path
and the CUDA path (``WITH_CUDA``, kernels built for sm_103a) -- is assembled
in ``baseline/_ref/`` (git-ignored, the slot of the reference install) for the
benchmark's reference arm:

* :func:`stage_reference` copies the files of the reference's source
  distribution (its ``MANIFEST.in``: ``FastGeodis/*.{py,cpp,cu,h}`` and the
  header-only ``dependency/fmm``) into ``baseline/_ref/src`` where the
  reference tree is mounted, so that they travel with the working copy;
* :func:`build_reference_install` compiles them on the machine that runs them
  (``g++`` for the C++ files, ``nvcc`` for ``fastgeodis_cuda.cu`` with the
  compiler's defaults, as the reference's ``setup.py`` would) into
  ``baseline/_ref/FastGeodisCpp*.so`` and copies the Python package beside it.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
and reference arm may load these libraries.
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
PORT_SRC = os.path.join(HERE, "fg_oracle.c")
PORT_LIB = os.path.join(BUILD_DIR, "libfg_oracle.so")
REF_MODULE = "fastgeodis_ref_cpu"
DEFAULT_REF_ROOT = os.environ.get("FG_REFERENCE_ROOT", "/root/reference")


def _newer(target: str, *sources: str) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_port(force: bool = False, verbose: bool = False) -> str:
    """Compile the C restatement.  ``-ffp-contract=off`` keeps every float
    operation separately rounded on aarch64 as well, which is how the
    reference's x86-64 build (no ``-march``, so no FMA) evaluates them."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and _newer(PORT_LIB, PORT_SRC):
        return PORT_LIB
    cmd = [
        "gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math", "-fsigned-char",
        PORT_SRC, "-o", PORT_LIB + ".tmp", "-lm",
    ]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(PORT_LIB + ".tmp", PORT_LIB)
    return PORT_LIB


def reference_module_path() -> str:
    return os.path.join(REF_DIR, REF_MODULE + sysconfig.get_config_var("EXT_SUFFIX"))


def build_reference(ref_root: str = DEFAULT_REF_ROOT, force: bool = False,
                    verbose: bool = False) -> str | None:
    """Compile the reference's CPU path (all of ``FastGeodis/*.cpp``; the
    pybind module in ``fastgeodis.cpp`` references every backend) into a
    Python extension module under ``oracle/_ref``.  Returns None when the
    reference tree is absent (for example on the GPU host)."""
    src_dir = os.path.join(ref_root, "FastGeodis")
    if not os.path.isdir(src_dir):
        return None
    import torch
    from torch.utils import cpp_extension

    out = reference_module_path()
    sources = sorted(
        os.path.join(src_dir, f) for f in os.listdir(src_dir) if f.endswith(".cpp")
    )
    if not force and _newer(out, *sources):
        return out
    os.makedirs(REF_DIR, exist_ok=True)
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    inc = [f"-I{p}" for p in cpp_extension.include_paths()]
    inc += [f"-I{sysconfig.get_paths()['include']}", f"-I{src_dir}",
            f"-I{os.path.join(ref_root, 'dependency')}"]
    defs = ["-DTORCH_API_INCLUDE_EXTENSION_H", f"-DTORCH_EXTENSION_NAME={REF_MODULE}",
            f"-D_GLIBCXX_USE_CXX11_ABI={abi}", "-DAT_PARALLEL_OPENMP=1"]
    flags = ["-O2", "-g0", "-std=c++17", "-fPIC", "-fopenmp"]
    objs = []

    def compile_one(src: str) -> str:
        obj = os.path.join(REF_DIR, os.path.basename(src) + ".o")
        cmd = ["g++", *flags, *defs, *inc, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, sources))
    lib_dir = os.path.join(os.path.dirname(torch.__file__), "lib")
    link = ["g++", "-shared", "-fopenmp", *objs, "-o", out + ".tmp",
            f"-L{lib_dir}", "-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python",
            f"-Wl,-rpath,{lib_dir}"]
    if verbose:
        print(" ".join(link))
    subprocess.check_call(link)
    os.replace(out + ".tmp", out)
    for o in objs:
        os.remove(o)
    return out


ROOT = os.path.dirname(HERE)
INSTALL_DIR = os.path.join(ROOT, "baseline", "_ref")
STAGE_DIR = os.path.join(INSTALL_DIR, "src")
INSTALL_MODULE = "FastGeodisCpp"


def stage_reference(ref_root: str = DEFAULT_REF_ROOT) -> str | None:
    """Copy the reference's source-distribution files into baseline/_ref/src
    (git-ignored).  Returns the staged root, or None without a reference tree."""
    import shutil

    src_dir = os.path.join(ref_root, "FastGeodis")
    if not os.path.isdir(src_dir):
        return None
    dst = os.path.join(STAGE_DIR, "FastGeodis")
    os.makedirs(dst, exist_ok=True)
    for f in sorted(os.listdir(src_dir)):
        if f.endswith((".py", ".cpp", ".cu", ".h")):
            shutil.copyfile(os.path.join(src_dir, f), os.path.join(dst, f))
    fmm = os.path.join(ref_root, "dependency", "fmm", "include")
    if os.path.isdir(fmm):
        shutil.copytree(fmm, os.path.join(STAGE_DIR, "dependency", "fmm", "include"), dirs_exist_ok=True)
    return STAGE_DIR


def install_module_path() -> str:
    return os.path.join(INSTALL_DIR, INSTALL_MODULE + sysconfig.get_config_var("EXT_SUFFIX"))


def build_reference_install(force: bool = False, verbose: bool = False, cuda: bool = True) -> str | None:
    """Compile the staged reference (or the mounted tree) into the extension
    module ``FastGeodisCpp`` under baseline/_ref and copy its Python package
    there.  The compile follows what the reference's setup.py asks of
    torch.utils.cpp_extension: the C++ files with OpenMP and ``WITH_CUDA``,
    ``fastgeodis_cuda.cu`` with nvcc's defaults (FMA contraction on) for
    sm_103a.  Returns the module path, or None when no sources are present."""
    import shutil

    root = STAGE_DIR if os.path.isdir(os.path.join(STAGE_DIR, "FastGeodis")) else DEFAULT_REF_ROOT
    src_dir = os.path.join(root, "FastGeodis")
    if not os.path.isdir(src_dir):
        return None
    import torch
    from torch.utils import cpp_extension

    out = install_module_path()
    cpp = sorted(os.path.join(src_dir, f) for f in os.listdir(src_dir) if f.endswith(".cpp"))
    cu = sorted(os.path.join(src_dir, f) for f in os.listdir(src_dir) if f.endswith(".cu")) if cuda else []
    pkg = os.path.join(INSTALL_DIR, "FastGeodis")
    os.makedirs(pkg, exist_ok=True)
    for f in os.listdir(src_dir):
        if f.endswith(".py"):
            shutil.copyfile(os.path.join(src_dir, f), os.path.join(pkg, f))
    if not force and _newer(out, *(cpp + cu)):
        return out
    tmp = os.path.join(INSTALL_DIR, "_obj")
    os.makedirs(tmp, exist_ok=True)
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    inc = [f"-I{p}" for p in cpp_extension.include_paths()]
    inc += [f"-I{os.path.join(cuda_home, 'include')}", f"-I{sysconfig.get_paths()['include']}", f"-I{src_dir}",
            f"-I{os.path.join(root, 'dependency')}"]
    defs = ["-DTORCH_API_INCLUDE_EXTENSION_H", f"-DTORCH_EXTENSION_NAME={INSTALL_MODULE}",
            f"-D_GLIBCXX_USE_CXX11_ABI={abi}", "-DAT_PARALLEL_OPENMP=1"] + (["-DWITH_CUDA"] if cu else [])

    def compile_one(src: str) -> str:
        obj = os.path.join(tmp, os.path.basename(src) + ".o")
        if src.endswith(".cu"):
            nvcc = os.path.join(cuda_home, "bin", "nvcc")
            cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler", "-fPIC",
                   *cpp_extension.COMMON_NVCC_FLAGS, *defs, *inc, "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-g0", "-std=c++17", "-fPIC", "-fopenmp", *defs, *inc, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, cpp + cu))
    lib_dir = os.path.join(os.path.dirname(torch.__file__), "lib")
    libs = ["-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python"]
    if cu:
        libs += ["-lc10_cuda", "-ltorch_cuda", f"-L{os.path.join(cuda_home, 'lib64')}", "-lcudart"]
    link = ["g++", "-shared", "-fopenmp", *objs, "-o", out + ".tmp", f"-L{lib_dir}", *libs,
            f"-Wl,-rpath,{lib_dir}"]
    if verbose:
        print(" ".join(link), flush=True)
    subprocess.check_call(link)
    os.replace(out + ".tmp", out)
    shutil.rmtree(tmp, ignore_errors=True)
    return out


def load_reference_install():
    """Import the reference's own Python package over its built extension
    (``import FastGeodis`` from baseline/_ref); None if it was not built."""
    if not os.path.exists(install_module_path()):
        return None
    import torch  # noqa: F401  (loads libtorch before the extension)

    if INSTALL_DIR not in sys.path:
        sys.path.insert(0, INSTALL_DIR)
    import FastGeodis  # the reference's FastGeodis/__init__.py

    return FastGeodis


FMM_SRC = os.path.join(HERE, "fg_fastmarch.cpp")
FMM_LIB = os.path.join(REF_DIR, "libfg_fastmarch.so")


def fmm_include_dir() -> str | None:
    """The reference's vendored fast-marching header (dependency/fmm/include):
    in the mounted reference tree, else in its staged copy."""
    for root in (DEFAULT_REF_ROOT, STAGE_DIR):
        d = os.path.join(root, "dependency", "fmm", "include")
        if os.path.isfile(os.path.join(d, "thinks", "fast_marching_method", "fast_marching_method.hpp")):
            return d
    return None


def build_fastmarch(force: bool = False, verbose: bool = False) -> str | None:
    """Compile the fast-marching accuracy harness (oracle/fg_fastmarch.cpp over
    the reference's vendored solver header) into oracle/_ref; None when the
    header is not available."""
    inc = fmm_include_dir()
    if inc is None:
        return None
    hdr = os.path.join(inc, "thinks", "fast_marching_method", "fast_marching_method.hpp")
    if not force and _newer(FMM_LIB, FMM_SRC, hdr):
        return FMM_LIB
    os.makedirs(REF_DIR, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{inc}", FMM_SRC, "-o", FMM_LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(FMM_LIB + ".tmp", FMM_LIB)
    return FMM_LIB


def load_reference():
    """Import the compiled reference CPU module (None if it was not built)."""
    path = reference_module_path()
    if not os.path.exists(path):
        return None
    import importlib.util
    import torch  # noqa: F401  (loads libtorch before the extension)

    spec = importlib.util.spec_from_file_location(REF_MODULE, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_port(force=force, verbose=True))
    print(build_reference(force=force, verbose=True))
    print(build_fastmarch(force=force, verbose=True))
    if "--install" in sys.argv:  # the reference as installed, for the benchmark's reference arm
        print(stage_reference())
        print(build_reference_install(force=force, verbose=True))
