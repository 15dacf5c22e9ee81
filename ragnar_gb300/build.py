"""In-tree build of the ragnar_gb300 native code.

* ``ragnar_gb300/_lib/libragnar_gb300.so`` -- the CUDA library behind the C ABI
  (``include/ragnar_gb300.h``), compiled for sm_103a only.
* ``ragnar_gb300/_ragnar<ext>`` -- the pybind11 drop-in module, host C++ that
  talks to the library through the C ABI.

Translation units compile in parallel; objects are rebuilt only when a source
or header is newer.  Run it by path, ``python ragnar_gb300/build.py`` (importing
the package first would need the extension this script builds).
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libragnar_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build ragnar_gb300")
    return cand


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _pybind11_include() -> str:
    try:
        import pybind11  # noqa: PLC0415

        return pybind11.get_include()
    except ImportError:
        import torch  # noqa: PLC0415  (its wheel ships the pybind11 headers)

        return os.path.join(os.path.dirname(torch.__file__), "include")


def nvcc_flags() -> list[str]:
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", f"-I{INCLUDE}", f"-I{CSRC}"]


def build_library(verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs, todo = [], []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            todo.append([nvcc, *nvcc_flags(), "-c", src, "-o", obj])
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for _ in ex.map(_run, todo):
                pass
    if _newer(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC"])
    if verbose:
        print("built", LIB)
    return LIB


def build_module(verbose: bool = False) -> str:
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    out = os.path.join(PKG, "_ragnar" + ext)
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    deps = srcs + glob.glob(os.path.join(HOST, "*.hpp")) + [os.path.join(INCLUDE, "ragnar_gb300.h"), LIB]
    if _newer(out, deps):
        cxx = os.environ.get("CXX", "g++")
        pyinc = sysconfig.get_paths()["include"]
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden",
               "-ffp-contract=off", f"-I{INCLUDE}", f"-I{_pybind11_include()}", f"-I{pyinc}",
               *srcs, "-o", out, f"-L{LIBDIR}", "-lragnar_gb300", "-Wl,-rpath,$ORIGIN/_lib"]
        _run(cmd)
    if verbose:
        print("built", out)
    return out


def build(verbose: bool = False) -> None:
    build_library(verbose)
    build_module(verbose)


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
