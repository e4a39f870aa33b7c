"""In-tree build of libepseon_cuda.so (nvcc, sm_103a) and the _libepseon_cuda
Python module (g++ against the pybind11 headers bundled with torch).

Artifacts land next to the sources (``epseon_backend_gb300/lib/``) and are
git-ignored; every machine builds its own (the GPU host is aarch64).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(CSRC, "host")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libepseon_cuda.so")
PYMOD_DIR = os.path.join(PKG, "device", "cuda")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_cuda(force: bool = False, verbose: bool = False) -> str:
    """Compile csrc/*.cu in parallel and link libepseon_cuda.so."""
    os.makedirs(OBJDIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + [
        os.path.join(INCLUDE, "epscu.h")
    ]
    objs = []
    jobs = []
    for src in sources:
        obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [
                nvcc(),
                *ARCH,
                "-O3",
                "-lineinfo",
                "-std=c++17",
                "-Xcompiler",
                "-fPIC,-O2",
                "-I" + INCLUDE,
                "-I" + CSRC,
                "-c",
                src,
                "-o",
                obj,
            ]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose:
                    print(r.stdout, r.stderr)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


def _python_include() -> str:
    return sysconfig.get_paths()["include"]


def _pybind_include() -> str:
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec is not None and spec.origin:
        inc = os.path.join(os.path.dirname(spec.origin), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    try:
        import pybind11  # noqa: F401

        return pybind11.get_include()
    except ImportError as e:  # pragma: no cover
        raise RuntimeError("pybind11 headers not found (torch/include or pybind11)") from e


def build_pymodule(force: bool = False) -> str:
    """Build the _libepseon_cuda extension (C++ host API + pybind11 binding)."""
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    target = os.path.join(PYMOD_DIR, "_libepseon_cuda" + ext)
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    hdrs = glob.glob(os.path.join(HOST, "*.hpp")) + [os.path.join(INCLUDE, "epscu.h"), LIB]
    if not srcs:
        return ""
    if not force and not _stale(target, srcs + hdrs):
        return target
    os.makedirs(PYMOD_DIR, exist_ok=True)
    tmp = target + ".tmp"
    cmd = [
        os.environ.get("CXX", "g++"),
        "-O2",
        "-std=c++20",
        "-shared",
        "-fPIC",
        "-fvisibility=hidden",
        "-I" + INCLUDE,
        "-I" + HOST,
        "-I" + _python_include(),
        "-isystem",
        _pybind_include(),
        *srcs,
        "-o",
        tmp,
        "-L" + LIBDIR,
        "-lepseon_cuda",
        "-Wl,-rpath,$ORIGIN/../../lib",
        "-lpthread",
    ]
    _run(cmd)
    os.replace(tmp, target)
    return target


def build(force: bool = False, verbose: bool = False) -> None:
    build_cuda(force=force, verbose=verbose)
    build_pymodule(force=force)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
