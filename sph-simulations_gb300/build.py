"""Builds libsphg.so (the CUDA library behind include/sphg.h) for sm_103a, and
the host driver sph_gb300_app (app/sph_gb300_app.cpp) linked against it.

Each .cu translation unit is compiled in parallel with nvcc, then linked into
one shared library next to this file.  Objects go to ``_build/``.
Usage:  python sph-simulations_gb300/build.py [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsphg.so")
HOST_APP = os.path.join(HERE, "sph_gb300_app")
APP_SRC = os.path.join(HERE, "app", "sph_gb300_app.cpp")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I" + os.path.join(ROOT, "include")]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsphg.so")
    return path


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(ROOT, "include", "sphg.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, force):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not force and not _stale(obj, [src] + headers()):
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if force or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link of libsphg.so failed:\n%s%s" % (r.stdout, r.stderr))
    if force or _stale(HOST_APP, [APP_SRC, LIB, os.path.join(ROOT, "include", "sphg.h")]):
        gxx = shutil.which("g++") or "g++"
        cmd = [gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), APP_SRC, "-o", HOST_APP,
               "-L" + HERE, "-lsphg", "-Wl,-rpath,$ORIGIN", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build of sph_gb300_app failed:\n%s%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB, "and", HOST_APP)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
