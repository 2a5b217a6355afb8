"""Build of the in-tree CUDA library libvoce_gpu.so (sm_103a only).

``python -m voce_gb300.build`` (or ``voce_gb300.build.build()``) compiles
every translation unit under csrc/ with nvcc for ``sm_103a`` in parallel and
links ``voce_gb300/lib/libvoce_gpu.so``, then the host-only legacy layer
``voce_gb300/lib/libvoce_legacy.so`` on top of it.  No cmake, no torch extension
machinery: the library has a plain C ABI (include/voce_gpu.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libvoce_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
# extra nvcc flags (e.g. -DVOCE_NR_MIXED_BLOCKS=3) for tuning builds
NVFLAGS += os.environ.get("VOCE_NVCC_EXTRA", "").split()
SOURCES = ["voce_kernels.cu", "voce_api.cu", "voce_server.cpp", "voce_io.cpp", "voce_parse.cpp"]
LEGACY = os.path.join(CSRC, "legacy")
LEGACY_SOURCES = ["voce_legacy.cpp", "voce_legacy_cxx.cpp"]
LEGACY_LIB = os.path.join(LIBDIR, "libvoce_legacy.so")


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    inc = os.path.join(ROOT, "include")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *NVFLAGS, "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    build_legacy(verbose, force)
    return LIB


def build_sanitized(dest: str, verbose: bool = False) -> str:
    """libvoce_gpu.so with AddressSanitizer and UndefinedBehaviorSanitizer in
    its host code (the device code is unchanged), into directory dest; for the
    host-side sanitizer test, which loads it with the sanitizer runtimes
    preloaded.  Returns the library's path."""
    os.makedirs(dest, exist_ok=True)
    nvcc = _nvcc()
    # one flag per -Xcompiler: nvcc splits its argument at commas
    san = ["-g"]
    for f in ("-fsanitize=address", "-fsanitize=undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=all"):
        san += ["-Xcompiler", f]
    flags = [f for f in NVFLAGS if f != "-O3"] + ["-O1"]
    jobs, objs = [], []
    for src in SOURCES:
        o = os.path.join(dest, src + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, *flags, *san, "-c", os.path.join(CSRC, src), "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    lib = os.path.join(dest, "libvoce_gpu.so")
    run([nvcc, *ARCH, "-shared", *san, "-o", lib, *objs, "-lcudart"])
    return lib


def build_legacy(verbose: bool = False, force: bool = False) -> str:
    """libvoce_legacy.so (include/voce_legacy.h): host C++ only, linked
    against libvoce_gpu.so; its undefined symbols are the reference program's
    globals, resolved when a program defining them loads it."""
    srcs = [os.path.join(LEGACY, f) for f in LEGACY_SOURCES]
    deps = srcs + [os.path.join(LEGACY, "voce_legacy_impl.h"), LIB] + [
        os.path.join(ROOT, "include", h) for h in ("voce_gpu.h", "voce_io.h", "voce_legacy.h")]
    if not (force or _stale(LEGACY_LIB, deps)):
        return LEGACY_LIB
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-I" + os.path.join(ROOT, "include"),
           *srcs, "-L" + LIBDIR, "-lvoce_gpu", "-Wl,-rpath,$ORIGIN", "-o", LEGACY_LIB]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("legacy build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LEGACY_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
