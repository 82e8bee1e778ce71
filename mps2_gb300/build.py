"""Build ``libgqmps2_gb300.so`` in-tree with nvcc for sm_103a.

Every translation unit under ``csrc/`` is compiled in parallel into
``_build/`` and linked into ``mps2_gb300/libgqmps2_gb300.so``.  Objects are
rebuilt when a source or any header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgqmps2_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return env
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _nvcc() -> str:
    return os.path.join(cuda_home(), "bin", "nvcc")


def _flags():
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
                   "--expt-relaxed-constexpr", "-I", CSRC,
                   "-I", os.path.join(os.path.dirname(HERE), "include")]


def _compile(src: str, extra=()) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    headers = glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(os.path.dirname(HERE), "include", "*.h"))
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in headers])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [_nvcc(), "-x", "cu", "-c", src, "-o", obj] + _flags() + list(extra)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra=()) -> str:
    # objects from another machine architecture are discarded
    stamp = os.path.join(BUILD, "MACHINE")
    mach = platform.machine()
    if os.path.isdir(BUILD):
        old = open(stamp).read().strip() if os.path.exists(stamp) else ""
        if old != mach:
            shutil.rmtree(BUILD)
            if os.path.exists(LIB):
                os.remove(LIB)
    os.makedirs(BUILD, exist_ok=True)
    with open(stamp, "w") as f:
        f.write(mach)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= newest):
        libdir = os.path.join(cuda_home(), "lib64")
        cmd = [_nvcc(), "-shared", "-o", LIB] + objs + ARCH + [
            "-L", libdir, "-lcusolver", "-lcublas", "-lcudart", "-lpthread",
            "-Xlinker", f"-rpath,{libdir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
