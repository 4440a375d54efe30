"""Build libgopf_gpu.so in-tree with nvcc for sm_103a.

The library is the product: CUDA kernels plus the C ABI declared in
include/gopf_gpu.h.  Translation units compile in parallel; the result is
gopf_gb300/libgopf_gpu.so (git-ignored, rebuilt on every machine).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgopf_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src: str, extra: list[str]) -> str:
    nvcc = nvcc_path()
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH, "-c", path, "-o", obj, *extra]
    if src.endswith(".cpp"):
        cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-x", "c++", "-c", path, "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def needs_rebuild() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "gopf_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and not needs_rebuild():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc_path(), "-shared", *ARCH, "-o", tmp, *objs, "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        # libcuda stubs are not needed at link time: the runtime loads the driver itself
        cmd = [c for c in cmd if c != "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
