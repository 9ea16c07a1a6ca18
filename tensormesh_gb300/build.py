"""Build the native library ``libtmgb300.so`` in-tree.

CUDA sources are compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``); host sources with g++.  Translation units
compile in parallel; the library is relinked only when a source or header
changed (a hash of their contents is stored beside it).
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtmgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = [shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tensormesh_gb300")


def _sources():
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    hdrs = sorted(f for f in os.listdir(CSRC) if f.endswith((".h", ".cuh")))
    return srcs, hdrs


def _digest(srcs, hdrs) -> str:
    h = hashlib.sha256()
    for f in srcs + hdrs:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode() + fh.read())
    for f in sorted(os.listdir(INCLUDE)):
        with open(os.path.join(INCLUDE, f), "rb") as fh:
            h.update(f.encode() + fh.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def _compile(src: str, nvcc: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", INCLUDE, "-c", path, "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-c", path, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        sys.stderr.write(res.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    srcs, hdrs = _sources()
    digest = _digest(srcs, hdrs)
    stamp = LIB + ".sha256"
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, verbose_ptxas), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
