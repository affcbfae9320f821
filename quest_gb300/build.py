"""Builds the backend library in-tree: quest_gb300/_build/libquest_gb300.so.

Every translation unit under quest_gb300/csrc is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, and linked into one
shared library that exports the C ABI of include/quest_gb300.h and the
QuEST-named host API.  Usage:  python -m quest_gb300.build  [--force]
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
LIB = os.path.join(BUILD, "libquest_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3",
              "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wno-unknown-pragmas", "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the backend")


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def sources():
    srcs = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".cpp"):
            srcs.append(os.path.join(CSRC, f))
    return srcs


def _headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hpp"))]
    return hs


def _compile(src, obj):
    if src.endswith(".cu"):
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I" + os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {os.path.basename(src)} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force=False, verbose=False):
    """Compiles what changed and links the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    newest_header = max((os.path.getmtime(h) for h in _headers()), default=0)
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        stale = force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), newest_header)
        if stale:
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o) for s, o in jobs]
            for f in futs:
                f.result()
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        if verbose:
            print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
