"""In-tree build of libgsea103.so for GB300 (sm_103a).

Every CUDA translation unit is compiled with nvcc for ``compute_103a/sm_103a``
only, host C++ units with g++, in parallel, then linked into
``cudagsea_gb300/_lib/libgsea103.so``.  Objects are rebuilt only when a source
or a header is newer.  No CMake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_obj")
LIB_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIB_DIR, "libgsea103.so")
CLI = os.path.join(LIB_DIR, "gsea103")
CLI_SRC = os.path.join(CSRC, "cli.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h*"))


def _foreign(path: str) -> bool:
    """True for an ELF object built for another machine (copied from another host)."""
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if head[:4] != b"\x7fELF":
        return False
    mach = int.from_bytes(head[18:20], "little")
    here = {"x86_64": 62, "aarch64": 183}.get(platform.machine())
    return here is not None and mach != here


def _stale(obj: str, src: str, newest_header: float) -> bool:
    if not os.path.exists(obj) or _foreign(obj):
        return True
    t = os.path.getmtime(obj)
    return t < os.path.getmtime(src) or t < newest_header


def _compile(src: str, obj: str, verbose: bool) -> None:
    # written under a temporary name and renamed: a build running beside
    # this one (one process per GPU) never links a half-written object
    tmp = obj + f".tmp{os.getpid()}"
    if src.endswith(".cu"):
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", tmp]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I" + os.path.join(_cuda_home(), "include"), "-c", src, "-o", tmp]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        if os.path.exists(tmp):
            os.remove(tmp)
        raise RuntimeError(f"compilation of {os.path.basename(src)} failed:\n{r.stdout}")
    os.replace(tmp, obj)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    srcs = [s for s in srcs if s != CLI_SRC]
    newest_header = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, s, newest_header):
            todo.append((s, o))
    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(lambda so: _compile(so[0], so[1], verbose), todo))
    if (todo or not os.path.exists(LIB) or _foreign(LIB)
            or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}")
        os.replace(tmp, LIB)
    if (not os.path.exists(CLI) or _foreign(CLI) or os.path.getmtime(CLI) < os.path.getmtime(LIB)
            or os.path.getmtime(CLI) < os.path.getmtime(CLI_SRC)):
        tmp = CLI + f".tmp{os.getpid()}"
        cmd = ["g++"] + CXX_FLAGS + ["-o", tmp, CLI_SRC, "-L" + LIB_DIR, "-lgsea103", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed:\n{r.stdout}")
        os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
